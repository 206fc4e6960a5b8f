// dgcu.hpp -- C++ stand-ins for HopeFOAM's DG operator API over the dgcu C ABI.
//
// A HopeFOAM solver loop such as tutorials/DG/2D/isentropicVortex/dgEulerFoam/
// dgEulerFoam.C:64-131 keeps its shape and its call signatures:
//
//   dgcu::dgMesh mesh(desc, order, gamma, cubature);       // dgMesh(IOobject)        dgMesh/dgMesh.C:71-116
//   dgcu::dgScalarField rho(mesh), Ener(mesh);             // GeometricDofField       fields/GeometricDofField
//   dgcu::dgVectorField rhoU(mesh);
//   dgcu::godunovScheme Godunov(mesh, "Roe");              // godunovScheme           DG/godunovFlux/godunovScheme.C:41-73
//   ...
//   rho1.updateGaussField(); rhoU1.updateGaussField(); Ener1.updateGaussField();
//   dgcu::dgGaussVectorField gther_U = rhoU1.gaussField() / rho1.gaussField();
//   dgcu::dgGaussScalarField gther_p = dgcu::pressure(gamma, rho1.gaussField(), gther_U, Ener1.gaussField());
//   Godunov.update(gther_U, gther_p, gamma, rho1.gaussField(), rhoU1.gaussField(), Ener1.gaussField());
//   dgcu::dg::solveEquation(dgcu::dgm::ddt(rho1)  + dgcu::dgc::div(gther_U, rho1,  Godunov.fluxRho()));
//   dgcu::dg::solveEquation(dgcu::dgm::ddt(rhoU1) + dgcu::dgc::div(gther_U, rhoU1, Godunov.fluxRhoU())
//                                                 + dgcu::dgc::grad(gther_p));
//   dgcu::dg::solveEquation(dgcu::dgm::ddt(Ener1) + dgcu::dgc::div(gther_U, Ener1, Godunov.fluxEner())
//                                                 + dgcu::dgc::div(gther_U, gther_p));
//
// The GPU evaluates the three conserved equations of one stage in a single
// fused kernel (cubature and face values, primitive variables, fluxes and the
// weak divergence are all formed inside it), so the gauss fields and the
// equations are recorded, not evaluated, and the stage runs on the device when
// the last of the three is solved (the reference solves them back to back on
// the same state, dgEulerFoam.C:86-90, so the result is the same).
//
// Device residency: after a stage the new state stays on the device and the
// fields' host arrays are refreshed only when they are read (component()),
// so a sequence of solveEquation stages moves no right-hand side and no state
// across PCIe.  A field handed out for writing (non-const component()) drops
// the device copy; the next stage uploads the host values again.
//
// Errors throw dgcu::Error (a std::runtime_error carrying the DG_ERR_* code),
// the analogue of the reference's FatalError.
#pragma once

#include <array>
#include <stdexcept>
#include <string>
#include <vector>

#include "dgcu.h"

namespace dgcu {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(dg_ctx* ctx, int rc, const char* what) {
    if (rc != DG_OK) throw Error(rc, std::string(what) + ": " + (ctx ? dg_last_error(ctx) : "") + " (code " +
                                         std::to_string(rc) + ")");
}

struct MeshData {
    std::vector<int32_t> EToV, EToE, EToF, ROT;
    std::vector<double> VXY;  // K x 3 x 2
    int32_t K() const { return (int32_t)(EToV.size() / 3); }
};

template <int NC>
class GeometricDofField;
using dgScalarField = GeometricDofField<1>;
using dgVectorField = GeometricDofField<2>;  // x, y (the reference's z component stays 0)

// the three conserved fields of the Euler system
struct EulerState {
    dgScalarField* rho;
    dgVectorField* rhoU;
    dgScalarField* Ener;
    bool operator==(const EulerState& o) const { return rho == o.rho && rhoU == o.rhoU && Ener == o.Ener; }
};

class dgMesh {
   public:
    dgMesh(const MeshData& m, int order, double gamma, const std::vector<double>& cubature) : mesh_(m) {
        dg_mesh_desc d{m.K(), m.EToV.data(), m.VXY.data(), m.EToE.data(), m.EToF.data(),
                       m.ROT.empty() ? nullptr : m.ROT.data(), nullptr};
        dg_opts o{order, cubature.data(), (int32_t)(cubature.size() / 3), gamma, nullptr};
        check(nullptr, dg_ctx_create(&d, &o, &ctx_), "dgMesh");
        check(ctx_, dg_get_info(ctx_, &info_), "dgMesh info");
    }
    ~dgMesh() { dg_ctx_destroy(ctx_); }
    dgMesh(const dgMesh&) = delete;
    dgMesh& operator=(const dgMesh&) = delete;
    dg_ctx* ctx() const { return ctx_; }
    int nCells() const { return info_.K; }
    int nDofPerCell() const { return info_.Np; }
    int totalDof() const { return info_.K * info_.Np; }
    const MeshData& data() const { return mesh_; }

    // --- device residency of one conserved state ---------------------------
    // true when field f belongs to the state the device holds
    bool holds(const void* f) const {
        return f && (f == res_.rho || f == res_.rhoU || f == res_.Ener);
    }
    // the device's values into the resident fields' host arrays, if newer
    inline void pull() const;
    // forget the device copy (after pulling it)
    void drop() const {
        res_ = EulerState{nullptr, nullptr, nullptr};
        host_stale_ = false;
    }
    // make s the device's state (uploads its host values unless s is resident)
    inline void make_resident(const EulerState& s) const;
    // the device holds a newer state than the fields' host arrays
    void mark_device_newer() const { host_stale_ = true; }
    bool host_stale() const { return host_stale_; }

   private:
    MeshData mesh_;
    dg_ctx* ctx_ = nullptr;
    dg_info info_{};
    mutable EulerState res_{nullptr, nullptr, nullptr};
    mutable bool host_stale_ = false;
};

// nodal DOF field: component arrays of K*Np doubles in the reference node order
template <int NC>
class GeometricDofField {
   public:
    explicit GeometricDofField(const dgMesh& m) : mesh_(&m) {
        for (auto& c : comp_) c.assign(m.totalDof(), 0.0);
    }
    // copy (the reference's dgScalarField rho1("rho1", rho)): reads o's current values
    GeometricDofField(const GeometricDofField& o) : mesh_(o.mesh_) {
        o.read_sync();
        comp_ = o.comp_;
    }
    // assignment (rho1 = rho, dgEulerFoam.C:70-72)
    GeometricDofField& operator=(const GeometricDofField& o) {
        if (this != &o) {
            o.read_sync();
            write_sync();
            comp_ = o.comp_;
        }
        return *this;
    }
    ~GeometricDofField() {
        if (mesh_->holds(this)) {
            try {
                mesh_->pull();  // the other fields of the state keep their values
            } catch (...) {
            }
            mesh_->drop();
        }
    }
    // writable host values: brings them up to date and drops the device copy
    std::vector<double>& component(int c) {
        write_sync();
        return comp_[c];
    }
    // read-only host values: brings them up to date, the device copy stays valid
    const std::vector<double>& component(int c) const {
        read_sync();
        return comp_[c];
    }
    const dgMesh& mesh() const { return *mesh_; }
    // old-time level kept on the device by the time integrators
    void storeOldTime() {}
    void correctBoundaryConditions() {}
    // cubature / face values are formed inside the fused stage kernel
    void updateGaussField() {}
    struct GaussField {
        const GeometricDofField* field;
    };
    GaussField gaussField() const { return GaussField{this}; }

   private:
    friend class dgMesh;
    void read_sync() const {
        if (mesh_->holds(this) && mesh_->host_stale()) mesh_->pull();
    }
    void write_sync() {
        read_sync();
        if (mesh_->holds(this)) mesh_->drop();
    }
    const dgMesh* mesh_;
    std::array<std::vector<double>, NC> comp_;
};

// gauss-point fields of dgGaussField (fields/dgGaussField/dgGaussField.H:115-121)
template <int NC>
using dgGaussField = typename GeometricDofField<NC>::GaussField;

// gther_U = rhoU.gaussField() / rho.gaussField() (dgEulerFoam.C:81): the
// velocity at the cubature and face points, recorded by its operands
struct dgGaussVectorField {
    const dgVectorField* rhoU = nullptr;
    const dgScalarField* rho = nullptr;
};
inline dgGaussVectorField operator/(const dgGaussField<2>& rhoU, const dgGaussField<1>& rho) {
    return dgGaussVectorField{rhoU.field, rho.field};
}

// gther_p = (gamma - 1) (Ener - 0.5 rho |U|^2) at the same points (dgEulerFoam.C:82)
struct dgGaussScalarField {
    const dgScalarField* rho = nullptr;
    const dgVectorField* rhoU = nullptr;
    const dgScalarField* Ener = nullptr;
    double gamma = 0.0;
};
inline dgGaussScalarField pressure(double gamma, const dgGaussField<1>& rho, const dgGaussVectorField& U,
                                   const dgGaussField<1>& Ener) {
    if (U.rho != rho.field) throw Error(DG_ERR_ARG, "pressure: velocity and density of different states");
    return dgGaussScalarField{rho.field, U.rhoU, Ener.field, gamma};
}

inline void dgMesh::pull() const {
    if (!host_stale_ || !res_.rho) return;
    const size_t n = totalDof();
    std::vector<double> q(4 * n);
    check(ctx_, dg_download_state(ctx_, q.data()), "download");
    std::copy(q.begin(), q.begin() + n, res_.rho->comp_[0].begin());
    std::copy(q.begin() + n, q.begin() + 2 * n, res_.rhoU->comp_[0].begin());
    std::copy(q.begin() + 2 * n, q.begin() + 3 * n, res_.rhoU->comp_[1].begin());
    std::copy(q.begin() + 3 * n, q.end(), res_.Ener->comp_[0].begin());
    host_stale_ = false;
}

inline void dgMesh::make_resident(const EulerState& s) const {
    if (res_ == s) return;
    pull();  // another state's newer device values reach its fields first
    const size_t n = totalDof();
    std::vector<double> q(4 * n);
    std::copy(s.rho->comp_[0].begin(), s.rho->comp_[0].end(), q.begin());
    std::copy(s.rhoU->comp_[0].begin(), s.rhoU->comp_[0].end(), q.begin() + n);
    std::copy(s.rhoU->comp_[1].begin(), s.rhoU->comp_[1].end(), q.begin() + 2 * n);
    std::copy(s.Ener->comp_[0].begin(), s.Ener->comp_[0].end(), q.begin() + 3 * n);
    check(ctx_, dg_upload_state(ctx_, q.data()), "upload");
    res_ = s;
    host_stale_ = false;
}

class godunovScheme;

// Godunov.fluxRho() / fluxRhoU() / fluxEner(): the numerical flux of one
// conserved variable, evaluated inside the stage kernel
template <int NC>
struct FluxField {
    const godunovScheme* scheme;
    int var;  // 0 rho, 1 rhoU, 2 Ener
};

class godunovScheme {
   public:
    godunovScheme(const dgMesh& m, const std::string& flux) : mesh_(&m) {
        if (flux == "Roe") kind_ = DG_FLUX_ROE;
        else if (flux == "LF") kind_ = DG_FLUX_LF;
        else throw Error(DG_ERR_ARG, "unknown godunov flux scheme " + flux);
    }
    // godunovScheme::update(U, p, gamma, rho, rhoU, Ener) (godunovScheme.C:75-86):
    // records the state whose fluxes the next stage evaluates
    void update(const dgGaussVectorField& U, const dgGaussScalarField& p, double gamma, const dgGaussField<1>& rho,
                const dgGaussField<2>& rhoU, const dgGaussField<1>& Ener) {
        if (U.rho != rho.field || U.rhoU != rhoU.field || p.Ener != Ener.field || p.rho != rho.field)
            throw Error(DG_ERR_ARG, "godunovScheme::update: primitive fields of another state");
        (void)gamma;  // the context's gamma (dg_opts) is used by the kernels
        state_ = {const_cast<dgScalarField*>(rho.field), const_cast<dgVectorField*>(rhoU.field),
                  const_cast<dgScalarField*>(Ener.field)};
    }
    void update(dgScalarField& rho, dgVectorField& rhoU, dgScalarField& Ener) { state_ = {&rho, &rhoU, &Ener}; }
    int kind() const { return kind_; }
    const EulerState& state() const { return state_; }
    FluxField<1> fluxRho() const { return {this, 0}; }
    FluxField<2> fluxRhoU() const { return {this, 1}; }
    FluxField<1> fluxEner() const { return {this, 2}; }
    const dgMesh& mesh() const { return *mesh_; }

   private:
    const dgMesh* mesh_;
    int kind_ = DG_FLUX_ROE;
    EulerState state_{nullptr, nullptr, nullptr};
};

// recorded equation: ddt(field) + div(U, field, flux) [+ pressure term]
struct Equation {
    int var = -1;  // 0 rho, 1 rhoU, 2 Ener
    const void* field = nullptr;
    bool ddt = false;
    bool div = false;
    bool pressure = false;
    const godunovScheme* scheme = nullptr;
};
inline Equation operator+(Equation a, const Equation& b) {
    if (a.field && b.field && a.field != b.field) throw Error(DG_ERR_ARG, "equation terms of different fields");
    a.var = a.var >= 0 ? a.var : b.var;
    a.field = a.field ? a.field : b.field;
    a.scheme = a.scheme ? a.scheme : b.scheme;
    a.ddt |= b.ddt;
    a.div |= b.div;
    a.pressure |= b.pressure;
    return a;
}

namespace dgm {
// dgm::ddt(vf) (dgmDdt.C:46-54)
template <int NC>
inline Equation ddt(const GeometricDofField<NC>& f) {
    Equation e;
    e.field = &f;
    e.ddt = true;
    return e;
}
}  // namespace dgm

namespace dgc {
// dgc::div(U, vf, flux) (dgcDiv.H:76-90): the weak divergence of the
// convective flux of vf with the Godunov numerical flux on the faces
template <int NC>
inline Equation div(const dgGaussVectorField& U, const GeometricDofField<NC>& vf, const FluxField<NC>& flux) {
    (void)U;
    Equation e;
    e.var = flux.var;
    e.field = &vf;
    e.div = true;
    e.scheme = flux.scheme;
    return e;
}
// dgc::grad(gther_p) (EquationGradScheme.H:70): the momentum equation's pressure term
inline Equation grad(const dgGaussScalarField&) {
    Equation e;
    e.var = 1;
    e.pressure = true;
    return e;
}
// dgc::div(gther_U, gther_p) (EquationConvectionScheme.H:89-96): the energy equation's p U term
inline Equation div(const dgGaussVectorField&, const dgGaussScalarField&) {
    Equation e;
    e.var = 2;
    e.pressure = true;
    return e;
}
}  // namespace dgc

// time control of the stages: dgm::ddt's deltaT (runTime.deltaT()), the
// scheme whose state is advanced and the arithmetic of the stage kernel
class StageRunner {
   public:
    static StageRunner& get() {
        static StageRunner r;
        return r;
    }
    godunovScheme* scheme = nullptr;
    double dt = 0.0;
    int precision = DG_PREC_FP64;
    unsigned seen = 0;
};

namespace dg {
// Forward-Euler stage dg::solveEquation(dgm::ddt(q) + R(q)) for the three
// conserved fields (Equation/Equation.C:39-75): runs one fused stage on the
// device (dg_forward_euler_stage) when the set {rho, rhoU, Ener} of the
// current stage is complete; the new state stays on the device.
inline void solveEquation(const Equation& e) {
    StageRunner& R = StageRunner::get();
    if (!e.ddt || !e.div || e.var < 0) throw Error(DG_ERR_ARG, "solveEquation: expected ddt(q) + dgc::div(U, q, flux)");
    godunovScheme* g = R.scheme ? R.scheme : const_cast<godunovScheme*>(e.scheme);
    if (!g || !(R.dt > 0)) throw Error(DG_ERR_ARG, "solveEquation: stage not configured (scheme, deltaT)");
    const EulerState& s = g->state();
    const void* want[3] = {s.rho, s.rhoU, s.Ener};
    if (e.field != want[e.var]) throw Error(DG_ERR_ARG, "solveEquation: field is not the scheme's current state");
    R.seen |= 1u << e.var;
    if (R.seen == 7u) {
        const dgMesh& m = g->mesh();
        m.make_resident(s);
        check(m.ctx(), dg_forward_euler_stage(m.ctx(), R.dt, g->kind(), R.precision), "solveEquation");
        m.mark_device_newer();
        R.seen = 0;
    }
}
}  // namespace dg

// whole time steps on the device (state uploaded unless resident, read back on access)
inline void lserk4(const EulerState& s, const godunovScheme& g, double dt, int nsteps, int precision) {
    const dgMesh& m = s.rho->mesh();
    m.make_resident(s);
    check(m.ctx(), dg_lserk4_step(m.ctx(), dt, nsteps, g.kind(), precision), "lserk4");
    m.mark_device_newer();
}

inline void ssprk2(const EulerState& s, const godunovScheme& g, double dt, int nsteps, int precision) {
    const dgMesh& m = s.rho->mesh();
    m.make_resident(s);
    check(m.ctx(), dg_ssprk2_step(m.ctx(), dt, nsteps, g.kind(), precision), "ssprk2");
    m.mark_device_newer();
}

// pressure equation: dg::solveEquation(dgm::laplacian(p) == b) with KSP cg
class laplacianSolver {
   public:
    laplacianSolver(const dgMesh& m, double tau_coef = 20.0) : mesh_(&m) {
        check(m.ctx(), dg_ipdg_setup(m.ctx(), tau_coef), "dgm::laplacian");
    }
    // solves laplacian(p) = b_ref (reference sign) to rtol; returns the stats
    dg_solve_stats solve(const std::vector<double>& b_ref, dgScalarField& p, double rtol, int maxit,
                         int pc = DG_PC_BLOCK_JACOBI, int precision = DG_PREC_SPLIT) {
        std::vector<double> b(b_ref.size());
        for (size_t i = 0; i < b.size(); i++) b[i] = -b_ref[i];
        dg_solve_stats st{};
        check(mesh_->ctx(), dg_pcg_solve(mesh_->ctx(), b.data(), p.component(0).data(), rtol, maxit, pc, precision, &st),
              "dg::solveEquation(laplacian)");
        return st;
    }
    // the same on device vectors (reference sign handled by the caller: b_dev
    // is the SPD system's right-hand side, -b_ref), no host staging
    dg_solve_stats solve_device(const double* b_dev, double* p_dev, double rtol, int maxit,
                                int pc = DG_PC_BLOCK_JACOBI, int precision = DG_PREC_SPLIT) {
        dg_solve_stats st{};
        check(mesh_->ctx(), dg_pcg_solve_device(mesh_->ctx(), b_dev, p_dev, rtol, maxit, pc, precision, &st),
              "dg::solveEquation(laplacian)");
        return st;
    }

   private:
    const dgMesh* mesh_;
};

}  // namespace dgcu
