// dgcu.hpp -- C++ stand-ins for HopeFOAM's DG operator API over the dgcu C ABI.
//
// A HopeFOAM solver loop such as tutorials/DG/2D/isentropicVortex/dgEulerFoam/
// dgEulerFoam.C:64-131 keeps its shape:
//
//   dgcu::dgMesh mesh(desc, order, gamma);                 // dgMesh(IOobject)       dgMesh/dgMesh.C:71-116
//   dgcu::dgScalarField rho(mesh), Ener(mesh);             // GeometricDofField      fields/GeometricDofField
//   dgcu::dgVectorField rhoU(mesh);
//   dgcu::godunovScheme Godunov(mesh, "Roe");              // godunovScheme          DG/godunovFlux/godunovScheme.C:41-73
//   ...
//   Godunov.update(rho1, rhoU1, Ener1);                    // godunovScheme::update  :75-86
//   dgcu::dg::solveEquation(dgcu::dgm::ddt(rho1)  + dgcu::dgc::div(Godunov.fluxRho()));
//   dgcu::dg::solveEquation(dgcu::dgm::ddt(rhoU1) + dgcu::dgc::div(Godunov.fluxRhoU()) + dgcu::dgc::grad());
//   dgcu::dg::solveEquation(dgcu::dgm::ddt(Ener1) + dgcu::dgc::div(Godunov.fluxEner()) + dgcu::dgc::divUp());
//
// The GPU evaluates the three conserved equations of one stage in a single
// fused kernel, so the equations are recorded and the stage runs when the
// last of the three is solved (the reference solves them back to back on the
// same state, dgEulerFoam.C:86-90, so the result is the same).  Time stepping
// helpers (lserk4, ssprk2) run whole steps on the device.  Errors throw
// dgcu::Error (a std::runtime_error carrying the DG_ERR_* code), the analogue
// of the reference's FatalError.
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

   private:
    MeshData mesh_;
    dg_ctx* ctx_ = nullptr;
    dg_info info_{};
};

// nodal DOF field: component arrays of K*Np doubles in the reference node order
template <int NC>
class GeometricDofField {
   public:
    explicit GeometricDofField(const dgMesh& m) : mesh_(&m) {
        for (auto& c : comp_) c.assign(m.totalDof(), 0.0);
    }
    std::vector<double>& component(int c) { return comp_[c]; }
    const std::vector<double>& component(int c) const { return comp_[c]; }
    const dgMesh& mesh() const { return *mesh_; }
    // old-time level kept on the device by the time integrators
    void storeOldTime() {}
    void correctBoundaryConditions() {}

   private:
    const dgMesh* mesh_;
    std::array<std::vector<double>, NC> comp_;
};
using dgScalarField = GeometricDofField<1>;
using dgVectorField = GeometricDofField<2>;  // x, y (the reference's z component stays 0)

// the three conserved fields of the Euler system
struct EulerState {
    dgScalarField* rho;
    dgVectorField* rhoU;
    dgScalarField* Ener;
};

inline void upload(const EulerState& s) {
    const dgMesh& m = s.rho->mesh();
    const size_t n = m.totalDof();
    std::vector<double> q(4 * n);
    std::copy(s.rho->component(0).begin(), s.rho->component(0).end(), q.begin());
    std::copy(s.rhoU->component(0).begin(), s.rhoU->component(0).end(), q.begin() + n);
    std::copy(s.rhoU->component(1).begin(), s.rhoU->component(1).end(), q.begin() + 2 * n);
    std::copy(s.Ener->component(0).begin(), s.Ener->component(0).end(), q.begin() + 3 * n);
    check(m.ctx(), dg_upload_state(m.ctx(), q.data()), "upload");
}

inline void download(const EulerState& s) {
    const dgMesh& m = s.rho->mesh();
    const size_t n = m.totalDof();
    std::vector<double> q(4 * n);
    check(m.ctx(), dg_download_state(m.ctx(), q.data()), "download");
    std::copy(q.begin(), q.begin() + n, s.rho->component(0).begin());
    std::copy(q.begin() + n, q.begin() + 2 * n, s.rhoU->component(0).begin());
    std::copy(q.begin() + 2 * n, q.begin() + 3 * n, s.rhoU->component(1).begin());
    std::copy(q.begin() + 3 * n, q.end(), s.Ener->component(0).begin());
}

class godunovScheme {
   public:
    godunovScheme(const dgMesh& m, const std::string& flux) : mesh_(&m) {
        if (flux == "Roe") kind_ = DG_FLUX_ROE;
        else if (flux == "LF") kind_ = DG_FLUX_LF;
        else throw Error(DG_ERR_ARG, "unknown godunov flux scheme " + flux);
    }
    void update(dgScalarField& rho, dgVectorField& rhoU, dgScalarField& Ener) { state_ = {&rho, &rhoU, &Ener}; }
    int kind() const { return kind_; }
    const EulerState& state() const { return state_; }
    // flux handles, as fluxRho() / fluxRhoU() / fluxEner() of the reference
    int fluxRho() const { return 0; }
    int fluxRhoU() const { return 1; }
    int fluxEner() const { return 2; }
    const dgMesh& mesh() const { return *mesh_; }

   private:
    const dgMesh* mesh_;
    int kind_ = DG_FLUX_ROE;
    EulerState state_{nullptr, nullptr, nullptr};
};

// recorded equation: ddt(field) + div(flux) [+ pressure term]
struct Equation {
    int var = -1;        // 0 rho, 1 rhoU, 2 Ener
    bool ddt = false;
    bool div = false;
    bool pressure = false;
};
inline Equation operator+(Equation a, const Equation& b) {
    a.var = a.var >= 0 ? a.var : b.var;
    a.ddt |= b.ddt;
    a.div |= b.div;
    a.pressure |= b.pressure;
    return a;
}

namespace dgm {
inline Equation ddt(const dgScalarField&) { return Equation{-1, true, false, false}; }
inline Equation ddt(const dgVectorField&) { return Equation{-1, true, false, false}; }
}  // namespace dgm

namespace dgc {
inline Equation div(int flux_component) { return Equation{flux_component, false, true, false}; }
inline Equation grad() { return Equation{1, false, false, true}; }   // dgc::grad(gther_p)
inline Equation divUp() { return Equation{2, false, false, true}; }  // dgc::div(gther_U, gther_p)
}  // namespace dgc

// Forward-Euler stage dg::solveEquation(dgm::ddt(q) + R(q)) for the three
// conserved fields (Equation/Equation.C:39-75): runs one fused stage on the
// device when the set {rho, rhoU, Ener} of the current stage is complete.
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
inline void solveEquation(const Equation& e) {
    StageRunner& R = StageRunner::get();
    if (!R.scheme || !e.ddt || !e.div) throw Error(DG_ERR_ARG, "solveEquation: stage not configured");
    R.seen |= 1u << e.var;
    if (R.seen == 7u) {
        const EulerState& s = R.scheme->state();
        dg_ctx* ctx = R.scheme->mesh().ctx();
        upload(s);
        // one forward-Euler stage q <- q + dt M^-1 R_weak(q)
        std::vector<double> rhs(4 * (size_t)R.scheme->mesh().totalDof());
        check(ctx, dg_euler_rhs(ctx, R.scheme->kind(), R.precision, rhs.data()), "solveEquation");
        const size_t n = R.scheme->mesh().totalDof();
        for (size_t i = 0; i < n; i++) {
            s.rho->component(0)[i] += R.dt * rhs[i];
            s.rhoU->component(0)[i] += R.dt * rhs[n + i];
            s.rhoU->component(1)[i] += R.dt * rhs[2 * n + i];
            s.Ener->component(0)[i] += R.dt * rhs[3 * n + i];
        }
        R.seen = 0;
    }
}
}  // namespace dg

// whole time steps on the device (state uploaded once, downloaded at the end)
inline void lserk4(const EulerState& s, const godunovScheme& g, double dt, int nsteps, int precision) {
    dg_ctx* ctx = s.rho->mesh().ctx();
    upload(s);
    check(ctx, dg_lserk4_step(ctx, dt, nsteps, g.kind(), precision), "lserk4");
    download(s);
}

inline void ssprk2(const EulerState& s, const godunovScheme& g, double dt, int nsteps, int precision) {
    dg_ctx* ctx = s.rho->mesh().ctx();
    upload(s);
    check(ctx, dg_ssprk2_step(ctx, dt, nsteps, g.kind(), precision), "ssprk2");
    download(s);
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

   private:
    const dgMesh* mesh_;
};

}  // namespace dgcu
