// dgEulerFoam.cpp -- the reference's isentropic-vortex solver loop
// (tutorials/DG/2D/isentropicVortex/dgEulerFoam/dgEulerFoam.C:64-131) written
// against the dgcu C++ stand-ins, with the reference's call signatures: SSP-RK2
// stages as three dg::solveEquation calls each (the state stays on the device
// between the stages), on a periodic square mesh, then the same number
// of steps with the device-resident integrator; prints both results' rho error
// against the exact advected vortex and their difference.
//
// usage: dgEulerFoam <tri_cubature.txt> [nx] [order] [steps]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>

#include "../../include/dgcu.hpp"

static std::vector<double> load_cubature(const char* path, int strength) {
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream is(line);
        std::string tag;
        int q, n;
        is >> tag >> q >> n;
        std::vector<double> out;
        for (int i = 0; i < n; i++) {
            std::getline(f, line);
            std::istringstream ps(line);
            double r, s, w;
            ps >> r >> s >> w;
            out.push_back(r);
            out.push_back(s);
            out.push_back(w);
        }
        if (q == strength) return out;
    }
    return {};
}

static dgcu::MeshData periodic(int nx, double L) {
    dgcu::MeshData m;
    const double h = L / nx;
    auto vid = [&](int i, int j) { return ((j + nx) % nx) * nx + (i + nx) % nx; };
    for (int j = 0; j < nx; j++)
        for (int i = 0; i < nx; i++) {
            const int v00 = vid(i, j), v10 = vid(i + 1, j), v11 = vid(i + 1, j + 1), v01 = vid(i, j + 1);
            const double x0 = i * h, y0 = j * h, x1 = x0 + h, y1 = y0 + h;
            m.EToV.insert(m.EToV.end(), {v00, v10, v11});
            m.VXY.insert(m.VXY.end(), {x0, y0, x1, y0, x1, y1});
            m.EToV.insert(m.EToV.end(), {v00, v11, v01});
            m.VXY.insert(m.VXY.end(), {x0, y0, x1, y1, x0, y1});
        }
    const int K = m.K();
    m.EToE.assign(3 * K, -1);
    m.EToF.assign(3 * K, -1);
    // connectivity by shared vertex pairs
    std::vector<std::vector<std::pair<int, int>>> byv(nx * nx);
    for (int k = 0; k < K; k++)
        for (int f = 0; f < 3; f++) byv[m.EToV[3 * k + f]].push_back({k, f});
    for (int k = 0; k < K; k++)
        for (int f = 0; f < 3; f++) {
            const int a = m.EToV[3 * k + f], b = m.EToV[3 * k + (f + 1) % 3];
            for (auto& kf : byv[b]) {
                const int k2 = kf.first, f2 = kf.second;
                if (k2 != k && m.EToV[3 * k2 + (f2 + 1) % 3] == a) {
                    m.EToE[3 * k + f] = k2;
                    m.EToF[3 * k + f] = f2;
                }
            }
        }
    return m;
}

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s tri_cubature.txt [nx] [order] [steps]\n", argv[0]);
        return 2;
    }
    const int nx = argc > 2 ? atoi(argv[2]) : 16;
    const int N = argc > 3 ? atoi(argv[3]) : 3;
    const int steps = argc > 4 ? atoi(argv[4]) : 10;
    const double L = 10.0, gamma = 1.4, beta = 5.0, pi = 3.14159265358979323846;
    try {
        dgcu::dgMesh mesh(periodic(nx, L), N, gamma, load_cubature(argv[1], 3 * (N + 1)));
        const int Np = mesh.nDofPerCell(), K = mesh.nCells();
        std::vector<double> r(Np), s(Np);
        std::vector<double> cub = load_cubature(argv[1], 3 * (N + 1));
        dgcu::check(nullptr, dg_reference_operators(N, cub.data(), (int)cub.size() / 3, r.data(), s.data(), nullptr,
                                                    nullptr, nullptr, nullptr, nullptr),
                    "operators");
        dgcu::dgScalarField rho(mesh), Ener(mesh), rho2(mesh), Ener2(mesh);
        dgcu::dgVectorField rhoU(mesh), rhoU2(mesh);
        auto exact = [&](double x, double y, double t, double* q) {  // setNonUniformInlet.H:20-26, centre (5,5)
            const double dx = x - 5.0 - t, dy = y - 5.0, r2 = dx * dx + dy * dy;
            const double rh = std::pow(1.0 - (gamma - 1.0) * beta * beta * std::exp(2.0 * (1.0 - r2)) / (16.0 * gamma * pi * pi),
                                       1.0 / (gamma - 1.0));
            const double u = 1.0 - beta * std::exp(1.0 - r2) * dy / (2.0 * pi);
            const double v = beta * std::exp(1.0 - r2) * dx / (2.0 * pi);
            q[0] = rh;
            q[1] = rh * u;
            q[2] = rh * v;
            q[3] = std::pow(rh, gamma) / (gamma - 1.0) + 0.5 * rh * (u * u + v * v);
        };
        const auto& M = mesh.data();
        std::vector<double> X(K * Np), Y(K * Np);
        for (int k = 0; k < K; k++)
            for (int i = 0; i < Np; i++) {
                const double* v = &M.VXY[6 * k];
                X[k * Np + i] = -(r[i] + s[i]) * 0.5 * v[0] + (r[i] + 1) * 0.5 * v[2] + (s[i] + 1) * 0.5 * v[4];
                Y[k * Np + i] = -(r[i] + s[i]) * 0.5 * v[1] + (r[i] + 1) * 0.5 * v[3] + (s[i] + 1) * 0.5 * v[5];
                double q[4];
                exact(X[k * Np + i], Y[k * Np + i], 0.0, q);
                rho.component(0)[k * Np + i] = rho2.component(0)[k * Np + i] = q[0];
                rhoU.component(0)[k * Np + i] = rhoU2.component(0)[k * Np + i] = q[1];
                rhoU.component(1)[k * Np + i] = rhoU2.component(1)[k * Np + i] = q[2];
                Ener.component(0)[k * Np + i] = Ener2.component(0)[k * Np + i] = q[3];
            }
        const double dt = 0.2 * (L / nx) / ((N + 1) * (N + 1) * 2.5);
        dgcu::godunovScheme Godunov(mesh, "Roe");
        dgcu::StageRunner::get().scheme = &Godunov;
        dgcu::StageRunner::get().dt = dt;
        // the reference's loop: two solveEquation stages and the SSP average
        dgcu::dgScalarField rho1(rho), Ener1(Ener);
        dgcu::dgVectorField rhoU1(rhoU);
        for (int n = 0; n < steps; n++) {
            rho1 = rho;
            rhoU1 = rhoU;
            Ener1 = Ener;
            for (int stage = 0; stage < 2; stage++) {
                rho1.updateGaussField();
                rhoU1.updateGaussField();
                Ener1.updateGaussField();
                dgcu::dgGaussVectorField gther_U = rhoU1.gaussField() / rho1.gaussField();
                dgcu::dgGaussScalarField gther_p = dgcu::pressure(gamma, rho1.gaussField(), gther_U, Ener1.gaussField());
                Godunov.update(gther_U, gther_p, gamma, rho1.gaussField(), rhoU1.gaussField(), Ener1.gaussField());
                dgcu::dg::solveEquation(dgcu::dgm::ddt(rho1) + dgcu::dgc::div(gther_U, rho1, Godunov.fluxRho()));
                dgcu::dg::solveEquation(dgcu::dgm::ddt(rhoU1) + dgcu::dgc::div(gther_U, rhoU1, Godunov.fluxRhoU()) +
                                        dgcu::dgc::grad(gther_p));
                dgcu::dg::solveEquation(dgcu::dgm::ddt(Ener1) + dgcu::dgc::div(gther_U, Ener1, Godunov.fluxEner()) +
                                        dgcu::dgc::div(gther_U, gther_p));
            }
            // rho = 0.5 rho + 0.5 rho1 (the stage results stay on the device until read here)
            const dgcu::dgScalarField& r1 = rho1;
            const dgcu::dgVectorField& ru1 = rhoU1;
            const dgcu::dgScalarField& e1 = Ener1;
            std::vector<double>&a = rho.component(0), &b = rhoU.component(0), &c = rhoU.component(1),
                              &d = Ener.component(0);
            for (size_t i = 0; i < (size_t)K * Np; i++) {
                a[i] = 0.5 * a[i] + 0.5 * r1.component(0)[i];
                b[i] = 0.5 * b[i] + 0.5 * ru1.component(0)[i];
                c[i] = 0.5 * c[i] + 0.5 * ru1.component(1)[i];
                d[i] = 0.5 * d[i] + 0.5 * e1.component(0)[i];
            }
        }
        // the same steps with the device-resident integrator
        dgcu::ssprk2({&rho2, &rhoU2, &Ener2}, Godunov, dt, steps, DG_PREC_FP64);
        double err = 0, diff = 0, nrm = 0;
        for (size_t i = 0; i < (size_t)K * Np; i++) {
            double q[4];
            exact(X[i], Y[i], steps * dt, q);
            err += std::fabs(rho.component(0)[i] - q[0]);
            diff = std::fmax(diff, std::fabs(rho.component(0)[i] - rho2.component(0)[i]));
            nrm = std::fmax(nrm, std::fabs(rho2.component(0)[i]));
        }
        printf("dgEulerFoam K=%d N=%d steps=%d dt=%.3e  rho mean abs error %.3e  solveEquation-vs-integrator max diff %.3e\n",
               K, N, steps, dt, err / (K * Np), diff / nrm);
        return (diff / nrm < 1e-12) ? 0 : 1;
    } catch (const dgcu::Error& e) {
        fprintf(stderr, "dgcu error: %s\n", e.what());
        return 3;
    }
}
