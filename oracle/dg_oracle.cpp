// dg_oracle.cpp -- CPU restatement (FP64) of HopeFOAM's 2D nodal-DG hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU path is
// checked against (parity tests, smoke check) and the CPU baseline that
// bench.py times.  Nothing in the product library links or calls it.
//
// It follows the reference's algorithms and loop structure function by
// function (paths relative to HopeFOAM-0.1/src/DG):
//   Legendre.C:38-166 (JacobiGQ), :169-183 (JacobiGL), :185-220 (JacobiP),
//     :222-241 (GradJacobiP), :245-250 (gamma), :253-310 (Vandermonde1D/2D),
//     :387-450 (GradVandermonde2D), :540- (matrixInv)
//   element/baseFunctions/.../triangleBaseFunction.C:46-71 (ctor), :75-94
//     (faceToCellIndex), :122-186 (warp-blend nodes), :189-234 (warpFactor),
//     :236-246 (Dr), :303-343 (x(r,s), dxdr, drdx), :393-419 (faceFscale)
//   element/gaussIntegration/gaussIntegration/gaussIntegration.C:62-69
//   element/gaussIntegration/gaussTriangleIntegration/gaussTriangleIntegration.C
//     :45-97 (cubature, cellVandermonde, cellDr, face Gauss rule, faceInterp),
//     :127-151 (cellDrdx, cellWJ), :153-192 (faceNxWJ)
//   element/physicalElementData/physicalCellElement.C:72-110 (initElement,
//     mass matrix, cellD1dx)
//   element/physicalElementData/physicalElementData.C:60-161 (faces, gauss
//     starts), :228-263 (normals, WJ, fscale), :265-343 (face Dn)
//   fields/dgGaussField/dgGaussField.C:190-269 (initField: cell and face
//     gauss interpolation, boundary traces)
//   DG/godunovFlux/fluxSchemes/scheme/RoeFlux/RoeFlux.C:46-191 (Roe flux)
//   DG/convectionSchemes/defaultConvectionScheme/defaultConvectionScheme.C:48-129
//   DG/gradSchemes/defaultGrad/defaultGrad.C:87-166
//   DG/divSchemes/defaultDivScheme/defaultDivScheme.C:85-166
//   DG/ddtSchemes/EulerDdtScheme/EulerDdtScheme.C:118-144, Equation/Equation.C:39-75,
//     dgMatrices/dgMatrix/dgMatrix.C:383-405 (b = M q_old/dt + R; b *= dt;
//     solve M q = b with the exact block LU of dgMesh.C:129-172)
//   tutorials/DG/2D/isentropicVortex/dgEulerFoam/dgEulerFoam.C:64-131 (SSP-RK2),
//     createFields.H:119-138 (LSERK4 coefficients), setBoundaryValues.H (exact
//     vortex boundary traces)
//   DG/laplacianSchemes/defaultLaplacianScheme/defaultLaplacianScheme.C:63-288
//     (SIPG element rows)
// Third-party arithmetic at the reference boundary (PETSc LU / KSP, SLEPc EPS)
// is replaced by dense LU with partial pivoting and an implicit-shift QL
// tridiagonal eigensolver; both agree with the reference to round-off.
//
// Additions that have no reference code and are pinned only by this oracle:
// the Euler Lax-Friedrichs (Rusanov) flux, LSERK4 time stepping, periodic
// faces treated as interior faces (rotation from shared vertex ids, exactly
// dgPolyMesh.C:866-893), and CG with a block-Jacobi preconditioner.

#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

typedef std::vector<double> vec;

struct Mat {
    int r = 0, c = 0;
    vec a;
    Mat() {}
    Mat(int r_, int c_, double v = 0.0) : r(r_), c(c_), a((size_t)r_ * c_, v) {}
    double& operator()(int i, int j) { return a[(size_t)i * c + j]; }
    double operator()(int i, int j) const { return a[(size_t)i * c + j]; }
};

static Mat matmul(const Mat& A, const Mat& B) {  // denseMatrix::MatMatMult loop order
    Mat C(A.r, B.c, 0.0);
    for (int i = 0; i < A.r; i++)
        for (int k = 0; k < A.c; k++) {
            double aik = A(i, k);
            for (int j = 0; j < B.c; j++) C(i, j) += aik * B(k, j);
        }
    return C;
}

// Legendre.C:540- (matrixInv via PETSc LU) -> dense LU with partial pivoting.
static Mat matinv(const Mat& A) {
    int n = A.r;
    Mat LU = A, X(n, n, 0.0);
    std::vector<int> piv(n);
    for (int i = 0; i < n; i++) piv[i] = i;
    for (int k = 0; k < n; k++) {
        int p = k;
        double best = std::fabs(LU(k, k));
        for (int i = k + 1; i < n; i++)
            if (std::fabs(LU(i, k)) > best) { best = std::fabs(LU(i, k)); p = i; }
        if (p != k) {
            for (int j = 0; j < n; j++) std::swap(LU(k, j), LU(p, j));
            std::swap(piv[k], piv[p]);
        }
        for (int i = k + 1; i < n; i++) {
            LU(i, k) /= LU(k, k);
            double l = LU(i, k);
            for (int j = k + 1; j < n; j++) LU(i, j) -= l * LU(k, j);
        }
    }
    for (int col = 0; col < n; col++) {
        vec y(n);
        for (int i = 0; i < n; i++) {
            double s = (piv[i] == col) ? 1.0 : 0.0;
            for (int j = 0; j < i; j++) s -= LU(i, j) * y[j];
            y[i] = s;
        }
        for (int i = n - 1; i >= 0; i--) {
            double s = y[i];
            for (int j = i + 1; j < n; j++) s -= LU(i, j) * X(j, col);
            X(i, col) = s / LU(i, i);
        }
    }
    return X;
}

// Legendre.C:245-250: gamma(x) = (x-1)! for integer arguments
static double lgamma_int(int x) {
    double ans = 1.0;
    for (int i = 2; i < x; i++) ans *= i;
    return ans;
}

// Legendre.C:185-220
static vec JacobiP(const vec& xp, double alpha, double beta, int N) {
    int dims = (int)xp.size();
    std::vector<vec> PL(N + 1, vec(dims, 0.0));
    double gamma0 = std::pow(2, alpha + beta + 1) / (alpha + beta + 1) * lgamma_int((int)(alpha + 1)) *
                    lgamma_int((int)(beta + 1)) / lgamma_int((int)(alpha + beta + 1));
    double gamma1 = (alpha + 1) * (beta + 1) / (alpha + beta + 3) * gamma0;
    for (int i = 0; i < dims; i++) PL[0][i] = 1.0 / std::sqrt(gamma0);
    if (N == 0) return PL[0];
    for (int i = 0; i < dims; i++) PL[1][i] = ((alpha + beta + 2) / 2 * xp[i] + (alpha - beta) / 2) / std::sqrt(gamma1);
    if (N == 1) return PL[1];
    double aold = 2 / (2 + alpha + beta) * std::sqrt((alpha + 1) * (beta + 1) / (alpha + beta + 3));
    for (int i = 1; i < N; i++) {
        double h1 = 2.0 * i + alpha + beta;
        double anew = 2 / (h1 + 2) *
                      std::sqrt((i + 1) * (i + 1 + alpha + beta) * (i + 1 + alpha) * (i + 1 + beta) / (h1 + 1) / (h1 + 3));
        double bnew = -(alpha * alpha - beta * beta) / h1 / (h1 + 2);
        for (int j = 0; j < dims; j++)
            PL[i + 1][j] = 1 / anew * ((0.0 - aold) * PL[i - 1][j] + (xp[j] - bnew) * PL[i][j]);
        aold = anew;
    }
    return PL[N];
}

// Legendre.C:222-231
static vec GradJacobiP(const vec& xp, double alpha, double beta, int N) {
    vec dP(xp.size(), 0.0);
    if (N == 0) return dP;
    vec p = JacobiP(xp, alpha + 1, beta + 1, N - 1);
    double f = std::sqrt(N * (N + alpha + beta + 1));
    for (size_t i = 0; i < p.size(); i++) dP[i] = f * p[i];
    return dP;
}

// Symmetric tridiagonal eigensolver (implicit-shift QL, eigenvectors
// accumulated).  Stands in for SLEPc's EPSSolve in Legendre.C:100-110.
static void tridiag_eig(vec d, vec e, vec& evals, Mat& Z) {
    int n = (int)d.size();
    Z = Mat(n, n, 0.0);
    for (int i = 0; i < n; i++) Z(i, i) = 1.0;
    e.push_back(0.0);
    for (int l = 0; l < n; l++) {
        int iter = 0;
        while (true) {
            int m;
            for (m = l; m < n - 1; m++) {
                double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
                if (std::fabs(e[m]) <= 1e-300 + 4e-17 * dd) break;
            }
            if (m == l) break;
            if (++iter > 200) { fprintf(stderr, "tridiag_eig: no convergence\n"); abort(); }
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = std::hypot(g, 1.0);
            g = d[m] - d[l] + e[l] / (g + (g >= 0 ? std::fabs(r) : -std::fabs(r)));
            double s = 1.0, c = 1.0, p = 0.0;
            int i;
            for (i = m - 1; i >= l; i--) {
                double f = s * e[i], b = c * e[i];
                r = std::hypot(f, g);
                e[i + 1] = r;
                if (r == 0.0) { d[i + 1] -= p; e[m] = 0.0; break; }
                s = f / r; c = g / r;
                g = d[i + 1] - p;
                r = (d[i] - g) * s + 2.0 * c * b;
                p = s * r;
                d[i + 1] = g + p;
                g = c * r - b;
                for (int k = 0; k < n; k++) {
                    f = Z(k, i + 1);
                    Z(k, i + 1) = s * Z(k, i) + c * f;
                    Z(k, i) = c * Z(k, i) - s * f;
                }
            }
            if (r == 0.0 && i >= l) continue;
            d[l] -= p; e[l] = g; e[m] = 0.0;
        }
    }
    evals = d;
}

// Legendre.C:38-166: Gauss nodes/weights from the Golub-Welsch matrix, then the
// reference's ascending sort and weight symmetrisation (:137-153).
static void JacobiGQ(double alpha, double beta, int N, vec& x, vec& w) {
    x.assign(N + 1, 0.0);
    w.assign(N + 1, 0.0);
    if (N == 0) {
        x[0] = -(alpha - beta) / (alpha + beta + 2);
        w[0] = 2;
        return;
    }
    vec d(N + 1, 0.0), e(N, 0.0);
    for (int i = 0; i < N; i++) {
        int j = i + 1;
        e[i] = 2 / (2 * i + alpha + beta + 2) *
               std::sqrt(j * (j + alpha + beta) * (j + alpha) * (j + beta) / (2 * i + alpha + beta + 1) /
                         (2 * i + alpha + beta + 3));
    }
    // The reference sets only the off-diagonal (and J(0,0)=0): valid for alpha == beta.
    vec ev;
    Mat Z;
    tridiag_eig(d, e, ev, Z);
    for (int i = 0; i <= N; i++) {
        x[i] = ev[i];
        double v0 = Z(0, i);
        w[i] = (v0 * v0) * std::pow(2, alpha + beta + 1) / (alpha + beta + 1) * lgamma_int((int)(alpha + 1)) *
               lgamma_int((int)(beta + 1)) / lgamma_int((int)(alpha + beta + 1));
    }
    for (int i = 0; i < N; i++)
        for (int j = i + 1; j <= N; j++)
            if (x[i] > x[j]) { std::swap(x[i], x[j]); std::swap(w[i], w[j]); }
    for (int i = 0; i <= (N - 1) / 2; i++) {
        double t = (w[i] + w[N - i]) * 0.5;
        w[i] = w[N - i] = t;
    }
}

// Legendre.C:169-183
static vec JacobiGL(double alpha, double beta, int N) {
    vec ans(N + 1, 0.0);
    ans[0] = -1.0;
    ans[N] = 1.0;
    if (N < 2) return ans;
    vec xi, wi;
    JacobiGQ(alpha + 1, beta + 1, N - 2, xi, wi);
    for (int i = 1; i < N; i++) ans[i] = xi[i - 1];
    return ans;
}

// Legendre.C:253-266
static Mat Vandermonde1D(int N, const vec& r) {
    Mat V((int)r.size(), N + 1);
    for (int i = 0; i <= N; i++) {
        vec t = JacobiP(r, 0, 0, i);
        for (size_t j = 0; j < r.size(); j++) V((int)j, i) = t[j];
    }
    return V;
}

// Legendre.C:277-301
static Mat Vandermonde2D(int N, const vec& r, const vec& s) {
    int n = (int)r.size();
    Mat V(n, (N + 1) * (N + 2) / 2);
    vec a(n), b(s);
    for (int i = 0; i < n; i++) a[i] = (s[i] != 1.0) ? 2 * (1 + r[i]) / (1 - s[i]) - 1 : -1.0;
    int sk = 0;
    double sqrt2 = std::sqrt(2.0);
    for (int i = 0; i <= N; i++)
        for (int j = 0; j <= N - i; j++) {
            vec h1 = JacobiP(a, 0, 0, i), h2 = JacobiP(b, 2 * i + 1, 0, j);
            for (int p = 0; p < n; p++) V(p, sk) = sqrt2 * h1[p] * h2[p] * std::pow(1 - b[p], i);
            sk++;
        }
    return V;
}

// Legendre.C:387-450
static void GradVandermonde2D(int N, const vec& r, const vec& s, Mat& Vr, Mat& Vs) {
    int n = (int)r.size(), Np = (N + 1) * (N + 2) / 2;
    Vr = Mat(n, Np);
    Vs = Mat(n, Np);
    vec a(n), b(s);
    for (int i = 0; i < n; i++) a[i] = (s[i] != 1.0) ? 2 * (1 + r[i]) / (1 - s[i]) - 1 : -1.0;
    int sk = 0;
    for (int i = 0; i <= N; i++)
        for (int j = 0; j <= N - i; j++) {
            vec fa = JacobiP(a, 0, 0, i), gb = JacobiP(b, 2 * i + 1, 0, j);
            vec dfa = GradJacobiP(a, 0, 0, i), dgb = GradJacobiP(b, 2 * i + 1, 0, j);
            double drCoeff = std::pow(2.0, i + 0.5);
            for (int p = 0; p < n; p++) {
                if (i > 0) {
                    Vr(p, sk) = dfa[p] * gb[p] * drCoeff * std::pow(0.5 * (1.0 - b[p]), i - 1);
                    double t = dgb[p] * std::pow(0.5 * (1 - b[p]), i) - 0.5 * i * gb[p] * std::pow(0.5 * (1 - b[p]), i - 1);
                    Vs(p, sk) = (dfa[p] * gb[p] * 0.5 * (1 + a[p]) * std::pow(0.5 * (1 - b[p]), i - 1) + fa[p] * t) *
                                std::pow(2.0, i + 0.5);
                } else {
                    Vr(p, sk) = dfa[p] * gb[p] * drCoeff;
                    double t = dgb[p] * std::pow(0.5 * (1 - b[p]), i);
                    Vs(p, sk) = (dfa[p] * gb[p] * 0.5 * (1 + a[p]) + fa[p] * t) * std::pow(2.0, i + 0.5);
                }
            }
            sk++;
        }
}

// ---------------------------------------------------------------------------
// triangleBaseFunction + gaussTriangleIntegration

struct TriBase {
    int N, Np, Nfp, Ng, Nfq;
    vec r, s;                 // nodes (reference order)
    Mat V, invV, Dr, Ds;      // Np x Np
    int fci[3][2][16];        // faceToCellIndex[face][rot][i]
    Mat invV1D;               // 1D inverse Vandermonde on LGL nodes
    vec gr, gs, gw;           // volume cubature
    Mat cellV, cellDr, cellDs;  // Ng x Np
    vec fq, fw;               // face Gauss points / weights (N+2)
    Mat faceInterp;           // Nfq x Nfp
    Mat faceInterpRot;        // columns permuted by rotate index 1
};

// triangleBaseFunction.C:189-234
static vec warpFactor(int N, const vec& rout) {
    vec LGLr = JacobiGL(0, 0, N);
    vec req(N + 1);
    double interval = 2.0 / N;
    for (int i = 0; i <= N; i++) req[i] = interval * i - 1;
    Mat Veq = Vandermonde1D(N, req);
    int n = (int)rout.size();
    Mat Pmat(N + 1, n);
    for (int i = 0; i <= N; i++) {
        vec t = JacobiP(rout, 0, 0, i);
        for (int j = 0; j < n; j++) Pmat(i, j) = t[j];
    }
    Mat VeqT(N + 1, N + 1);
    for (int i = 0; i <= N; i++)
        for (int j = 0; j <= N; j++) VeqT(i, j) = Veq(j, i);
    Mat Lmat = matmul(matinv(VeqT), Pmat);
    vec warp(n, 0.0);
    for (int j = 0; j < n; j++) {  // Lmat' * (LGLr - req)
        double sacc = 0;
        for (int k = 0; k <= N; k++) sacc += Lmat(k, j) * (LGLr[k] - req[k]);
        warp[j] = sacc;
    }
    for (int i = 0; i < n; i++) {
        double zerof = (std::fabs(rout[i]) < (1.0 - 1.0e-10)) ? 1.0 : 0.0;
        double sf = 1.0 - (zerof * rout[i]) * (zerof * rout[i]);
        warp[i] = warp[i] / sf + warp[i] * (zerof - 1.0);
    }
    return warp;
}

static void build_base(int N, const double* cub, int Ng, TriBase& B) {
    B.N = N;
    B.Np = (N + 1) * (N + 2) / 2;
    B.Nfp = N + 1;
    int Np = B.Np;
    // triangleBaseFunction.C:122-186 (warp-blend nodes)
    static const double alpopt[15] = {0.0000, 0.0000, 1.4152, 0.1001, 0.2751, 0.9800, 1.0999, 1.2832,
                                      1.3648, 1.4773, 1.4959, 1.5743, 1.5770, 1.6223, 1.6258};
    double alpha = (N < 16) ? alpopt[N - 1] : 5.0 / 3.0;
    vec L1(Np), L2(Np), L3(Np), X(Np), Y(Np);
    int sk = 0;
    for (int n = 1; n <= N + 1; n++)
        for (int m = 1; m <= N + 2 - n; m++) {
            L1[sk] = (double)(n - 1) / N;
            L3[sk] = (double)(m - 1) / N;
            sk++;
        }
    for (int i = 0; i < Np; i++) {
        L2[i] = 1.0 - L1[i] - L3[i];
        X[i] = L3[i] - L2[i];
        Y[i] = (2 * L1[i] - L2[i] - L3[i]) / std::sqrt(3.0);
    }
    vec d1(Np), d2(Np), d3(Np);
    for (int i = 0; i < Np; i++) { d1[i] = L3[i] - L2[i]; d2[i] = L1[i] - L3[i]; d3[i] = L2[i] - L1[i]; }
    vec w1 = warpFactor(N, d1), w2 = warpFactor(N, d2), w3 = warpFactor(N, d3);
    for (int i = 0; i < Np; i++) {
        w1[i] = 4 * L2[i] * L3[i] * w1[i] * (1 + (alpha * L1[i]) * (alpha * L1[i]));
        w2[i] = 4 * L1[i] * L3[i] * w2[i] * (1 + (alpha * L2[i]) * (alpha * L2[i]));
        w3[i] = 4 * L1[i] * L2[i] * w3[i] * (1 + (alpha * L3[i]) * (alpha * L3[i]));
    }
    const double pi = 3.14159265358979323846;
    double cos1 = std::cos(2 * pi / 3), cos2 = std::cos(4 * pi / 3);
    double sin1 = std::sin(2 * pi / 3), sin2 = std::sin(4 * pi / 3);
    B.r.assign(Np, 0.0);
    B.s.assign(Np, 0.0);
    for (int i = 0; i < Np; i++) {
        X[i] += 1 * w1[i] + cos1 * w2[i] + cos2 * w3[i];
        Y[i] += 0 * w1[i] + sin1 * w2[i] + sin2 * w3[i];
        double l1 = (std::sqrt(3.0) * Y[i] + 1.0) / 3.0;
        double l2 = (-3.0 * X[i] - std::sqrt(3.0) * Y[i] + 2.0) / 6.0;
        double l3 = (3.0 * X[i] - std::sqrt(3.0) * Y[i] + 2.0) / 6.0;
        B.r[i] = l3 - l2 - l1;
        B.s[i] = l1 - l2 - l3;
    }
    B.V = Vandermonde2D(N, B.r, B.s);
    B.invV = matinv(B.V);
    // 1D line element (lineBaseFunction.C:44-66)
    vec lgl = JacobiGL(0, 0, N);
    B.invV1D = matinv(Vandermonde1D(N, lgl));
    // faceToCellIndex (triangleBaseFunction.C:75-94)
    int Nfp = N + 1;
    for (int i = 0; i < Nfp; i++) B.fci[0][0][i] = i;
    B.fci[1][0][0] = N;
    B.fci[2][0][0] = Np - 1;
    for (int i = 1; i < Nfp; i++) {
        B.fci[1][0][i] = B.fci[1][0][i - 1] + (Nfp - i);
        B.fci[2][0][i] = B.fci[2][0][i - 1] - i - 1;
    }
    for (int f = 0; f < 3; f++)
        for (int i = 0; i < Nfp; i++) B.fci[f][1][i] = B.fci[f][0][N - i];
    // Dr (triangleBaseFunction.C:236-246)
    Mat Vr, Vs;
    GradVandermonde2D(N, B.r, B.s, Vr, Vs);
    B.Dr = matmul(Vr, B.invV);
    B.Ds = matmul(Vs, B.invV);
    // gaussTriangleIntegration.C:45-97
    B.Ng = Ng;
    B.gr.resize(Ng);
    B.gs.resize(Ng);
    B.gw.resize(Ng);
    for (int i = 0; i < Ng; i++) { B.gr[i] = cub[3 * i]; B.gs[i] = cub[3 * i + 1]; B.gw[i] = cub[3 * i + 2]; }
    B.cellV = matmul(Vandermonde2D(N, B.gr, B.gs), B.invV);
    Mat Gr, Gs;
    GradVandermonde2D(N, B.gr, B.gs, Gr, Gs);
    B.cellDr = matmul(Gr, B.invV);
    B.cellDs = matmul(Gs, B.invV);
    JacobiGQ(0, 0, (2 * (N + 1)) / 2, B.fq, B.fw);
    B.Nfq = (int)B.fq.size();
    B.faceInterp = matmul(Vandermonde1D(N, B.fq), B.invV1D);
    B.faceInterpRot = Mat(B.Nfq, Nfp);
    for (int i = 0; i < B.Nfq; i++)
        for (int j = 0; j < Nfp; j++) B.faceInterpRot(i, j) = B.faceInterp(i, N - j);
}

// ---------------------------------------------------------------------------
// mesh, elements, faces

struct Face {
    int owner, nbr, fo, fn, rot;  // rot = firstPointIndex of the owner face
    int start;                    // ownerFaceStart_
    vec nx, ny, wJ;               // at owner gauss points
    double fscale;
    Mat DnO, DnN, DnNrot;         // gaussOwnerFaceDn_, gaussNeighborFaceDn_, ...Rotate_
};

struct Oracle {
    TriBase B;
    int K;
    std::vector<int> EToV;      // K x 3 (after CCW reorder)
    vec VXY;                    // K x 3 x 2 element vertex coordinates
    vec x, y;                   // physical nodes, K x Np
    std::vector<std::array<double, 4>> dxdr;   // at nodes: xr, yr, xs, ys (K*Np)
    vec wJ;                     // K x Ng jacobianWeights
    vec D1x, D1y;               // K x Ng x Np cellD1dx
    std::vector<Mat> M, Minv;   // per element mass matrix and its inverse
    std::vector<Face> faces;
    std::vector<std::array<int, 3>> cellFace;  // face id of each element face
    std::vector<std::array<int, 3>> EToE, EToF;
    int nFaceGauss = 0;
};


static void build_oracle(Oracle& O, int N, int K, const int* EToV_in, const double* VXY_in, const double* cub, int Ng) {
    build_base(N, cub, Ng, O.B);
    TriBase& B = O.B;
    int Np = B.Np, Nfp = B.Nfp;
    O.K = K;
    O.EToV.assign(EToV_in, EToV_in + 3 * K);
    O.VXY.assign(VXY_in, VXY_in + 6 * K);
    // dgPolyMesh.C:486-506: make every triangle counter-clockwise
    for (int k = 0; k < K; k++) {
        double* v = &O.VXY[6 * k];
        double ax = v[2] - v[0], ay = v[3] - v[1], bx = v[4] - v[0], by = v[5] - v[1];
        if (ax * by - ay * bx < 0) {
            std::swap(O.EToV[3 * k + 1], O.EToV[3 * k + 2]);
            std::swap(v[2], v[4]);
            std::swap(v[3], v[5]);
        }
    }
    // element data (physicalCellElement.C:72-110)
    O.x.assign((size_t)K * Np, 0);
    O.y.assign((size_t)K * Np, 0);
    O.dxdr.resize((size_t)K * Np);
    O.wJ.assign((size_t)K * Ng, 0);
    O.D1x.assign((size_t)K * Ng * Np, 0);
    O.D1y.assign((size_t)K * Ng * Np, 0);
    O.M.resize(K);
    O.Minv.resize(K);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; k++) {
        const double* v = &O.VXY[6 * k];
        double* xk = &O.x[(size_t)k * Np];
        double* yk = &O.y[(size_t)k * Np];
        for (int i = 0; i < Np; i++) {  // triangleBaseFunction.C:303-313
            double r = B.r[i], s = B.s[i];
            xk[i] = -(r + s) * 0.5 * v[0] + (r + 1) * 0.5 * v[2] + (s + 1) * 0.5 * v[4];
            yk[i] = -(r + s) * 0.5 * v[1] + (r + 1) * 0.5 * v[3] + (s + 1) * 0.5 * v[5];
        }
        for (int i = 0; i < Np; i++) {  // dxdr at nodes (MatVecOuterProduct)
            double xr = 0, yr = 0, xs = 0, ys = 0;
            for (int j = 0; j < Np; j++) {
                xr += B.Dr(i, j) * xk[j];
                yr += B.Dr(i, j) * yk[j];
                xs += B.Ds(i, j) * xk[j];
                ys += B.Ds(i, j) * yk[j];
            }
            O.dxdr[(size_t)k * Np + i] = {xr, yr, xs, ys};
        }
        vec rx(Ng), sx(Ng), ry(Ng), sy(Ng);
        for (int g = 0; g < Ng; g++) {  // cellDxdr, cellWJ, cellDrdx at cubature points
            double xr = 0, yr = 0, xs = 0, ys = 0;
            for (int j = 0; j < Np; j++) {
                xr += B.cellDr(g, j) * xk[j];
                yr += B.cellDr(g, j) * yk[j];
                xs += B.cellDs(g, j) * xk[j];
                ys += B.cellDs(g, j) * yk[j];
            }
            double J = xr * ys - yr * xs;
            O.wJ[(size_t)k * Ng + g] = J * B.gw[g];
            rx[g] = ys / J;
            sx[g] = -yr / J;
            ry[g] = -xs / J;
            sy[g] = xr / J;
        }
        Mat Mk(Np, Np, 0.0);  // MatDiagMatMult(Vg, wJ, Vg)
        for (int g = 0; g < Ng; g++)
            for (int i = 0; i < Np; i++)
                for (int j = 0; j < Np; j++) Mk(i, j) += B.cellV(g, i) * B.cellV(g, j) * O.wJ[(size_t)k * Ng + g];
        O.M[k] = Mk;
        O.Minv[k] = matinv(Mk);
        for (int g = 0; g < Ng; g++)
            for (int j = 0; j < Np; j++) {
                size_t p = ((size_t)k * Ng + g) * Np + j;
                O.D1x[p] = B.cellDr(g, j) * rx[g] + B.cellDs(g, j) * sx[g];
                O.D1y[p] = B.cellDr(g, j) * ry[g] + B.cellDs(g, j) * sy[g];
            }
    }
    // edge connectivity (dgPolyMesh calEdgeNeighbour / calNeighbourFace):
    // element faces are (v0,v1), (v1,v2), (v2,v0) (dgPolyMesh.C:601-613)
    O.EToE.assign(K, {-1, -1, -1});
    O.EToF.assign(K, {-1, -1, -1});
    std::map<std::pair<int, int>, std::pair<int, int>> edges;
    for (int k = 0; k < K; k++)
        for (int f = 0; f < 3; f++) {
            int a = O.EToV[3 * k + f], b = O.EToV[3 * k + (f + 1) % 3];
            std::pair<int, int> key(std::min(a, b), std::max(a, b));
            auto it = edges.find(key);
            if (it == edges.end()) {
                edges[key] = {k, f};
            } else {
                int k2 = it->second.first, f2 = it->second.second;
                O.EToE[k][f] = k2; O.EToF[k][f] = f2;
                O.EToE[k2][f2] = k; O.EToF[k2][f2] = f;
            }
        }
    // faces in cell-loop order, owner = lower element index
    // (physicalElementData.C:60-161, ownerFaceStart_ at :143-155)
    O.cellFace.assign(K, {-1, -1, -1});
    int Nfq = B.Nfq;
    for (int k = 0; k < K; k++)
        for (int f = 0; f < 3; f++) {
            int n = O.EToE[k][f];
            if (n >= 0 && n < k) continue;  // owned by the lower index
            Face F;
            F.owner = k; F.fo = f; F.nbr = n; F.fn = O.EToF[k][f];
            F.start = O.nFaceGauss;
            O.nFaceGauss += Nfq;
            if (n >= 0) {
                // dgPolyMesh.C:866-893: index of the owner face's first point in
                // the neighbour face's point list
                int first = O.EToV[3 * k + f];
                int nb0 = O.EToV[3 * n + F.fn], nb1 = O.EToV[3 * n + (F.fn + 1) % 3];
                F.rot = (first == nb0) ? 0 : (first == nb1 ? 1 : -1);
                if (F.rot < 0) { fprintf(stderr, "oracle: face rotation not found\n"); abort(); }
            } else {
                F.rot = -1;
            }
            int id = (int)O.faces.size();
            O.cellFace[k][f] = id;
            if (n >= 0) O.cellFace[n][F.fn] = id;
            O.faces.push_back(F);
        }
    // face normals, WJ, fscale (physicalElementData.C:228-263,
    // gaussTriangleIntegration.C:153-192, triangleBaseFunction.C:393-419)
    auto faceNormalJs = [](int f, double xr, double yr, double xs, double ys, double& nx, double& ny) {
        if (f == 0) { nx = yr; ny = -xr; }
        else if (f == 1) { nx = ys - yr; ny = xr - xs; }
        else { nx = -ys; ny = xs; }
        return std::sqrt(nx * nx + ny * ny);
    };
    for (Face& F : O.faces) {
        int k = F.owner, f = F.fo;
        F.nx.assign(Nfq, 0); F.ny.assign(Nfq, 0); F.wJ.assign(Nfq, 0);
        for (int i = 0; i < Nfq; i++) {
            double t[4] = {0, 0, 0, 0};
            for (int j = 0; j < Nfp; j++) {
                const std::array<double, 4>& d = O.dxdr[(size_t)k * Np + B.fci[f][0][j]];
                for (int c = 0; c < 4; c++) t[c] += B.faceInterp(i, j) * d[c];
            }
            double nx, ny;
            double Js = faceNormalJs(f, t[0], t[1], t[2], t[3], nx, ny);
            F.nx[i] = nx / Js; F.ny[i] = ny / Js;
            F.wJ[i] = Js * B.fw[i];
        }
        {
            const std::array<double, 4>& d = O.dxdr[(size_t)k * Np + B.fci[f][0][0]];
            double nx, ny;
            double Js = faceNormalJs(f, d[0], d[1], d[2], d[3], nx, ny);
            F.fscale = Js / (d[0] * d[3] - d[1] * d[2]);
        }
        if (F.nbr >= 0) {
            const std::array<double, 4>& d = O.dxdr[(size_t)F.nbr * Np + B.fci[F.fn][F.rot][0]];
            double nx, ny;
            double Js = faceNormalJs(F.fn, d[0], d[1], d[2], d[3], nx, ny);
            F.fscale = std::max(F.fscale, Js / (d[0] * d[3] - d[1] * d[2]));
        }
    }
}

// physicalElementData.C:265-343 (face normal-derivative matrices for SIPG)
static void build_face_dn(Oracle& O) {
    TriBase& B = O.B;
    int Np = B.Np, Nfp = B.Nfp, Nfq = B.Nfq;
    for (Face& F : O.faces) {
        for (int side = 0; side < 2; side++) {
            if (side == 1 && F.nbr < 0) break;
            int k = side == 0 ? F.owner : F.nbr;
            int f = side == 0 ? F.fo : F.fn;
            const int* map = B.fci[f][0];  // owner mapping / neighborNoRotateDofMapping
            // drdx at face nodes interpolated to the gauss points
            Mat Dn(Nfq, Np, 0.0);
            for (int i = 0; i < Nfq; i++) {
                double g[4] = {0, 0, 0, 0};  // rx, sx, ry, sy
                for (int j = 0; j < Nfp; j++) {
                    const std::array<double, 4>& d = O.dxdr[(size_t)k * Np + map[j]];
                    double J = d[0] * d[3] - d[1] * d[2];
                    double rx = d[3] / J, sx = -d[1] / J, ry = -d[2] / J, sy = d[0] / J;
                    g[0] += B.faceInterp(i, j) * rx;
                    g[1] += B.faceInterp(i, j) * sx;
                    g[2] += B.faceInterp(i, j) * ry;
                    g[3] += B.faceInterp(i, j) * sy;
                }
                for (int c = 0; c < Np; c++) {
                    double dr = 0, ds = 0;  // faceVand * Dr.subRows(map)
                    for (int j = 0; j < Nfp; j++) {
                        dr += B.faceInterp(i, j) * B.Dr(map[j], c);
                        ds += B.faceInterp(i, j) * B.Ds(map[j], c);
                    }
                    double ddx = dr * g[0] + ds * g[1];
                    double ddy = dr * g[2] + ds * g[3];
                    double v = F.nx[i] * ddx + F.ny[i] * ddy;
                    Dn(i, c) = side == 0 ? v : -v;
                }
            }
            if (side == 0) F.DnO = Dn;
            else {
                F.DnN = Dn;
                F.DnNrot = Mat(Nfq, Np);
                for (int i = 0; i < Nfq; i++) {
                    int ri = F.rot == 1 ? Nfq - 1 - i : i;  // gaussFaceRotateIndex
                    for (int c = 0; c < Np; c++) F.DnNrot(i, c) = Dn(ri, c);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Euler right-hand side

enum { FLUX_LF = 0, FLUX_ROE = 1 };

struct VortexBC {  // setBoundaryValues.H
    double beta, x0, y0, uinf, gamma, t;
};

static void vortex_exact(const VortexBC& bc, double px, double py, double* q4) {
    const double pi = 3.14159265358979323846;
    double g = bc.gamma;
    double dx = px - bc.x0 - bc.uinf * bc.t, dy = py - bc.y0;
    double r = dx * dx + dy * dy;
    double rho = std::pow(1.0 - (g - 1.0) * (bc.beta * bc.beta) * std::exp(2.0 * (1.0 - r)) / (16.0 * g * pi * pi),
                          1.0 / (g - 1.0));
    double u = bc.uinf - bc.beta * std::exp(1 - r) * dy / (2.0 * pi);
    double v = bc.beta * std::exp(1 - r) * dx / (2.0 * pi);
    q4[0] = rho;
    q4[1] = rho * u;
    q4[2] = rho * v;
    double mu = rho * u, mv = rho * v;
    q4[3] = std::pow(rho, g) / (g - 1.0) + 0.5 * (mu * mu + mv * mv) / rho;
}

// Roe flux, RoeFlux.C:109-178 (one gauss point; returns n.F* for 4 vars)
static void roe_point(double gamma, double nx, double ny, const double* qO, const double* qN, double* F) {
    double QP2 = nx * qN[1] + ny * qN[2], QM2 = nx * qO[1] + ny * qO[2];
    double QP3 = nx * qN[2] - ny * qN[1], QM3 = nx * qO[2] - ny * qO[1];
    double rhoP = qN[0], rhoM = qO[0];
    double uM = QM2 / rhoM, uP = QP2 / rhoP, vM = QM3 / rhoM, vP = QP3 / rhoP;
    double pM = (gamma - 1) * (qO[3] - 0.5 * (QM2 * uM + QM3 * vM));
    double pP = (gamma - 1) * (qN[3] - 0.5 * (QP2 * uP + QP3 * vP));
    double HM = (qO[3] + pM) / rhoM, HP = (qN[3] + pP) / rhoP;
    double fr = (QM2 + QP2) / 2;
    double fu = (QM2 * uM + pM + QP2 * uP + pP) / 2;
    double fv = (QM3 * uM + QP3 * uP) / 2;
    double fe = (uM * (qO[3] + pM) + uP * (qN[3] + pP)) / 2;
    double rhoMs = std::sqrt(rhoM), rhoPs = std::sqrt(rhoP);
    double rhob = rhoMs * rhoPs;
    double u = (rhoMs * uM + rhoPs * uP) / (rhoMs + rhoPs);
    double v = (rhoMs * vM + rhoPs * vP) / (rhoMs + rhoPs);
    double H = (rhoMs * HM + rhoPs * HP) / (rhoMs + rhoPs);
    double c2 = (gamma - 1) * (H - 0.5 * (u * u + v * v));
    double c = std::sqrt(std::fabs(c2) + 0.0);
    double dw1 = (-0.5 * rhob * (uP - uM) / c + 0.5 * (pP - pM) / c2) * std::fabs(u - c);
    double dw2 = ((rhoP - rhoM) - (pP - pM) / c2) * std::fabs(u);
    double dw3 = (rhob * (vP - vM)) * std::fabs(u);
    double dw4 = (0.5 * rhob * (uP - uM) / c + 0.5 * (pP - pM) / c2) * std::fabs(u + c);
    fr -= (dw1 + dw2 + dw4) / 2;
    fu -= (dw1 * (u - c) + dw2 * u + dw4 * (u + c)) / 2;
    fv -= (dw1 * v + dw2 * v + dw3 + dw4 * v) / 2;
    fe -= (dw1 * (H - u * c) + dw2 * (u * u + v * v) / 2 + dw3 * v + dw4 * (H + u * c)) / 2;
    F[0] = fr;
    F[1] = nx * fu - ny * fv;
    F[2] = ny * fu + nx * fv;
    F[3] = fe;
}

static void euler_phys_flux(double gamma, const double* q, double* fx, double* fy) {
    double rho = q[0], u = q[1] / rho, v = q[2] / rho;
    double p = (gamma - 1) * (q[3] - 0.5 * rho * (u * u + v * v));
    fx[0] = q[1]; fx[1] = q[1] * u + p; fx[2] = q[2] * u; fx[3] = u * (q[3] + p);
    fy[0] = q[2]; fy[1] = q[1] * v; fy[2] = q[2] * v + p; fy[3] = v * (q[3] + p);
}

// Face flux of one owner face at all gauss points (n.F*), LF or Roe.
static void face_flux(int kind, double gamma, int Nfq, const double* nx, const double* ny, const double* qO,
                      const double* qN, double* F) {
    if (kind == FLUX_ROE) {
        for (int i = 0; i < Nfq; i++) {
            double a[4] = {qO[i], qO[Nfq + i], qO[2 * Nfq + i], qO[3 * Nfq + i]};
            double b[4] = {qN[i], qN[Nfq + i], qN[2 * Nfq + i], qN[3 * Nfq + i]};
            double out[4];
            roe_point(gamma, nx[i], ny[i], a, b, out);
            for (int v = 0; v < 4; v++) F[v * Nfq + i] = out[v];
        }
        return;
    }
    // Euler Lax-Friedrichs (Rusanov): 1/2 (F- + F+).n + 1/2 lam (q- - q+),
    // lam = max over the face's gauss points of |u.n| + c on both sides.
    double lam = 0;
    for (int i = 0; i < Nfq; i++)
        for (int side = 0; side < 2; side++) {
            const double* q = side ? qN : qO;
            double rho = q[i], u = q[Nfq + i] / rho, v = q[2 * Nfq + i] / rho;
            double p = (gamma - 1) * (q[3 * Nfq + i] - 0.5 * rho * (u * u + v * v));
            double c = std::sqrt(std::fabs(gamma * p / rho));
            lam = std::max(lam, std::fabs(u * nx[i] + v * ny[i]) + c);
        }
    for (int i = 0; i < Nfq; i++) {
        double a[4] = {qO[i], qO[Nfq + i], qO[2 * Nfq + i], qO[3 * Nfq + i]};
        double b[4] = {qN[i], qN[Nfq + i], qN[2 * Nfq + i], qN[3 * Nfq + i]};
        double fxa[4], fya[4], fxb[4], fyb[4];
        euler_phys_flux(gamma, a, fxa, fya);
        euler_phys_flux(gamma, b, fxb, fyb);
        for (int v = 0; v < 4; v++)
            F[v * Nfq + i] = 0.5 * ((fxa[v] + fxb[v]) * nx[i] + (fya[v] + fyb[v]) * ny[i]) + 0.5 * lam * (a[v] - b[v]);
    }
}

// Weak right-hand side b (before the mass solve) for all 4 conserved variables.
// q layout: q[v*K*Np + k*Np + i], v = rho, rhou, rhov, E.
// traces (optional): boundary values per boundary slot (boundary faces in
// element, face order) [slot][4][Nfp] at the owner's face nodes
static void euler_weak(const Oracle& O, const double* q, int kind, double gamma, const VortexBC* bc, double* bw,
                       const double* traces = nullptr) {
    const TriBase& B = O.B;
    int K = O.K, Np = B.Np, Ng = B.Ng, Nfp = B.Nfp, Nfq = B.Nfq;
    size_t KN = (size_t)K * Np;
    std::vector<int> slot(3 * K, -1);
    {
        int nb = 0;
        for (int k = 0; k < K; k++)
            for (int f = 0; f < 3; f++)
                if (O.EToE[k][f] < 0) slot[3 * k + f] = nb++;
    }
    // face fluxes on owner faces (dgGaussField::initField + godunovScheme::update)
    vec flux((size_t)4 * O.nFaceGauss);
    int nF = (int)O.faces.size();
#pragma omp parallel for schedule(static)
    for (int fi = 0; fi < nF; fi++) {
        const Face& F = O.faces[fi];
        double qO[4 * 16], qN[4 * 16], ftmp[4 * 16];
        for (int v = 0; v < 4; v++) {
            const double* qv = q + v * KN;
            for (int i = 0; i < Nfq; i++) {
                double so = 0;
                for (int j = 0; j < Nfp; j++) so += B.faceInterp(i, j) * qv[(size_t)F.owner * Np + B.fci[F.fo][0][j]];
                qO[v * Nfq + i] = so;
            }
        }
        if (F.nbr >= 0) {
            for (int v = 0; v < 4; v++) {
                const double* qv = q + v * KN;
                for (int i = 0; i < Nfq; i++) {
                    double sn = 0;
                    for (int j = 0; j < Nfp; j++)
                        sn += B.faceInterp(i, j) * qv[(size_t)F.nbr * Np + B.fci[F.fn][F.rot][j]];
                    qN[v * Nfq + i] = sn;
                }
            }
        } else {
            // boundary: exact-solution traces at the owner's face nodes
            // (setBoundaryValues.H), interpolated to gauss points
            double tr[4][16];
            for (int j = 0; j < Nfp; j++) {
                int node = B.fci[F.fo][0][j];
                double q4[4];
                if (traces) {
                    const double* t = traces + (size_t)slot[3 * F.owner + F.fo] * 4 * Nfp;
                    for (int v = 0; v < 4; v++) q4[v] = t[v * Nfp + j];
                } else if (bc) vortex_exact(*bc, O.x[(size_t)F.owner * Np + node], O.y[(size_t)F.owner * Np + node], q4);
                else for (int v = 0; v < 4; v++) q4[v] = q[v * KN + (size_t)F.owner * Np + node];
                for (int v = 0; v < 4; v++) tr[v][j] = q4[v];
            }
            for (int v = 0; v < 4; v++)
                for (int i = 0; i < Nfq; i++) {
                    double sn = 0;
                    for (int j = 0; j < Nfp; j++) sn += B.faceInterp(i, j) * tr[v][j];
                    qN[v * Nfq + i] = sn;
                }
        }
        face_flux(kind, gamma, Nfq, F.nx.data(), F.ny.data(), qO, qN, ftmp);
        for (int v = 0; v < 4; v++)
            for (int i = 0; i < Nfq; i++) flux[(size_t)v * O.nFaceGauss + F.start + i] = ftmp[v * Nfq + i];
    }
    // element loop (Equation::evaluate -> calculateCell)
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; k++) {
        double qg[4][128], b[4][64];
        for (int v = 0; v < 4; v++) {  // cell gauss field (dgGaussField.C:193-202)
            const double* qv = q + v * KN + (size_t)k * Np;
            for (int g = 0; g < Ng; g++) {
                double sacc = 0;
                for (int j = 0; j < Np; j++) sacc += B.cellV(g, j) * qv[j];
                qg[v][g] = sacc;
            }
            for (int j = 0; j < Np; j++) b[v][j] = 0;
        }
        const double* wJ = &O.wJ[(size_t)k * Ng];
        const double* D1x = &O.D1x[(size_t)k * Ng * Np];
        const double* D1y = &O.D1y[(size_t)k * Ng * Np];
        for (int g = 0; g < Ng; g++) {
            double rho = qg[0][g], U = qg[1][g] / rho, V = qg[2][g] / rho;  // gther_U
            double p = (gamma - 1) * (qg[3][g] - 0.5 * (rho * (U * U + V * V)));  // gther_p
            // dgc::div(U, q, flux) volume + dgc::grad(p) + dgc::div(U, p)
            double tX[4] = {U * rho * wJ[g], U * qg[1][g] * wJ[g], U * qg[2][g] * wJ[g], U * qg[3][g] * wJ[g]};
            double tY[4] = {V * rho * wJ[g], V * qg[1][g] * wJ[g], V * qg[2][g] * wJ[g], V * qg[3][g] * wJ[g]};
            double pw = p * wJ[g];
            for (int j = 0; j < Np; j++) {
                double dx = D1x[(size_t)g * Np + j], dy = D1y[(size_t)g * Np + j];
                b[0][j] += dx * tX[0] + dy * tY[0];
                b[1][j] += dx * tX[1] + dy * tY[1] + dx * pw;
                b[2][j] += dx * tX[2] + dy * tY[2] + dy * pw;
                b[3][j] += dx * tX[3] + dy * tY[3] + (dx * (U * pw) + dy * (V * pw));
            }
        }
        for (int f = 0; f < 3; f++) {  // face lift (defaultConvectionScheme.C:93-128)
            const Face& F = O.faces[O.cellFace[k][f]];
            bool own = (F.owner == k) && (F.fo == f);
            const int* map = own ? B.fci[F.fo][0] : B.fci[F.fn][F.rot];
            double sgn = own ? -1.0 : 1.0;
            for (int v = 0; v < 4; v++)
                for (int i = 0; i < Nfq; i++) {
                    double t = F.wJ[i] * flux[(size_t)v * O.nFaceGauss + F.start + i];
                    for (int j = 0; j < Nfp; j++) b[v][map[j]] += sgn * t * B.faceInterp(i, j);
                }
        }
        for (int v = 0; v < 4; v++)
            for (int j = 0; j < Np; j++) bw[v * KN + (size_t)k * Np + j] = b[v][j];
    }
}

// R(q) = M^{-1} b_weak (per element, exact inverse)
static void euler_rhs(const Oracle& O, const double* q, int kind, double gamma, const VortexBC* bc, double* rhs) {
    int K = O.K, Np = O.B.Np;
    size_t KN = (size_t)K * Np;
    vec bw(4 * KN);
    euler_weak(O, q, kind, gamma, bc, bw.data());
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; k++)
        for (int v = 0; v < 4; v++)
            for (int i = 0; i < Np; i++) {
                double s = 0;
                for (int j = 0; j < Np; j++) s += O.Minv[k](i, j) * bw[v * KN + (size_t)k * Np + j];
                rhs[v * KN + (size_t)k * Np + i] = s;
            }
}

// One dg::solveEquation(dgm::ddt(q) + R) forward-Euler stage, the reference's
// way: b = M (q_old/dt) + b_weak; b *= dt; q_new = M^{-1} b.
static void euler_stage_ref(const Oracle& O, const double* qold, double* qnew, double dt, int kind, double gamma,
                            const VortexBC* bc) {
    int K = O.K, Np = O.B.Np;
    size_t KN = (size_t)K * Np;
    vec bw(4 * KN);
    euler_weak(O, qold, kind, gamma, bc, bw.data());
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; k++)
        for (int v = 0; v < 4; v++) {
            double b[64];
            for (int i = 0; i < Np; i++) {
                double s = bw[v * KN + (size_t)k * Np + i];
                for (int j = 0; j < Np; j++) s += O.M[k](i, j) * (qold[v * KN + (size_t)k * Np + j] / dt);
                b[i] = s * dt;
            }
            for (int i = 0; i < Np; i++) {
                double s = 0;
                for (int j = 0; j < Np; j++) s += O.Minv[k](i, j) * b[j];
                qnew[v * KN + (size_t)k * Np + i] = s;
            }
        }
}

// LSERK4 coefficients (createFields.H:119-138)
static const double rk4a[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                               -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
static const double rk4b[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                               1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                               2277821191437.0 / 14882151754819.0};
static const double rk4c[5] = {0.0, 1432997174477.0 / 9575080441755.0, 2526269341429.0 / 6820363962896.0,
                               2006345519317.0 / 3224310063776.0, 2802321613138.0 / 2924317926251.0};

// ---------------------------------------------------------------------------
// SIPG operator rows (defaultLaplacianScheme.C:63-288), assembled as element
// blocks: diag[k] (Np x Np) and off[k][f] (Np x Np, columns of EToE[k][f]).

struct Ipdg {
    std::vector<Mat> diag;
    std::vector<std::array<Mat, 3>> off;
    vec bdir;   // Dirichlet contribution to b per unit boundary data (computed for given g)
};

// C = A^T diag(x) B (denseMatrix.C:356-384)
static Mat AtDB(const Mat& A, const double* x, const Mat& Bm) {
    Mat C(A.c, Bm.c, 0.0);
    for (int k = 0; k < A.r; k++)
        for (int i = 0; i < A.c; i++)
            for (int j = 0; j < Bm.c; j++) C(i, j) += A(k, i) * Bm(k, j) * x[k];
    return C;
}

// Assembles the reference-sign SIPG operator A (negative semi-definite) and
// the Dirichlet part of b for boundary data gD (values at boundary face
// nodes, indexed [face id][Nfp], ignored where NULL -> 0).
// btype (optional, per element face k*3+f, read on boundary faces):
// 0 fixesValue (Dirichlet, data gD), 1 fixesGradient (data gN: b -= I^T W I gN,
// no matrix terms, defaultLaplacianScheme.C:210-220), 2 neither (zeroGradient:
// nothing).  With kf_data the data arrays are indexed [(k*3+f)*Nfp + i] in the
// element's own face-node order, else [face id * Nfp + i].
static void ipdg_assemble(const Oracle& O, double tau_coef, Ipdg& L, const double* gD, vec& b,
                          const int* btype = nullptr, const double* gN = nullptr, bool kf_data = false) {
    const TriBase& B = O.B;
    int K = O.K, Np = B.Np, Ng = B.Ng, Nfp = B.Nfp, Nfq = B.Nfq, N = B.N;
    L.diag.assign(K, Mat());
    L.off.assign(K, {Mat(), Mat(), Mat()});
    b.assign((size_t)K * Np, 0.0);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; k++) {
        Mat diag(Np, Np, 0.0);
        const double* wJ = &O.wJ[(size_t)k * Ng];
        const double* D1x = &O.D1x[(size_t)k * Ng * Np];
        const double* D1y = &O.D1y[(size_t)k * Ng * Np];
        for (int g = 0; g < Ng; g++)
            for (int i = 0; i < Np; i++)
                for (int j = 0; j < Np; j++)
                    diag(i, j) -= (D1x[g * Np + i] * D1x[g * Np + j] + D1y[g * Np + i] * D1y[g * Np + j]) * wJ[g];
        for (int f = 0; f < 3; f++) {
            const Face& F = O.faces[O.cellFace[k][f]];
            double gtau = F.fscale * tau_coef * std::pow(N + 1, 2);
            bool own = (F.owner == k) && (F.fo == f);
            const double* fwJ = F.wJ.data();
            if (F.nbr < 0) {
                const int bt = btype ? btype[k * 3 + f] : 0;
                const size_t didx = kf_data ? (size_t)(k * 3 + f) * Nfp : (size_t)O.cellFace[k][f] * Nfp;
                const Mat& I1 = B.faceInterp;
                const int* m1 = B.fci[F.fo][0];
                if (bt == 1) {
                    // fixesGradient: data only
                    if (gN) {
                        Mat t = AtDB(I1, fwJ, I1);
                        const double* g = gN + didx;
                        for (int i = 0; i < Nfp; i++) {
                            double s = 0;
                            for (int j = 0; j < Nfp; j++) s += t(j, i) * g[j];
                            b[(size_t)k * Np + m1[i]] -= s;
                        }
                    }
                    continue;
                }
                if (bt == 2) continue;
                // Dirichlet (fixesValue) boundary face
                const Mat& Dn1 = F.DnO;
                Mat t = AtDB(I1, fwJ, I1);
                for (auto& e : t.a) e *= gtau;
                for (int i = 0; i < Nfp; i++)
                    for (int j = 0; j < Nfp; j++) diag(m1[i], m1[j]) -= t(i, j);
                const double* g = gD ? gD + didx : nullptr;
                if (g) {
                    for (int i = 0; i < Nfp; i++) {
                        double s = 0;
                        for (int j = 0; j < Nfp; j++) s += t(j, i) * g[j];
                        b[(size_t)k * Np + m1[i]] -= s;
                    }
                }
                Mat t2 = AtDB(I1, fwJ, Dn1);
                for (int i = 0; i < Nfp; i++)
                    for (int j = 0; j < Np; j++) diag(m1[i], j) += t2(i, j);
                Mat t3 = AtDB(Dn1, fwJ, I1);
                for (int i = 0; i < Np; i++)
                    for (int j = 0; j < Nfp; j++) diag(i, m1[j]) += t3(i, j);
                if (g) {
                    for (int i = 0; i < Np; i++) {
                        double s = 0;
                        for (int j = 0; j < Nfp; j++) s += t3(i, j) * g[j];
                        b[(size_t)k * Np + i] += s;
                    }
                }
                continue;
            }
            const Mat *I1, *I2, *I3, *I4, *Dn1, *Dn2;
            const int *m1, *m2;
            if (own) {
                I1 = &B.faceInterp; I2 = &B.faceInterp; I3 = &B.faceInterp; I4 = &B.faceInterp;
                Dn1 = &F.DnO; Dn2 = &F.DnNrot;
                m1 = B.fci[F.fo][0]; m2 = B.fci[F.fn][F.rot];
            } else {
                const Mat& Irot = F.rot == 1 ? B.faceInterpRot : B.faceInterp;
                I2 = &B.faceInterp; I4 = &Irot; I3 = &B.faceInterp; I1 = &Irot;
                Dn2 = &F.DnO; Dn1 = &F.DnN;
                m2 = B.fci[F.fo][0]; m1 = B.fci[F.fn][F.rot];
            }
            Mat t = AtDB(*I1, fwJ, *I1);
            for (int i = 0; i < Nfp; i++)
                for (int j = 0; j < Nfp; j++) diag(m1[i], m1[j]) -= t(i, j) * (gtau * 0.5);
            Mat t2 = AtDB(*I1, fwJ, *Dn1);
            for (int i = 0; i < Nfp; i++)
                for (int j = 0; j < Np; j++) diag(m1[i], j) += t2(i, j) * 0.5;
            Mat t3 = AtDB(*Dn1, fwJ, *I1);
            for (int i = 0; i < Np; i++)
                for (int j = 0; j < Nfp; j++) diag(i, m1[j]) += t3(i, j) * 0.5;
            Mat off(Np, Np, 0.0);
            Mat u1 = AtDB(*I3, fwJ, *I2);
            for (int i = 0; i < Nfp; i++)
                for (int j = 0; j < Nfp; j++) off(m1[i], m2[j]) += u1(i, j) * (gtau * 0.5);
            Mat u2 = AtDB(*I3, fwJ, *Dn2);
            for (int i = 0; i < Nfp; i++)
                for (int j = 0; j < Np; j++) off(m1[i], j) -= u2(i, j) * 0.5;
            Mat u3 = AtDB(*Dn1, fwJ, *I4);
            for (int i = 0; i < Np; i++)
                for (int j = 0; j < Nfp; j++) off(i, m2[j]) -= u3(i, j) * 0.5;
            L.off[k][f] = off;
        }
        L.diag[k] = diag;
    }
}

// ---------------------------------------------------------------------------
// Operators of the Chorin (velocity-correction) step of
// tutorials/DG/2D/pearsonVortex/dgChorinFoam/dgChorinFoam.C:70-96.
// Vector fields are component-major: u[c * K*Np + k*Np + p], c = 0 (x), 1 (y).

// nodal derivatives of phi_j at node i of element k: d/dx = Dr rx + Ds sx, d/dy = Dr ry + Ds sy
// (defaultGrad.C:44-78 / defaultDivScheme.C:40-75: drdx at the element's nodes)
static void node_metrics(const Oracle& O, int k, int i, double& rx, double& sx, double& ry, double& sy) {
    const std::array<double, 4>& d = O.dxdr[(size_t)k * O.B.Np + i];  // xr, yr, xs, ys
    double J = d[0] * d[3] - d[1] * d[2];
    rx = d[3] / J;
    sx = -d[1] / J;
    ry = -d[2] / J;
    sy = d[0] / J;
}

// out = -(dgc::div(U) source) = strong nodal divergence (defaultDivScheme.C:40-75)
static void ins_div_nodal(const Oracle& O, const double* u, double* out) {
    const TriBase& B = O.B;
    int K = O.K, Np = B.Np;
    size_t KN = (size_t)K * Np;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; k++)
        for (int i = 0; i < Np; i++) {
            double rx, sx, ry, sy;
            node_metrics(O, k, i, rx, sx, ry, sy);
            double s = 0;
            for (int j = 0; j < Np; j++) {
                double dx = B.Dr(i, j) * rx + B.Ds(i, j) * sx, dy = B.Dr(i, j) * ry + B.Ds(i, j) * sy;
                s += dx * u[(size_t)k * Np + j] + dy * u[KN + (size_t)k * Np + j];
            }
            out[(size_t)k * Np + i] = s;
        }
}

// strong nodal gradient (defaultGrad.C:44-78, without its minus sign)
static void ins_grad_nodal(const Oracle& O, const double* p, double* out) {
    const TriBase& B = O.B;
    int K = O.K, Np = B.Np;
    size_t KN = (size_t)K * Np;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; k++)
        for (int i = 0; i < Np; i++) {
            double rx, sx, ry, sy;
            node_metrics(O, k, i, rx, sx, ry, sy);
            double gx = 0, gy = 0;
            for (int j = 0; j < Np; j++) {
                double pj = p[(size_t)k * Np + j];
                gx += (B.Dr(i, j) * rx + B.Ds(i, j) * sx) * pj;
                gy += (B.Dr(i, j) * ry + B.Ds(i, j) * sy) * pj;
            }
            out[(size_t)k * Np + i] = gx;
            out[KN + (size_t)k * Np + i] = gy;
        }
}

// curl(curl U) at nodes: w = dv/dx - du/dy, then (dw/dy, -dw/dx)
// (pEqnCorrect.H:28-46, element-local)
static void ins_curlcurl(const Oracle& O, const double* u, double* out) {
    const TriBase& B = O.B;
    int K = O.K, Np = B.Np;
    size_t KN = (size_t)K * Np;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; k++) {
        double w[64];
        for (int i = 0; i < Np; i++) {
            double rx, sx, ry, sy;
            node_metrics(O, k, i, rx, sx, ry, sy);
            double s = 0;
            for (int j = 0; j < Np; j++) {
                double dx = B.Dr(i, j) * rx + B.Ds(i, j) * sx, dy = B.Dr(i, j) * ry + B.Ds(i, j) * sy;
                s += -dy * u[(size_t)k * Np + j] + dx * u[KN + (size_t)k * Np + j];
            }
            w[i] = s;
        }
        for (int i = 0; i < Np; i++) {
            double rx, sx, ry, sy;
            node_metrics(O, k, i, rx, sx, ry, sy);
            double cx = 0, cy = 0;
            for (int j = 0; j < Np; j++) {
                double dx = B.Dr(i, j) * rx + B.Ds(i, j) * sx, dy = B.Dr(i, j) * ry + B.Ds(i, j) * sy;
                cx += dy * w[j];
                cy -= dx * w[j];
            }
            out[(size_t)k * Np + i] = cx;
            out[KN + (size_t)k * Np + i] = cy;
        }
    }
}

// dgc::div(U, U) with the LF flux on dof fields, solved against the mass
// matrix (dgm::Sp(convecU) == dgc::div(U, U)): returns div(U (x) U).
// Face flux at the face nodes (LFFlux.C:103-211): v = n.U on both sides,
// lambda = max |v| over the face's nodes and sides, F = (vO UO + vN UN)/2 +
// lambda (UO - UN)/2, interpolated to the face gauss points; boundary faces
// take ubnd (per element face, [(k*3+f)*2*Nfp + c*Nfp + i], owner face-node
// order).  Volume: products at the nodes, interpolated to the cubature points
// (defaultConvectionScheme.C:216-263); lift as :265-300.
static void ins_convection(const Oracle& O, const double* u, const double* ubnd, double* out) {
    const TriBase& B = O.B;
    int K = O.K, Np = B.Np, Ng = B.Ng, Nfp = B.Nfp, Nfq = B.Nfq;
    size_t KN = (size_t)K * Np;
    vec flux((size_t)2 * O.nFaceGauss);
    int nF = (int)O.faces.size();
#pragma omp parallel for schedule(static)
    for (int fi = 0; fi < nF; fi++) {
        const Face& F = O.faces[fi];
        double UO[2][16], UN[2][16], vO[16], vN[16], t[2][16];
        for (int i = 0; i < Nfp; i++) {
            size_t no = (size_t)F.owner * Np + B.fci[F.fo][0][i];
            UO[0][i] = u[no];
            UO[1][i] = u[KN + no];
            if (F.nbr >= 0) {
                size_t nn = (size_t)F.nbr * Np + B.fci[F.fn][F.rot][i];
                UN[0][i] = u[nn];
                UN[1][i] = u[KN + nn];
            } else {
                const double* g = ubnd + (size_t)(F.owner * 3 + F.fo) * 2 * Nfp;
                UN[0][i] = g[i];
                UN[1][i] = g[Nfp + i];
            }
        }
        double maxV = 0;
        for (int i = 0; i < Nfp; i++) {
            vO[i] = F.nx[i] * UO[0][i] + F.ny[i] * UO[1][i];
            vN[i] = F.nx[i] * UN[0][i] + F.ny[i] * UN[1][i];
            maxV = std::max(maxV, std::max(std::fabs(vO[i]), std::fabs(vN[i])));
        }
        for (int c = 0; c < 2; c++)
            for (int i = 0; i < Nfp; i++) t[c][i] = (vO[i] * UO[c][i] + vN[i] * UN[c][i]) * 0.5 + maxV * (UO[c][i] - UN[c][i]) * 0.5;
        for (int c = 0; c < 2; c++)
            for (int g = 0; g < Nfq; g++) {
                double s = 0;
                for (int i = 0; i < Nfp; i++) s += B.faceInterp(g, i) * t[c][i];
                flux[(size_t)c * O.nFaceGauss + F.start + g] = s;
            }
    }
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; k++) {
        double b[2][64], tx[64], gt[128];
        for (int c = 0; c < 2; c++)
            for (int j = 0; j < Np; j++) b[c][j] = 0;
        const double* wJ = &O.wJ[(size_t)k * Ng];
        const double* D1[2] = {&O.D1x[(size_t)k * Ng * Np], &O.D1y[(size_t)k * Ng * Np]};
        for (int d = 0; d < 2; d++)        // flux direction (the z direction contributes zero)
            for (int c = 0; c < 2; c++) {  // transported component
                for (int i = 0; i < Np; i++) tx[i] = u[d * KN + (size_t)k * Np + i] * u[c * KN + (size_t)k * Np + i];
                for (int g = 0; g < Ng; g++) {
                    double s = 0;
                    for (int j = 0; j < Np; j++) s += B.cellV(g, j) * tx[j];
                    gt[g] = s * wJ[g];
                }
                for (int g = 0; g < Ng; g++)
                    for (int j = 0; j < Np; j++) b[c][j] += D1[d][(size_t)g * Np + j] * gt[g];
            }
        for (int f = 0; f < 3; f++) {
            const Face& F = O.faces[O.cellFace[k][f]];
            bool own = (F.owner == k) && (F.fo == f);
            const int* map = own ? B.fci[F.fo][0] : B.fci[F.fn][F.rot];
            double sgn = own ? -1.0 : 1.0;
            for (int c = 0; c < 2; c++)
                for (int g = 0; g < Nfq; g++) {
                    double tt = F.wJ[g] * flux[(size_t)c * O.nFaceGauss + F.start + g];
                    for (int j = 0; j < Nfp; j++) b[c][map[j]] += sgn * tt * B.faceInterp(g, j);
                }
        }
        // Sp(convecU) == div: M convecU = -b
        for (int c = 0; c < 2; c++)
            for (int i = 0; i < Np; i++) {
                double s = 0;
                for (int j = 0; j < Np; j++) s -= O.Minv[k](i, j) * b[c][j];
                out[c * KN + (size_t)k * Np + i] = s;
            }
    }
}

// b[k][fci[f][0][i]] += (I^T W I g)[i] on the element faces with mask[k*3+f]
// (the face mass matrix of pCorrectEquation.H:90-110 and of the Neumann data)
static void face_mass_lift(const Oracle& O, const int* mask, const double* g, double* b) {
    const TriBase& B = O.B;
    int K = O.K, Np = B.Np, Nfp = B.Nfp;
    for (int k = 0; k < K; k++)
        for (int f = 0; f < 3; f++) {
            if (!mask[k * 3 + f]) continue;
            const Face& F = O.faces[O.cellFace[k][f]];
            if (!(F.owner == k && F.fo == f)) continue;
            Mat t = AtDB(B.faceInterp, F.wJ.data(), B.faceInterp);
            const double* gg = g + (size_t)(k * 3 + f) * Nfp;
            for (int i = 0; i < Nfp; i++) {
                double s = 0;
                for (int j = 0; j < Nfp; j++) s += t(i, j) * gg[j];
                b[(size_t)k * Np + B.fci[f][0][i]] += s;
            }
        }
}

// ---------------------------------------------------------------------------
// Slope limiter of the reference (DG/DG/godunovFlux/limiteSchemes/scheme/
// Trianglelimite/Trianglelimite.C:61-861), restated for one state.
// q: [4][K][Np] conserved variables (reference node order); bnd: per boundary
// slot (boundary faces in element, face order) the boundary-field values
// [slot][4][Nfp] at the owner's face nodes; kind: per slot 0 fixed value, 1
// reflective, 2 other; gref: per slot the slot whose node-0 value a
// fixed-value ghost cell takes (the reference takes the first value of the
// patch, :182-185).  gamma 1.4 as in the reference (:73).
static void limiter(const Oracle& O, double* q, const double* bnd, const int* kind, const int* gref) {
    const TriBase& B = O.B;
    const int K = O.K, Np = B.Np, Nfp = B.Nfp, N = B.N;
    const size_t KN = (size_t)K * Np;
    const double g = 1.4, tol = 1e-2, eps = 1e-10;
    // slot of each boundary element face
    std::vector<int> slot(3 * K, -1);
    int nb = 0;
    for (int k = 0; k < K; k++)
        for (int f = 0; f < 3; f++)
            if (O.EToE[k][f] < 0) slot[3 * k + f] = nb++;
    const int T = K + nb;  // cells + one ghost per boundary face
    // (1) averages with the column sums of the reference mass matrix / 2 (:103-137)
    // reference mass matrix (V V^T)^-1 = invV^T invV
    vec mpp(Np, 0.0);
    for (int i = 0; i < Np; i++)
        for (int j = 0; j < Np; j++) {
            double m = 0;
            for (int l = 0; l < Np; l++) m += B.invV(l, i) * B.invV(l, j);
            mpp[j] += m / 2;
        }
    vec A0(K, 0.0), avg[4], cx(T, 0.0), cy(T, 0.0);
    for (int v = 0; v < 4; v++) avg[v].assign(T, 0.0);
    for (int k = 0; k < K; k++) {
        const std::array<double, 4>& d = O.dxdr[(size_t)k * Np];
        const double J = d[0] * d[3] - d[1] * d[2];
        for (int i = 0; i < Np; i++) A0[k] += mpp[i] * J * 2 / 3;
        for (int j = 0; j < Np; j++) {
            for (int v = 0; v < 4; v++) avg[v][k] += q[v * KN + (size_t)k * Np + j] * mpp[j];
            cx[k] += O.x[(size_t)k * Np + j] * mpp[j];
            cy[k] += O.y[(size_t)k * Np + j] * mpp[j];
        }
    }
    // (2) ghost cells (:152-259): centre reflected across the face line
    for (int k = 0; k < K; k++)
        for (int f = 0; f < 3; f++) {
            const int sl = slot[3 * k + f];
            if (sl < 0) continue;
            const Face& F = O.faces[O.cellFace[k][f]];
            const int gc = K + sl;
            const double A = F.nx[0], Bn = F.ny[0];
            const int n0 = B.fci[f][0][0];
            const double C = -O.x[(size_t)k * Np + n0] * A - O.y[(size_t)k * Np + n0] * Bn;
            cx[gc] = (Bn * Bn - A * A) * cx[k] - 2 * A * Bn * cy[k] - 2 * A * C;
            cy[gc] = (-Bn * Bn + A * A) * cy[k] - 2 * A * Bn * cx[k] - 2 * Bn * C;
            if (kind[sl] == 1) {
                avg[0][gc] = avg[0][k];
                avg[1][gc] = avg[1][k] - A * (A * avg[1][k] + Bn * avg[2][k]);
                avg[2][gc] = avg[2][k] - Bn * (A * avg[1][k] + Bn * avg[2][k]);
                avg[3][gc] = avg[3][k];
            } else if (kind[sl] == 0) {
                for (int v = 0; v < 4; v++) avg[v][gc] = bnd[((size_t)gref[sl] * 4 + v) * Nfp];
            } else {
                for (int v = 0; v < 4; v++) avg[v][gc] = avg[v][k];
            }
        }
    // primitive averages (:295-306)
    vec U(T), V(T), P(T);
    for (int c = 0; c < T; c++) {
        U[c] = avg[1][c] / avg[0][c];
        V[c] = avg[2][c] / avg[0][c];
        P[c] = (g - 1) * (avg[3][c] - 0.5 * (avg[1][c] * avg[1][c] + avg[2][c] * avg[2][c]) / avg[0][c]);
    }
    // (3)-(5) per face owned by a cell, in cell-loop order (:308-459, :500-575)
    struct FaceV { int o, n; double A2, V[4][2]; };
    std::vector<FaceV> fv;
    vec CellA2(T, 0.0);
    for (int k = 0; k < K; k++)
        for (int f = 0; f < 3; f++) {
            const Face& F = O.faces[O.cellFace[k][f]];
            if (!(F.owner == k && F.fo == f)) continue;
            const int S = B.fci[f][0][0], E = B.fci[f][0][N];
            double qS[4], qE[4];
            int nc;
            if (F.nbr >= 0) {
                const int nS = B.fci[F.fn][F.rot][0], nE = B.fci[F.fn][F.rot][N];
                for (int v = 0; v < 4; v++) {
                    qS[v] = q[v * KN + (size_t)F.nbr * Np + nS];
                    qE[v] = q[v * KN + (size_t)F.nbr * Np + nE];
                }
                nc = F.nbr;
            } else {
                const int sl = slot[3 * k + f];
                for (int v = 0; v < 4; v++) {
                    qS[v] = bnd[((size_t)sl * 4 + v) * Nfp];
                    qE[v] = bnd[((size_t)sl * 4 + v) * Nfp + Nfp - 1];
                }
                nc = K + sl;
            }
            double f0[4], f1[4];
            for (int v = 0; v < 4; v++) {
                f0[v] = q[v * KN + (size_t)k * Np + S] * 0.5 + qS[v] * 0.5;
                f1[v] = q[v * KN + (size_t)k * Np + E] * 0.5 + qE[v] * 0.5;
            }
            const double x1v = O.x[(size_t)k * Np + S], y1v = O.y[(size_t)k * Np + S];
            const double x2v = O.x[(size_t)k * Np + E], y2v = O.y[(size_t)k * Np + E];
            FaceV w;
            w.o = k;
            w.n = nc;
            w.A2 = F.nbr >= 0 ? A0[k] + A0[F.nbr] : A0[k] + A0[k];
            const double x0c = cx[k], y0c = cy[k], x1c = cx[nc], y1c = cy[nc];
            const double Af = ((x1c - x0c) * (y2v - y1v) - (x2v - x1v) * (y1c - y0c)) * 0.5;
            // face primitives
            double p0[4], p1[4];
            p0[0] = f0[0];
            p1[0] = f1[0];
            p0[1] = f0[1] / f0[0];
            p1[1] = f1[1] / f1[0];
            p0[2] = f0[2] / f0[0];
            p1[2] = f1[2] / f1[0];
            p0[3] = (g - 1) * (f0[3] - 0.5 * f0[0] * (p0[1] * p0[1] + p0[2] * p0[2]));
            p1[3] = (g - 1) * (f1[3] - 0.5 * f1[0] * (p1[1] * p1[1] + p1[2] * p1[2]));
            const double* cq[4] = {avg[0].data(), U.data(), V.data(), P.data()};
            const double t1 = x2v - x1v, t2 = x1c - x0c;
            for (int m = 0; m < 4; m++) {
                w.V[m][0] = 0.5 * ((cq[m][nc] - cq[m][k]) * (y2v - y1v) + (p0[m] - p1[m]) * (y1c - y0c)) / Af;
                w.V[m][1] = -0.5 * ((cq[m][nc] - cq[m][k]) * t1 + (p0[m] - p1[m]) * t2) / Af;
            }
            CellA2[k] += w.A2;
            if (nc < K) CellA2[nc] += w.A2;
            fv.push_back(w);
        }
    std::vector<std::array<double, 8>> CV(T);
    for (auto& a : CV) a.fill(0.0);
    for (const FaceV& w : fv) {
        for (int m = 0; m < 4; m++)
            for (int d = 0; d < 2; d++) {
                CV[w.o][2 * m + d] += w.A2 * w.V[m][d] / CellA2[w.o];
                if (w.n < K) CV[w.n][2 * m + d] += w.A2 * w.V[m][d] / CellA2[w.n];
                else CV[w.n][2 * m + d] = w.V[m][d];
            }
    }
    // (6) weighted neighbour gradients and the linear reconstruction (:705-858)
    for (int k = 0; k < K; k++) {
        int c[3];
        for (int f = 0; f < 3; f++) c[f] = O.EToE[k][f] >= 0 ? O.EToE[k][f] : K + slot[3 * k + f];
        double L[4][2];
        for (int m = 0; m < 4; m++) {
            double gg[3];
            for (int i = 0; i < 3; i++) gg[i] = CV[c[i]][2 * m] * CV[c[i]][2 * m] + CV[c[i]][2 * m + 1] * CV[c[i]][2 * m + 1];
            const double fac = gg[0] * gg[0] + gg[1] * gg[1] + gg[2] * gg[2];
            const double w1 = (gg[1] * gg[2] + eps) / (fac + 3 * eps);
            const double w2 = (gg[0] * gg[2] + eps) / (fac + 3 * eps);
            const double w3 = (gg[1] * gg[0] + eps) / (fac + 3 * eps);
            for (int d = 0; d < 2; d++) L[m][d] = w1 * CV[c[0]][2 * m + d] + w2 * CV[c[1]][2 * m + d] + w3 * CV[c[2]][2 * m + d];
        }
        for (int p = 0; p < Np; p++) {
            const double dx = O.x[(size_t)k * Np + p] - cx[k], dy = O.y[(size_t)k * Np + p] - cy[k];
            double du = dx * L[0][0] + dy * L[0][1];
            const double du1 = dx * L[1][0] + dy * L[1][1];
            const double du2 = dx * L[2][0] + dy * L[2][1];
            const double du3 = dx * L[3][0] + dy * L[3][1];
            double Lrho = avg[0][k] + du;
            for (int it = 0; it < 64 && Lrho < tol; it++) {  // (the reference loops until positive)
                du *= 0.5;
                Lrho = avg[0][k] + du;
            }
            const size_t i = (size_t)k * Np + p;
            q[i] = Lrho;
            q[KN + i] = avg[1][k] + avg[0][k] * du1 + du * U[k];
            q[2 * KN + i] = avg[2][k] + avg[0][k] * du2 + du * V[k];
            const double dE = (1 / (g - 1)) * du3 + 0.5 * du * (U[k] * U[k] + V[k] * V[k]) +
                              avg[0][k] * (U[k] * du1 + V[k] * du2);
            q[3 * KN + i] = avg[3][k] + dE;
        }
    }
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C interface for the test harness (ctypes)

using namespace orc;

extern "C" {

void* orc_create(int N, int K, const int* EToV, const double* VXY, const double* cub, int Ng) {
    Oracle* O = new Oracle();
    build_oracle(*O, N, K, EToV, VXY, cub, Ng);
    return O;
}

void orc_destroy(void* h) { delete (Oracle*)h; }

void orc_sizes(void* h, int* out) {
    Oracle* O = (Oracle*)h;
    out[0] = O->B.Np; out[1] = O->B.Ng; out[2] = O->B.Nfp; out[3] = O->B.Nfq;
    out[4] = (int)O->faces.size(); out[5] = O->nFaceGauss;
}

void orc_ref_operators(void* h, double* r, double* s, double* V, double* Dr, double* Ds, double* cellV,
                       double* cellDr, double* cellDs, double* fq, double* fw, double* faceInterp, int* fci) {
    const TriBase& B = ((Oracle*)h)->B;
    int Np = B.Np, Ng = B.Ng, Nfq = B.Nfq, Nfp = B.Nfp;
    if (r) std::copy(B.r.begin(), B.r.end(), r);
    if (s) std::copy(B.s.begin(), B.s.end(), s);
    if (V) std::copy(B.V.a.begin(), B.V.a.end(), V);
    if (Dr) std::copy(B.Dr.a.begin(), B.Dr.a.end(), Dr);
    if (Ds) std::copy(B.Ds.a.begin(), B.Ds.a.end(), Ds);
    if (cellV) std::copy(B.cellV.a.begin(), B.cellV.a.end(), cellV);
    if (cellDr) std::copy(B.cellDr.a.begin(), B.cellDr.a.end(), cellDr);
    if (cellDs) std::copy(B.cellDs.a.begin(), B.cellDs.a.end(), cellDs);
    if (fq) std::copy(B.fq.begin(), B.fq.end(), fq);
    if (fw) std::copy(B.fw.begin(), B.fw.end(), fw);
    if (faceInterp) std::copy(B.faceInterp.a.begin(), B.faceInterp.a.end(), faceInterp);
    if (fci)
        for (int f = 0; f < 3; f++)
            for (int rr = 0; rr < 2; rr++)
                for (int i = 0; i < Nfp; i++) fci[(f * 2 + rr) * Nfp + i] = B.fci[f][rr][i];
    (void)Np; (void)Ng; (void)Nfq;
}

void orc_nodes(void* h, double* x, double* y) {
    Oracle* O = (Oracle*)h;
    std::copy(O->x.begin(), O->x.end(), x);
    std::copy(O->y.begin(), O->y.end(), y);
}

// node locations after a relocation (arc patches move nodes after the
// metrics are built, physicalElementData.C:186-224): only the code that reads
// node locations (the limiter, vortex boundary values) sees them
void orc_set_nodes(void* h, const double* x, const double* y) {
    Oracle* O = (Oracle*)h;
    std::copy(x, x + O->x.size(), O->x.begin());
    std::copy(y, y + O->y.size(), O->y.begin());
}

void orc_connectivity(void* h, int* EToE, int* EToF, int* rot) {
    Oracle* O = (Oracle*)h;
    for (int k = 0; k < O->K; k++)
        for (int f = 0; f < 3; f++) {
            EToE[3 * k + f] = O->EToE[k][f];
            EToF[3 * k + f] = O->EToF[k][f];
            const Face& F = O->faces[O->cellFace[k][f]];
            rot[3 * k + f] = F.nbr < 0 ? -1 : F.rot;
        }
}

void orc_mass(void* h, double* M) {
    Oracle* O = (Oracle*)h;
    int Np = O->B.Np;
    for (int k = 0; k < O->K; k++) std::copy(O->M[k].a.begin(), O->M[k].a.end(), M + (size_t)k * Np * Np);
}

static VortexBC make_bc(const double* bcp) {
    VortexBC bc;
    bc.beta = bcp[0]; bc.x0 = bcp[1]; bc.y0 = bcp[2]; bc.uinf = bcp[3]; bc.gamma = bcp[4]; bc.t = bcp[5];
    return bc;
}

// bcp: NULL (boundary faces copy the interior trace) or {beta, x0, y0, uinf, gamma, t}
void orc_euler_rhs(void* h, const double* q, double* rhs, int flux, double gamma, const double* bcp) {
    VortexBC bc;
    if (bcp) bc = make_bc(bcp);
    euler_rhs(*(Oracle*)h, q, flux, gamma, bcp ? &bc : nullptr, rhs);
}

void orc_euler_weak(void* h, const double* q, double* bw, int flux, double gamma, const double* bcp) {
    VortexBC bc;
    if (bcp) bc = make_bc(bcp);
    euler_weak(*(Oracle*)h, q, flux, gamma, bcp ? &bc : nullptr, bw);
}

// SSP-RK2 steps exactly as dgEulerFoam.C:64-131; bcp's t is advanced per step
// (boundary values set at t^n before stage 1, :73).
void orc_ssprk2(void* h, double* q, double dt, int nsteps, int flux, double gamma, const double* bcp, double t0) {
    Oracle& O = *(Oracle*)h;
    size_t n = (size_t)4 * O.K * O.B.Np;
    vec q1(n), q2(n);
    for (int step = 0; step < nsteps; step++) {
        VortexBC bc;
        if (bcp) { bc = make_bc(bcp); bc.t = t0 + step * dt; }
        euler_stage_ref(O, q, q1.data(), dt, flux, gamma, bcp ? &bc : nullptr);
        euler_stage_ref(O, q1.data(), q2.data(), dt, flux, gamma, bcp ? &bc : nullptr);
        for (size_t i = 0; i < n; i++) q[i] = 0.5 * q[i] + 0.5 * q2[i];
    }
}

// LSERK4 (5 stages): res = a_s res + dt R(q); q += b_s res.  res in/out.
void orc_lserk4(void* h, double* q, double* res, double dt, int nsteps, int flux, double gamma) {
    Oracle& O = *(Oracle*)h;
    size_t n = (size_t)4 * O.K * O.B.Np;
    vec rhs(n);
    for (int step = 0; step < nsteps; step++)
        for (int s = 0; s < 5; s++) {
            euler_rhs(O, q, flux, gamma, nullptr, rhs.data());
#pragma omp parallel for schedule(static)
            for (long long i = 0; i < (long long)n; i++) {
                res[i] = rk4a[s] * res[i] + dt * rhs[i];
                q[i] += rk4b[s] * res[i];
            }
        }
}

void orc_lserk4_coeffs(double* a, double* b, double* c) {
    for (int i = 0; i < 5; i++) { a[i] = rk4a[i]; b[i] = rk4b[i]; c[i] = rk4c[i]; }
}

// Face geometry per element face: nx, ny (first gauss point), fscale; [K*3*3]
void orc_face_geom(void* h, double* out) {
    Oracle* O = (Oracle*)h;
    for (int k = 0; k < O->K; k++)
        for (int f = 0; f < 3; f++) {
            const Face& F = O->faces[O->cellFace[k][f]];
            double sgn = (F.owner == k && F.fo == f) ? 1.0 : -1.0;
            out[9 * k + 3 * f + 0] = sgn * F.nx[0];
            out[9 * k + 3 * f + 1] = sgn * F.ny[0];
            out[9 * k + 3 * f + 2] = F.fscale;
        }
}

// SIPG: assemble the reference-sign operator; returns element blocks.
// diag: K*Np*Np, off: K*3*Np*Np (zero where boundary), b: K*Np (Dirichlet data part)
void orc_ipdg_blocks(void* h, double tau_coef, const double* gD, double* diag, double* off, double* b) {
    Oracle& O = *(Oracle*)h;
    build_face_dn(O);
    Ipdg L;
    vec bb;
    ipdg_assemble(O, tau_coef, L, gD, bb);
    int Np = O.B.Np;
    size_t NN = (size_t)Np * Np;
    for (int k = 0; k < O.K; k++) {
        std::copy(L.diag[k].a.begin(), L.diag[k].a.end(), diag + k * NN);
        for (int f = 0; f < 3; f++) {
            if (L.off[k][f].r) std::copy(L.off[k][f].a.begin(), L.off[k][f].a.end(), off + (k * 3 + f) * NN);
            else std::fill(off + (k * 3 + f) * NN, off + (k * 3 + f + 1) * NN, 0.0);
        }
    }
    if (b) std::copy(bb.begin(), bb.end(), b);
}

// y = A x with the assembled blocks (A = reference sign)
static void blk_apply(const Oracle& O, const double* diag, const double* off, const double* x, double* y) {
    int K = O.K, Np = O.B.Np;
    size_t NN = (size_t)Np * Np;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; k++) {
        for (int i = 0; i < Np; i++) {
            double s = 0;
            for (int j = 0; j < Np; j++) s += diag[k * NN + i * Np + j] * x[(size_t)k * Np + j];
            for (int f = 0; f < 3; f++) {
                int n = O.EToE[k][f];
                if (n < 0) continue;
                const double* A = off + (k * 3 + f) * NN;
                for (int j = 0; j < Np; j++) s += A[i * Np + j] * x[(size_t)n * Np + j];
            }
            y[(size_t)k * Np + i] = s;
        }
    }
}

void orc_blk_apply(void* h, const double* diag, const double* off, const double* x, double* y) {
    blk_apply(*(Oracle*)h, diag, off, x, y);
}

// CG on S = -A (SPD) with block-Jacobi preconditioner (inverse diagonal blocks
// of S).  Solves S x = rhs; x in/out.  Returns iterations, writes final
// relative residual ||r||/||rhs||.
int orc_pcg_bj(void* h, const double* diag, const double* off, const double* rhs, double* x, double rtol, int maxit,
               double* relres) {
    Oracle& O = *(Oracle*)h;
    int K = O.K, Np = O.B.Np;
    size_t n = (size_t)K * Np, NN = (size_t)Np * Np;
    std::vector<Mat> Pinv(K);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; k++) {
        Mat Dk(Np, Np);
        for (size_t i = 0; i < NN; i++) Dk.a[i] = -diag[k * NN + i];
        Pinv[k] = matinv(Dk);
    }
    vec r(n), z(n), p(n), Ap(n);
    auto applyS = [&](const double* xx, double* yy) {
        blk_apply(O, diag, off, xx, yy);
        for (size_t i = 0; i < n; i++) yy[i] = -yy[i];
    };
    auto precond = [&](const double* rr, double* zz) {
#pragma omp parallel for schedule(static)
        for (int k = 0; k < K; k++)
            for (int i = 0; i < Np; i++) {
                double s = 0;
                for (int j = 0; j < Np; j++) s += Pinv[k](i, j) * rr[(size_t)k * Np + j];
                zz[(size_t)k * Np + i] = s;
            }
    };
    applyS(x, Ap.data());
    double bnorm = 0;
    for (size_t i = 0; i < n; i++) { r[i] = rhs[i] - Ap[i]; bnorm += rhs[i] * rhs[i]; }
    bnorm = std::sqrt(bnorm);
    if (bnorm == 0) bnorm = 1;
    precond(r.data(), z.data());
    p = z;
    double rz = 0;
    for (size_t i = 0; i < n; i++) rz += r[i] * z[i];
    int it = 0;
    double rn = 0;
    for (size_t i = 0; i < n; i++) rn += r[i] * r[i];
    rn = std::sqrt(rn);
    while (it < maxit && rn / bnorm > rtol) {
        applyS(p.data(), Ap.data());
        double pAp = 0;
        for (size_t i = 0; i < n; i++) pAp += p[i] * Ap[i];
        double alpha = rz / pAp;
        rn = 0;
        for (size_t i = 0; i < n; i++) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; rn += r[i] * r[i]; }
        rn = std::sqrt(rn);
        precond(r.data(), z.data());
        double rz2 = 0;
        for (size_t i = 0; i < n; i++) rz2 += r[i] * z[i];
        double beta = rz2 / rz;
        rz = rz2;
        for (size_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
        it++;
    }
    *relres = rn / bnorm;
    return it;
}

// SIPG blocks with boundary types and data per element face (see ipdg_assemble)
void orc_ipdg_blocks_bc(void* h, double tau_coef, const int* btype, const double* gD, const double* gN, double* diag,
                        double* off, double* b) {
    Oracle& O = *(Oracle*)h;
    build_face_dn(O);
    Ipdg L;
    vec bb;
    ipdg_assemble(O, tau_coef, L, gD, bb, btype, gN, true);
    int Np = O.B.Np;
    size_t NN = (size_t)Np * Np;
    for (int k = 0; k < O.K; k++) {
        std::copy(L.diag[k].a.begin(), L.diag[k].a.end(), diag + k * NN);
        for (int f = 0; f < 3; f++) {
            if (L.off[k][f].r) std::copy(L.off[k][f].a.begin(), L.off[k][f].a.end(), off + (k * 3 + f) * NN);
            else std::fill(off + (k * 3 + f) * NN, off + (k * 3 + f + 1) * NN, 0.0);
        }
    }
    if (b) std::copy(bb.begin(), bb.end(), b);
}

void orc_ins_div_nodal(void* h, const double* u, double* out) { ins_div_nodal(*(Oracle*)h, u, out); }
void orc_ins_grad_nodal(void* h, const double* p, double* out) { ins_grad_nodal(*(Oracle*)h, p, out); }
void orc_ins_curlcurl(void* h, const double* u, double* out) { ins_curlcurl(*(Oracle*)h, u, out); }
void orc_ins_convection(void* h, const double* u, const double* ubnd, double* out) {
    ins_convection(*(Oracle*)h, u, ubnd, out);
}
void orc_face_mass_lift(void* h, const int* mask, const double* g, double* b) {
    face_mass_lift(*(Oracle*)h, mask, g, b);
}

// R(q) with boundary values per slot
void orc_euler_rhs_traces(void* h, const double* q, double* rhs, int flux, double gamma, const double* traces) {
    Oracle& O = *(Oracle*)h;
    const int K = O.K, Np = O.B.Np;
    const size_t KN = (size_t)K * Np;
    vec bw(4 * KN);
    euler_weak(O, q, flux, gamma, nullptr, bw.data(), traces);
    for (int v = 0; v < 4; v++)
        for (int k = 0; k < K; k++)
            for (int i = 0; i < Np; i++) {
                double sacc = 0;
                for (int j = 0; j < Np; j++) sacc += O.Minv[k](i, j) * bw[v * KN + (size_t)k * Np + j];
                rhs[v * KN + (size_t)k * Np + i] = sacc;
            }
}

void orc_limiter(void* h, double* q, const double* bnd, const int* kind, const int* gref) {
    limiter(*(Oracle*)h, q, bnd, kind, gref);
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
