// limiter.cu -- the reference's slope limiter and its limited SSP-RK2 step
// (DG/DG/godunovFlux/limiteSchemes/scheme/Trianglelimite/Trianglelimite.C:61-861;
// tutorials/DG/2D/doubleMach/dgEulerFoam/dgEulerFoam.C:50-101), FP64.
//
// The limiter replaces every element by a linear function: its cell average
// plus a gradient of the primitive variables (rho, u, v, p).  Per face the
// gradient over the quadrilateral of the two cell centres and the face's end
// points (Green-Gauss, with face values the average of both sides' end-node
// values); per cell the area-weighted mean of its faces' gradients; per cell
// the final gradient a weighted mean of its three neighbours' gradients with
// weights favouring the smallest (w_i ~ g_j g_k, g = |grad|^2).  Boundary faces
// have a ghost cell whose centre is the owner's reflected across the face line
// and whose averages are the owner's with the normal momentum removed
// (reflective), a boundary value (fixed value) or the owner's (otherwise).
//
// GPU structure: five kernels over elements or boundary slots; a face's
// gradient is computed by both of its elements (the formula is antisymmetric
// in the two sides twice, so both get the same bits), so no face list and no
// atomics are needed.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dgcu.h"
#include "dg_ctx.hpp"
#include "euler_flux.cuh"

struct LimState {
    bool ready = false;
    std::vector<void*> allocs;
    std::vector<int> kind_h, gref_h;
    int *kind = nullptr, *gref = nullptr, *sk = nullptr, *sf = nullptr;
    double *xn = nullptr, *yn = nullptr, *mpp = nullptr;  // node coordinates (ring order), mass column sums / 2
    double *cx = nullptr, *cy = nullptr, *avg = nullptr, *prim = nullptr;  // [T], [4][T]
    double *A0 = nullptr, *A2c = nullptr, *CV = nullptr;                 // [K], [K], [8][T]
    double* bq = nullptr;  // boundary field of the state (limited SSP-RK2)
    double* bs = nullptr;  // boundary field of the stage state
    double* bdata = nullptr;
    bool bq_set = false;
    bool dynamic = false;  // some slot is a wall or zero gradient (traces follow the state)
};

namespace dgk {

struct LimArgs {
    int K, N, Np, Nfp, nb, T;
    const double* geo;
    const int* conn;
    const double* xn;
    const double* yn;
    const double* mpp;
    const int* kind;
    const int* gref;
    const int* sk;
    const int* sf;
    double* cx;
    double* cy;
    double* avg;   // [4][T]
    double* prim;  // [4][T]: rho, u, v, p
    double* A0;
    double* A2c;   // CellA2
    double* CV;    // [8][T]
};

constexpr double kLimGamma = 1.4;  // Trianglelimite.C:73

__device__ __forceinline__ void lim_prim(const double* a, double* p) {
    p[0] = a[0];
    p[1] = a[1] / a[0];
    p[2] = a[2] / a[0];
    p[3] = (kLimGamma - 1) * (a[3] - 0.5 * (a[1] * a[1] + a[2] * a[2]) / a[0]);
}

// (1) cell averages, centres, A0 = 2/3 J (Trianglelimite.C:103-137); q: [K][4][Np]
// warp-aligned element groups: 32 / Np whole elements per warp (Np <= 32),
// lane q of an element handles its node q; lb is the lane of node 0
struct LimLanes {
    int k, q, lb;
    bool act;
};
__device__ __forceinline__ LimLanes lim_lanes(int Np, int K) {
    const int lane = threadIdx.x & 31, EW = 32 / Np;
    const int ew = lane / Np;
    LimLanes l;
    l.q = lane - ew * Np;
    l.lb = ew * Np;
    l.k = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * EW + ew;
    l.act = ew < EW && l.k < K;
    return l;
}
__host__ __device__ __forceinline__ unsigned lim_lane_blocks(int K, int Np) {
    const int per_block = 4 * (32 / Np);  // 128 threads
    return (unsigned)((K + per_block - 1) / per_block);
}

__global__ void lim_cells_kernel(LimArgs a, const double* __restrict__ q) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.K) return;
    const double* g = a.geo + 4 * (size_t)k;
    const double J = 1.0 / (g[0] * g[3] - g[1] * g[2]);
    double s = 0, av[4] = {0, 0, 0, 0}, x = 0, y = 0;
    for (int j = 0; j < a.Np; j++) {
        const double w = a.mpp[j];
        s += w * J * 2 / 3;
        for (int v = 0; v < 4; v++) av[v] += q[((size_t)k * 4 + v) * a.Np + j] * w;
        x += a.xn[(size_t)k * a.Np + j] * w;
        y += a.yn[(size_t)k * a.Np + j] * w;
    }
    a.A0[k] = s;
    a.cx[k] = x;
    a.cy[k] = y;
    double p[4];
    lim_prim(av, p);
    for (int v = 0; v < 4; v++) {
        a.avg[(size_t)v * a.T + k] = av[v];
        a.prim[(size_t)v * a.T + k] = p[v];
    }
}

// (2) ghost cells (Trianglelimite.C:152-259)
__global__ void lim_ghost_kernel(LimArgs a, const double* __restrict__ bnd) {
    const int sl = blockIdx.x * blockDim.x + threadIdx.x;
    if (sl >= a.nb) return;
    const int k = a.sk[sl], f = a.sf[sl], gc = a.K + sl;
    const double* g = a.geo + 4 * (size_t)k;
    double A, B, fsc;
    face_normal(f, g[0], g[1], g[2], g[3], A, B, fsc);
    const int n0 = (f * a.N) % (3 * a.N);
    const double C = -a.xn[(size_t)k * a.Np + n0] * A - a.yn[(size_t)k * a.Np + n0] * B;
    const double x0 = a.cx[k], y0 = a.cy[k];
    a.cx[gc] = (B * B - A * A) * x0 - 2 * A * B * y0 - 2 * A * C;
    a.cy[gc] = (-B * B + A * A) * y0 - 2 * A * B * x0 - 2 * B * C;
    double av[4];
    const double* ao = a.avg;
    if (a.kind[sl] == 1) {
        const double m = A * ao[(size_t)1 * a.T + k] + B * ao[(size_t)2 * a.T + k];
        av[0] = ao[k];
        av[1] = ao[(size_t)1 * a.T + k] - A * m;
        av[2] = ao[(size_t)2 * a.T + k] - B * m;
        av[3] = ao[(size_t)3 * a.T + k];
    } else if (a.kind[sl] == 0) {
        for (int v = 0; v < 4; v++) av[v] = bnd[((size_t)a.gref[sl] * 4 + v) * a.Nfp];
    } else {
        for (int v = 0; v < 4; v++) av[v] = ao[(size_t)v * a.T + k];
    }
    double p[4];
    lim_prim(av, p);
    for (int v = 0; v < 4; v++) {
        a.avg[(size_t)v * a.T + gc] = av[v];
        a.prim[(size_t)v * a.T + gc] = p[v];
    }
}

// neighbour cell of element face (k, f): element or ghost
__device__ __forceinline__ int lim_nbr_cell(const LimArgs& a, int k, int f, int& cn) {
    cn = a.conn[(size_t)k * 3 + f];
    return cn >= 0 ? (cn >> 3) : a.K + (-1 - cn);
}

// (3) CellA2: sum over the cell's faces of A0(own) + A0(other side or own)
__global__ void lim_a2_kernel(LimArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.K) return;
    double s = 0;
    for (int f = 0; f < 3; f++) {
        int cn;
        const int n = lim_nbr_cell(a, k, f, cn);
        s += cn >= 0 ? a.A0[k] + a.A0[n] : a.A0[k] + a.A0[k];
    }
    a.A2c[k] = s;
}

// gradient of face (k, f) seen from element k (Trianglelimite.C:308-459, 500-575)
__device__ void lim_face_grad(const LimArgs& a, const double* __restrict__ q, const double* __restrict__ bnd, int k,
                              int f, double V[8], double& A2, int& nc) {
    const int N = a.N, Np = a.Np, NB = 3 * N;
    int cn;
    nc = lim_nbr_cell(a, k, f, cn);
    const int S = (f * N) % NB, E = (f * N + N) % NB;
    double qS[4], qE[4];
    if (cn >= 0) {
        const int nb = cn >> 3, fn = cn & 3, rot = (cn >> 2) & 1;
        // the neighbour's nodes matching k's face nodes 0 and N
        const int nS = (fn * N + (rot ? N : 0)) % NB, nE = (fn * N + (rot ? 0 : N)) % NB;
        for (int v = 0; v < 4; v++) {
            qS[v] = q[((size_t)nb * 4 + v) * Np + nS];
            qE[v] = q[((size_t)nb * 4 + v) * Np + nE];
        }
        A2 = a.A0[k] + a.A0[nb];
    } else {
        const int sl = -1 - cn;
        for (int v = 0; v < 4; v++) {
            qS[v] = bnd[((size_t)sl * 4 + v) * a.Nfp];
            qE[v] = bnd[((size_t)sl * 4 + v) * a.Nfp + a.Nfp - 1];
        }
        A2 = a.A0[k] + a.A0[k];
    }
    double f0[4], f1[4];
    for (int v = 0; v < 4; v++) {
        f0[v] = q[((size_t)k * 4 + v) * Np + S] * 0.5 + qS[v] * 0.5;
        f1[v] = q[((size_t)k * 4 + v) * Np + E] * 0.5 + qE[v] * 0.5;
    }
    double p0[4], p1[4];
    p0[0] = f0[0];
    p1[0] = f1[0];
    p0[1] = f0[1] / f0[0];
    p1[1] = f1[1] / f1[0];
    p0[2] = f0[2] / f0[0];
    p1[2] = f1[2] / f1[0];
    p0[3] = (kLimGamma - 1) * (f0[3] - 0.5 * f0[0] * (p0[1] * p0[1] + p0[2] * p0[2]));
    p1[3] = (kLimGamma - 1) * (f1[3] - 0.5 * f1[0] * (p1[1] * p1[1] + p1[2] * p1[2]));
    const double x1v = a.xn[(size_t)k * Np + S], y1v = a.yn[(size_t)k * Np + S];
    const double x2v = a.xn[(size_t)k * Np + E], y2v = a.yn[(size_t)k * Np + E];
    const double x0c = a.cx[k], y0c = a.cy[k], x1c = a.cx[nc], y1c = a.cy[nc];
    const double Af = ((x1c - x0c) * (y2v - y1v) - (x2v - x1v) * (y1c - y0c)) * 0.5;
    const double t1 = x2v - x1v, t2 = x1c - x0c;
    for (int m = 0; m < 4; m++) {
        const double dq = a.prim[(size_t)m * a.T + nc] - a.prim[(size_t)m * a.T + k];
        V[2 * m] = 0.5 * (dq * (y2v - y1v) + (p0[m] - p1[m]) * (y1c - y0c)) / Af;
        V[2 * m + 1] = -0.5 * (dq * t1 + (p0[m] - p1[m]) * t2) / Af;
    }
}

// (4) cell gradients CV (area-weighted over the cell's faces); ghosts take their face's
__global__ void lim_cv_kernel(LimArgs a, const double* __restrict__ q, const double* __restrict__ bnd) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.K) return;
    double cv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const double A2k = a.A2c[k];
    for (int f = 0; f < 3; f++) {
        double V[8], A2;
        int nc;
        lim_face_grad(a, q, bnd, k, f, V, A2, nc);
        for (int m = 0; m < 8; m++) cv[m] += A2 * V[m] / A2k;
        if (nc >= a.K)
            for (int m = 0; m < 8; m++) a.CV[(size_t)m * a.T + nc] = V[m];
    }
    for (int m = 0; m < 8; m++) a.CV[(size_t)m * a.T + k] = cv[m];
}

// (3) + (4) with a lane per face (lanes 4e .. 4e + 2 of a warp; lane 4e + 3
// idle): CellA2 and the area-weighted face gradients, added by the face-0
// lane in face order (the element-per-thread kernels' bits)
__global__ void lim_cv_lane_kernel(LimArgs a, const double* __restrict__ q, const double* __restrict__ bnd) {
    const int lane = threadIdx.x & 31, f = lane & 3, lb = lane & ~3;
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 2;
    const bool act = k < a.K && f < 3;
    double a2t = 0;
    if (act) {
        int cn;
        const int n = lim_nbr_cell(a, k, f, cn);
        a2t = cn >= 0 ? a.A0[k] + a.A0[n] : a.A0[k] + a.A0[k];
    }
    double A2k = 0;
    for (int g = 0; g < 3; g++) A2k += __shfl_sync(0xffffffffu, a2t, lb + g);
    double tv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (act) {
        double V[8], A2;
        int nc;
        lim_face_grad(a, q, bnd, k, f, V, A2, nc);
        for (int m = 0; m < 8; m++) tv[m] = A2 * V[m] / A2k;
        if (nc >= a.K)
            for (int m = 0; m < 8; m++) a.CV[(size_t)m * a.T + nc] = V[m];
    }
    double cv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int g = 0; g < 3; g++)
#pragma unroll
        for (int m = 0; m < 8; m++) cv[m] += __shfl_sync(0xffffffffu, tv[m], lb + g);
    if (k < a.K && f == 0) {
        a.A2c[k] = A2k;
        for (int m = 0; m < 8; m++) a.CV[(size_t)m * a.T + k] = cv[m];
    }
}

// (5) with the element's nodes on its lanes: lanes q < 4 form the weighted
// gradient of variable q, every lane reconstructs its node
__global__ void lim_reconstruct_lane_kernel(LimArgs a, double* __restrict__ q) {
    const LimLanes l = lim_lanes(a.Np, a.K);
    const int Np = a.Np, k = l.k;
    const double eps = 1e-10, tol = 1e-2;
    double Lm0 = 0, Lm1 = 0;  // this lane's variable m = q (q < 4)
    if (l.act && l.q < 4) {
        const int m = l.q;
        int c[3];
        for (int f = 0; f < 3; f++) {
            int cn;
            c[f] = lim_nbr_cell(a, k, f, cn);
        }
        double gg[3];
        for (int i = 0; i < 3; i++) {
            const double gx = a.CV[(size_t)(2 * m) * a.T + c[i]], gy = a.CV[(size_t)(2 * m + 1) * a.T + c[i]];
            gg[i] = gx * gx + gy * gy;
        }
        const double fac = gg[0] * gg[0] + gg[1] * gg[1] + gg[2] * gg[2];
        const double w1 = (gg[1] * gg[2] + eps) / (fac + 3 * eps);
        const double w2 = (gg[0] * gg[2] + eps) / (fac + 3 * eps);
        const double w3 = (gg[1] * gg[0] + eps) / (fac + 3 * eps);
        Lm0 = w1 * a.CV[(size_t)(2 * m) * a.T + c[0]] + w2 * a.CV[(size_t)(2 * m) * a.T + c[1]] +
              w3 * a.CV[(size_t)(2 * m) * a.T + c[2]];
        Lm1 = w1 * a.CV[(size_t)(2 * m + 1) * a.T + c[0]] + w2 * a.CV[(size_t)(2 * m + 1) * a.T + c[1]] +
              w3 * a.CV[(size_t)(2 * m + 1) * a.T + c[2]];
    }
    double L[4][2];
#pragma unroll
    for (int m = 0; m < 4; m++) {
        L[m][0] = __shfl_sync(0xffffffffu, Lm0, l.lb + m);
        L[m][1] = __shfl_sync(0xffffffffu, Lm1, l.lb + m);
    }
    if (!l.act) return;
    const double ar = a.avg[k], a1 = a.avg[(size_t)1 * a.T + k], a2 = a.avg[(size_t)2 * a.T + k],
                 a3 = a.avg[(size_t)3 * a.T + k];
    const double U = a.prim[(size_t)1 * a.T + k], V = a.prim[(size_t)2 * a.T + k];
    const int p = l.q;
    const double dx = a.xn[(size_t)k * Np + p] - a.cx[k], dy = a.yn[(size_t)k * Np + p] - a.cy[k];
    double du = dx * L[0][0] + dy * L[0][1];
    const double du1 = dx * L[1][0] + dy * L[1][1];
    const double du2 = dx * L[2][0] + dy * L[2][1];
    const double du3 = dx * L[3][0] + dy * L[3][1];
    double Lrho = ar + du;
    for (int it = 0; it < 64 && Lrho < tol; it++) {  // the reference loops until positive
        du *= 0.5;
        Lrho = ar + du;
    }
    double* qk = q + (size_t)k * 4 * Np;
    qk[p] = Lrho;
    qk[Np + p] = a1 + ar * du1 + du * U;
    qk[2 * Np + p] = a2 + ar * du2 + du * V;
    const double dE = (1 / (kLimGamma - 1)) * du3 + 0.5 * du * (U * U + V * V) + ar * (U * du1 + V * du2);
    qk[3 * Np + p] = a3 + dE;
}

// (5) weighted neighbour gradients and the linear reconstruction (Trianglelimite.C:705-858)
__global__ void lim_reconstruct_kernel(LimArgs a, double* __restrict__ q) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.K) return;
    const double eps = 1e-10, tol = 1e-2;
    int c[3];
    for (int f = 0; f < 3; f++) {
        int cn;
        c[f] = lim_nbr_cell(a, k, f, cn);
    }
    double L[4][2];
    for (int m = 0; m < 4; m++) {
        double gg[3];
        for (int i = 0; i < 3; i++) {
            const double gx = a.CV[(size_t)(2 * m) * a.T + c[i]], gy = a.CV[(size_t)(2 * m + 1) * a.T + c[i]];
            gg[i] = gx * gx + gy * gy;
        }
        const double fac = gg[0] * gg[0] + gg[1] * gg[1] + gg[2] * gg[2];
        const double w1 = (gg[1] * gg[2] + eps) / (fac + 3 * eps);
        const double w2 = (gg[0] * gg[2] + eps) / (fac + 3 * eps);
        const double w3 = (gg[1] * gg[0] + eps) / (fac + 3 * eps);
        for (int d = 0; d < 2; d++)
            L[m][d] = w1 * a.CV[(size_t)(2 * m + d) * a.T + c[0]] + w2 * a.CV[(size_t)(2 * m + d) * a.T + c[1]] +
                      w3 * a.CV[(size_t)(2 * m + d) * a.T + c[2]];
    }
    const double ar = a.avg[k], a1 = a.avg[(size_t)1 * a.T + k], a2 = a.avg[(size_t)2 * a.T + k],
                 a3 = a.avg[(size_t)3 * a.T + k];
    const double U = a.prim[(size_t)1 * a.T + k], V = a.prim[(size_t)2 * a.T + k];
    for (int p = 0; p < a.Np; p++) {
        const double dx = a.xn[(size_t)k * a.Np + p] - a.cx[k], dy = a.yn[(size_t)k * a.Np + p] - a.cy[k];
        double du = dx * L[0][0] + dy * L[0][1];
        const double du1 = dx * L[1][0] + dy * L[1][1];
        const double du2 = dx * L[2][0] + dy * L[2][1];
        const double du3 = dx * L[3][0] + dy * L[3][1];
        double Lrho = ar + du;
        for (int it = 0; it < 64 && Lrho < tol; it++) {  // the reference loops until positive
            du *= 0.5;
            Lrho = ar + du;
        }
        double* qk = q + (size_t)k * 4 * a.Np;
        qk[p] = Lrho;
        qk[a.Np + p] = a1 + ar * du1 + du * U;
        qk[2 * a.Np + p] = a2 + ar * du2 + du * V;
        const double dE = (1 / (kLimGamma - 1)) * du3 + 0.5 * du * (U * U + V * V) + ar * (U * du1 + V * du2);
        qk[3 * a.Np + p] = a3 + dE;
    }
}

// boundary field of reflective slots: the mirrored interior trace
// (reflectiveDgPatchField.C:79-111: (I - 2 n n^T) on the vector); of
// zero-gradient slots: the interior trace itself (dgPatchField's
// patchInternalField), both re-evaluated where the reference corrects its
// boundary conditions
__global__ void lim_reflect_kernel(LimArgs a, const double* __restrict__ q, double* __restrict__ bnd) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= a.nb * a.Nfp) return;
    const int sl = idx / a.Nfp, j = idx - sl * a.Nfp;
    const int kd = a.kind[sl];
    if (kd != 1 && kd != 3) return;
    const int k = a.sk[sl], f = a.sf[sl];
    const double* g = a.geo + 4 * (size_t)k;
    double nx, ny, fsc;
    face_normal(f, g[0], g[1], g[2], g[3], nx, ny, fsc);
    const int p = (f * a.N + j) % (3 * a.N);
    const double* qk = q + (size_t)k * 4 * a.Np;
    const double ru = qk[a.Np + p], rv = qk[2 * a.Np + p], m = kd == 1 ? nx * ru + ny * rv : 0.0;
    double* b = bnd + (size_t)sl * 4 * a.Nfp;
    b[j] = qk[p];
    b[a.Nfp + j] = ru - 2 * nx * m;
    b[2 * a.Nfp + j] = rv - 2 * ny * m;
    b[3 * a.Nfp + j] = qk[3 * a.Np + p];
}

// x = a x + b y
__global__ void lim_axpby_kernel(size_t n, double a, double* __restrict__ x, double b, const double* __restrict__ y) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = a * x[i] + b * y[i];
}

// slots of kind 0 take this step's boundary data
__global__ void lim_fixed_kernel(int nb, int Nfp, const int* __restrict__ kind, const double* __restrict__ data,
                                 double* __restrict__ bnd) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nb * 4 * Nfp) return;
    if (kind[idx / (4 * Nfp)] == 0) bnd[idx] = data[idx];
}

}  // namespace dgk

using namespace dgk;

namespace {

int lfail(dg_ctx* c, int code, const std::string& m) {
    c->err = m;
    return code;
}

#define LIM_CUDA(ctx, call)                                                                  \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) return lfail(ctx, DG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
int lim_upload(dg_ctx* c, LimState* s, T** p, const std::vector<T>& h) {
    if (cudaMalloc((void**)p, std::max<size_t>(h.size(), 1) * sizeof(T)) != cudaSuccess) {
        *p = nullptr;
        return lfail(c, DG_ERR_NOMEM, "cudaMalloc failed (limiter)");
    }
    s->allocs.push_back((void*)*p);
    if (!h.empty() && cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        return lfail(c, DG_ERR_CUDA, "upload failed (limiter)");
    return DG_OK;
}

template <typename T>
int lim_alloc(dg_ctx* c, LimState* s, T** p, size_t n) {
    return lim_upload(c, s, p, std::vector<T>(n));
}

LimArgs lim_args(dg_ctx* c) {
    LimState* s = c->lim;
    LimArgs a;
    a.K = c->K;
    a.N = c->N;
    a.Np = c->Np;
    a.Nfp = c->Nfp;
    a.nb = c->nb;
    a.T = c->K + c->nb;
    a.geo = c->d_geo;
    a.conn = c->d_conn;
    a.xn = s->xn;
    a.yn = s->yn;
    a.mpp = s->mpp;
    a.kind = s->kind;
    a.gref = s->gref;
    a.sk = s->sk;
    a.sf = s->sf;
    a.cx = s->cx;
    a.cy = s->cy;
    a.avg = s->avg;
    a.prim = s->prim;
    a.A0 = s->A0;
    a.A2c = s->A2c;
    a.CV = s->CV;
    return a;
}

unsigned nblk(size_t n) { return (unsigned)((n + 127) / 128); }

int run_limiter(dg_ctx* c, double* q, const double* bnd) {
    const LimArgs a = lim_args(c);
    cudaStream_t st = c->stream;
    // element groups on warp lanes (Np in 4..32: N = 2..6); element per thread otherwise
    // (the element-per-thread kernels run in 32-thread blocks: a few thousand
    // elements then cover every SM)
    const bool lanes = a.Np >= 4 && a.Np <= 32;
    lim_cells_kernel<<<(a.K + 31) / 32, 32, 0, st>>>(a, q);
    if (a.nb > 0) lim_ghost_kernel<<<(a.nb + 31) / 32, 32, 0, st>>>(a, bnd);
    if (lanes) {
        lim_cv_lane_kernel<<<nblk((size_t)a.K * 4), 128, 0, st>>>(a, q, bnd);
        lim_reconstruct_lane_kernel<<<lim_lane_blocks(a.K, a.Np), 128, 0, st>>>(a, q);
    } else {
        lim_a2_kernel<<<(a.K + 31) / 32, 32, 0, st>>>(a);
        lim_cv_kernel<<<(a.K + 31) / 32, 32, 0, st>>>(a, q, bnd);
        lim_reconstruct_kernel<<<(a.K + 31) / 32, 32, 0, st>>>(a, q);
    }
    LIM_CUDA(c, cudaGetLastError());
    return DG_OK;
}

int reflect(dg_ctx* c, const double* q, double* bnd) {
    const LimArgs a = lim_args(c);
    if (a.nb == 0) return DG_OK;
    lim_reflect_kernel<<<nblk((size_t)a.nb * a.Nfp), 128, 0, c->stream>>>(a, q, bnd);
    LIM_CUDA(c, cudaGetLastError());
    return DG_OK;
}

}  // namespace

// walls and zero-gradient slots: their boundary traces from the state q
// (the unlimited steppers call this before every stage, as the reference
// corrects its boundary conditions after every equation solve,
// dgMatrixSolve.C:209); no work when no slot is of those kinds
bool has_dynamic_traces(const dg_ctx* c) { return c->lim && c->lim->ready && c->lim->dynamic; }

int refresh_boundary_traces(dg_ctx* c, const double* q) {
    if (!c->lim || !c->lim->ready || !c->lim->dynamic) return DG_OK;
    return reflect(c, q, c->d_btrace);
}

void limiter_teardown(dg_ctx* c) {
    if (!c->lim) return;
    for (void* p : c->lim->allocs) cudaFree(p);
    delete c->lim;
    c->lim = nullptr;
}

// node locations in ring order: those of dg_set_node_locations, else the
// straight element's x = -(r+s)/2 v0 + (r+1)/2 v1 + (s+1)/2 v2
static void node_locations(const dg_ctx* c, std::vector<double>& xn, std::vector<double>& yn) {
    const int K = c->K, Np = c->Np;
    const dgb::RefOps& o = c->ops;
    const size_t KN = (size_t)K * Np;
    xn.resize(KN);
    yn.resize(KN);
    const bool given = c->node_xy_host.size() == 2 * KN;
    for (int k = 0; k < K; k++) {
        const double* v = &c->vxy_host[6 * (size_t)k];
        for (int p = 0; p < Np; p++) {
            const size_t d = (size_t)k * Np + p;
            if (given) {
                xn[d] = c->node_xy_host[(size_t)k * Np + o.ring[p]];
                yn[d] = c->node_xy_host[KN + (size_t)k * Np + o.ring[p]];
            } else {
                const double r = o.r[o.ring[p]], t = o.s[o.ring[p]];
                xn[d] = -(r + t) * 0.5 * v[0] + (r + 1) * 0.5 * v[2] + (t + 1) * 0.5 * v[4];
                yn[d] = -(r + t) * 0.5 * v[1] + (r + 1) * 0.5 * v[3] + (t + 1) * 0.5 * v[5];
            }
        }
    }
}

extern "C" {

int dg_set_node_locations(dg_ctx* c, const double* x, const double* y) {
    if (!c || !x || !y) return DG_ERR_ARG;
    const size_t KN = (size_t)c->K * c->Np;
    c->node_xy_host.assign(x, x + KN);
    c->node_xy_host.insert(c->node_xy_host.end(), y, y + KN);
    if (c->lim && c->lim->ready) {  // the limiter already holds node locations: replace them
        std::vector<double> xn, yn;
        node_locations(c, xn, yn);
        LIM_CUDA(c, cudaMemcpyAsync(c->lim->xn, xn.data(), KN * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        LIM_CUDA(c, cudaMemcpyAsync(c->lim->yn, yn.data(), KN * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        LIM_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return DG_OK;
}

int dg_set_boundary_kinds(dg_ctx* c, const int* kind, const int* gref) {
    if (!c || (c->nb > 0 && !kind)) return DG_ERR_ARG;
    for (int i = 0; i < c->nb; i++) {
        if (kind[i] < 0 || kind[i] > 3) return lfail(c, DG_ERR_ARG, "boundary kind must be 0, 1, 2 or 3");
        if (gref && (gref[i] < 0 || gref[i] >= c->nb)) return lfail(c, DG_ERR_ARG, "gref out of range");
    }
    limiter_teardown(c);
    LimState* s = new LimState();
    c->lim = s;
    const int K = c->K, Np = c->Np, N = c->N, nb = c->nb, T = K + nb;
    s->kind_h.assign(kind, kind + nb);
    for (int i = 0; i < nb; i++) s->dynamic |= kind[i] == 1 || kind[i] == 3;
    s->gref_h.resize(nb);
    for (int i = 0; i < nb; i++) s->gref_h[i] = gref ? gref[i] : i;
    std::vector<int> sk, sf;
    for (int k = 0; k < K; k++)
        for (int f = 0; f < 3; f++)
            if (c->conn_host[(size_t)k * 3 + f] < 0) {
                sk.push_back(k);
                sf.push_back(f);
            }
    const dgb::RefOps& o = c->ops;
    std::vector<double> xn, yn, mpp(Np, 0.0);
    node_locations(c, xn, yn);
    // column sums / 2 of the reference mass matrix (V V^T)^-1 (ring order)
    for (int p = 0; p < Np; p++) {
        double sm = 0;
        for (int i = 0; i < Np; i++) {
            double m = 0;
            for (int l = 0; l < Np; l++) m += o.invV[(size_t)l * Np + i] * o.invV[(size_t)l * Np + o.ring[p]];
            sm += m;
        }
        mpp[p] = sm / 2;
    }
    (void)N;
    int rc = 0;
    rc |= lim_upload(c, s, &s->kind, s->kind_h);
    rc |= lim_upload(c, s, &s->gref, s->gref_h);
    rc |= lim_upload(c, s, &s->sk, sk);
    rc |= lim_upload(c, s, &s->sf, sf);
    rc |= lim_upload(c, s, &s->xn, xn);
    rc |= lim_upload(c, s, &s->yn, yn);
    rc |= lim_upload(c, s, &s->mpp, mpp);
    rc |= lim_alloc(c, s, &s->cx, T);
    rc |= lim_alloc(c, s, &s->cy, T);
    rc |= lim_alloc(c, s, &s->avg, (size_t)4 * T);
    rc |= lim_alloc(c, s, &s->prim, (size_t)4 * T);
    rc |= lim_alloc(c, s, &s->A0, K);
    rc |= lim_alloc(c, s, &s->A2c, K);
    rc |= lim_alloc(c, s, &s->CV, (size_t)8 * T);
    const size_t nbv = (size_t)std::max(nb, 1) * 4 * c->Nfp;
    rc |= lim_alloc(c, s, &s->bq, nbv);
    rc |= lim_alloc(c, s, &s->bs, nbv);
    rc |= lim_alloc(c, s, &s->bdata, nbv);
    if (rc) { limiter_teardown(c); return DG_ERR_NOMEM; }
    s->ready = true;
    return DG_OK;
}

int dg_limit(dg_ctx* c) {
    if (!c || !c->lim || !c->lim->ready) return c ? lfail(c, DG_ERR_ARG, "dg_set_boundary_kinds not called") : DG_ERR_ARG;
    if (c->nb > 0 && !c->btrace_set) return lfail(c, DG_ERR_ARG, "boundary traces not set");
    int rc = run_limiter(c, c->d_q[c->cur], c->d_btrace);
    if (rc) return rc;
    LIM_CUDA(c, cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_reflect_boundary_traces(dg_ctx* c) {
    if (!c || !c->lim || !c->lim->ready) return c ? lfail(c, DG_ERR_ARG, "dg_set_boundary_kinds not called") : DG_ERR_ARG;
    int rc = reflect(c, c->d_q[c->cur], c->d_btrace);
    if (rc) return rc;
    c->btrace_set = true;
    LIM_CUDA(c, cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_limited_ssprk2_step(dg_ctx* c, double dt, const double* bdata_host, int flux, int precision) {
    if (!c || !(dt > 0)) return DG_ERR_ARG;
    if (!c->lim || !c->lim->ready) return lfail(c, DG_ERR_ARG, "dg_set_boundary_kinds not called");
    if (c->nb > 0 && !bdata_host) return DG_ERR_ARG;
    if (flux != DG_FLUX_LF && flux != DG_FLUX_ROE) return lfail(c, DG_ERR_ARG, "unknown flux");
    if (precision != DG_PREC_FP64 && precision != DG_PREC_SPLIT) return lfail(c, DG_ERR_ARG, "unknown precision");
    if (precision == DG_PREC_SPLIT && !c->split.ready) return lfail(c, DG_ERR_UNSUPPORTED, "split path not built for this order");
    LimState* s = c->lim;
    cudaStream_t st = c->stream;
    const int nb = c->nb, Nfp = c->Nfp;
    const size_t nbv = (size_t)nb * 4 * Nfp, nq = (size_t)c->K * 4 * c->Np;
    double* q = c->d_q[c->cur];
    double* q1 = c->d_q[c->cur ^ 1];
    double* q2 = c->d_stage;
    int rc;
    if (nb > 0) {
        LIM_CUDA(c, cudaMemcpyAsync(s->bdata, bdata_host, nbv * sizeof(double), cudaMemcpyHostToDevice, st));
        if (!s->bq_set) {
            // the state's boundary field on entry: this step's data, walls mirrored
            LIM_CUDA(c, cudaMemcpyAsync(s->bq, s->bdata, nbv * sizeof(double), cudaMemcpyDeviceToDevice, st));
            if ((rc = reflect(c, q, s->bq))) return rc;
            s->bq_set = true;
        }
        // rho1 = rho (with its boundary field), then setBoundaryValues on the non-wall slots
        LIM_CUDA(c, cudaMemcpyAsync(s->bs, s->bq, nbv * sizeof(double), cudaMemcpyDeviceToDevice, st));
        lim_fixed_kernel<<<nblk(nbv), 128, 0, st>>>(nb, Nfp, s->kind, s->bdata, s->bs);
        LIM_CUDA(c, cudaGetLastError());
    }
    // stage 1: q1 = q + dt R(q); the walls of q1's field follow q1; limit q1
    if ((rc = euler_stage_mode(c, q, q1, nullptr, MODE_EULER, dt, flux, precision, s->bs))) return rc;
    if ((rc = reflect(c, q1, s->bs))) return rc;
    if ((rc = run_limiter(c, q1, s->bs))) return rc;
    // stage 2: q2 = q1 + dt R(q1) with q1's field (walls from before the limiter)
    if ((rc = euler_stage_mode(c, q1, q2, nullptr, MODE_EULER, dt, flux, precision, s->bs))) return rc;
    if ((rc = reflect(c, q2, s->bs))) return rc;
    // q = q/2 + q2/2 together with the boundary fields, limit, walls follow q
    lim_axpby_kernel<<<nblk(nq), 128, 0, st>>>(nq, 0.5, q, 0.5, q2);
    if (nb > 0) lim_axpby_kernel<<<nblk(nbv), 128, 0, st>>>(nbv, 0.5, s->bq, 0.5, s->bs);
    LIM_CUDA(c, cudaGetLastError());
    if ((rc = run_limiter(c, q, s->bq))) return rc;
    if ((rc = reflect(c, q, s->bq))) return rc;
    // the context's traces: the state's boundary field
    if (nb > 0) LIM_CUDA(c, cudaMemcpyAsync(c->d_btrace, s->bq, nbv * sizeof(double), cudaMemcpyDeviceToDevice, st));
    c->btrace_set = true;
    return check_split_status(c, precision);
}

}  // extern "C"
