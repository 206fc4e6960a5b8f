// ipdg.cu -- matrix-free symmetric interior-penalty (SIPG) Laplacian and the
// preconditioned conjugate-gradient solve of the incompressible pressure
// equation (sm_103a).
//
// Operator (SPD sign, S = -A of the reference): for element k with outward
// normal n on face f, jump [u] = u- - u+, average normal flux
// sigma = (du-/dn + du+/dn) / 2 (both with k's normal) and penalty
// tau = tau_coef (N+1)^2 max(sJ/J of both sides)
// (DG/laplacianSchemes/defaultLaplacianScheme/defaultLaplacianScheme.C:114):
//   (S u)_i = int_K grad phi_i . grad u
//           + sum_f int_f [ (tau/2 [u] - sigma) phi_i - 1/2 [u] dphi_i/dn ]
// which is the element row of laplacianFunc (:96-102 volume, :222-286
// interior faces with their 1/2 weights).  Dirichlet faces (:157-209, full
// weights) are the same formula with u+ = -u-, du+/dn = du-/dn.  Boundary
// data enter the right-hand side, not the operator.
//
// On affine triangles the volume term is J (c_rr Srr + c_rs Srs2 + c_ss Sss) u
// with reference matrices Srr = Dr_g^T W Dr_g etc. and the constant metric
// products c_rr = rx^2 + ry^2, c_rs = rx sx + ry sy, c_ss = sx^2 + sy^2.
// Face terms run one thread per (element, face, Gauss point); the element
// row contraction one thread per (element, node).
//
// Arithmetic: the apply is templated on the type it computes in (double: the
// parity path and the outer residual of the solver; float: the inner
// iterations of the mixed-precision solve).  Vectors, dot products and the
// CG recurrences are FP64 (dot products reduced deterministically: per-block
// partial sums, then a fixed-order reduction).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/dgcu.h"
#include "dg_ctx.hpp"
#include "euler_flux.cuh"
#include "ipdg.hpp"

namespace dgk {

template <int N>
struct IpDims {
    static constexpr int Np = Dims<N>::Np, Nfp = Dims<N>::Nfp, Nfq = Dims<N>::Nfq;
    static constexpr int E = (N <= 3) ? 16 : 8;  // elements per CTA
    static constexpr int THREADS = 128;
};

// per-(element, face, Gauss point) coefficients of the face terms
//   c1 = wJ (tau/2 [u] - sigma)   (multiplies phi_i)
//   c2 = -wJ [u] / 2              (multiplies dphi_i/dn)
// Grid-stride over tiles of E elements so that the optional dot-product
// partial (u . y per CTA, into part[blockIdx.x]) has one entry per CTA.
template <int N, typename T>
__global__ void __launch_bounds__(128) ipdg_apply_kernel(IpdgArgs a, const double* __restrict__ u,
                                                         double* __restrict__ y, double* __restrict__ part,
                                                         const int* __restrict__ done) {
    using D = IpDims<N>;
    constexpr int Np = D::Np, Nfp = D::Nfp, Nfq = D::Nfq, E = D::E, NB = 3 * N;
    __shared__ T us[E][Np];
    __shared__ T c1[E][3][Nfq];
    __shared__ T c2[E][3][Nfq];
    __shared__ T ar[E][3], as_[E][3];
    __shared__ double red[D::THREADS / 32];
    if (done && *done) return;
    const int ntiles = (a.K + E - 1) / E;
    double dot = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int k0 = tile * E;
        const int ne = min(E, a.K - k0);
        for (int i = threadIdx.x; i < ne * Np; i += blockDim.x) us[i / Np][i % Np] = (T)u[(size_t)k0 * Np + i];
        __syncthreads();
        // face terms
        for (int it = threadIdx.x; it < ne * 3 * Nfq; it += blockDim.x) {
            const int e = it / (3 * Nfq), rem = it - e * 3 * Nfq, f = rem / Nfq, g = rem - f * Nfq;
            const int k = k0 + e;
            const double* gk = a.geo + (size_t)k * 4;
            double nxd, nyd, fscd;
            face_normal(f, gk[0], gk[1], gk[2], gk[3], nxd, nyd, fscd);
            const T nx = (T)nxd, ny = (T)nyd;
            const T arr = nx * (T)gk[0] + ny * (T)gk[2];  // n . grad r
            const T ass = nx * (T)gk[1] + ny * (T)gk[3];  // n . grad s
            if (g == 0) { ar[e][f] = arr; as_[e][f] = ass; }
            T um = 0, dm = 0;
#pragma unroll
            for (int j = 0; j < Nfp; j++) um += (T)a.If[g * Nfp + j] * us[e][(f * N + j) % NB];
            const double* drf = a.Drf + (size_t)(f * Nfq + g) * Np;
            const double* dsf = a.Dsf + (size_t)(f * Nfq + g) * Np;
#pragma unroll
            for (int p = 0; p < Np; p++) dm += (arr * (T)drf[p] + ass * (T)dsf[p]) * us[e][p];
            T up, dp;
            double tau;
            const int c = a.conn[(size_t)k * 3 + f];
            if (c >= 0) {
                const int nb = c >> 3, fn = c & 3, rot = (c >> 2) & 1;
                const double* gn = a.geo + (size_t)nb * 4;
                double nx2, ny2, fsc2;
                face_normal(fn, gn[0], gn[1], gn[2], gn[3], nx2, ny2, fsc2);
                tau = a.tau_coef * (N + 1) * (N + 1) * fmax(fscd, fsc2);
                const double* un = u + (size_t)nb * Np;
                up = 0;
#pragma unroll
                for (int j = 0; j < Nfp; j++) {
                    const int jj = rot ? (N - j) : j;
                    up += (T)a.If[g * Nfp + j] * (T)un[(fn * N + jj) % NB];
                }
                const int g2 = rot ? (Nfq - 1 - g) : g;
                const T ar2 = nx * (T)gn[0] + ny * (T)gn[2], as2 = nx * (T)gn[1] + ny * (T)gn[3];
                const double* drn = a.Drf + (size_t)(fn * Nfq + g2) * Np;
                const double* dsn = a.Dsf + (size_t)(fn * Nfq + g2) * Np;
                dp = 0;
#pragma unroll
                for (int p = 0; p < Np; p++) dp += (ar2 * (T)drn[p] + as2 * (T)dsn[p]) * (T)un[p];
            } else {
                tau = a.tau_coef * (N + 1) * (N + 1) * fscd;
                up = -um;
                dp = dm;
            }
            const T wJ = (T)(fscd * a.J[k] * a.fw[g]);
            const T jump = um - up;
            const T sigma = (T)0.5 * (dm + dp);
            c1[e][f][g] = wJ * ((T)(0.5 * tau) * jump - sigma);
            c2[e][f][g] = -(T)0.5 * wJ * jump;
        }
        __syncthreads();
        // element rows
        for (int it = threadIdx.x; it < ne * Np; it += blockDim.x) {
            const int e = it / Np, i = it - e * Np;
            const int k = k0 + e;
            const double* gk = a.geo + (size_t)k * 4;
            const T rx = (T)gk[0], sx = (T)gk[1], ry = (T)gk[2], sy = (T)gk[3];
            const T crr = rx * rx + ry * ry, crs = rx * sx + ry * sy, css = sx * sx + sy * sy;
            const double* srr = a.Srr + (size_t)i * Np;
            const double* srs = a.Srs2 + (size_t)i * Np;
            const double* sss = a.Sss + (size_t)i * Np;
            T v = 0;
#pragma unroll
            for (int p = 0; p < Np; p++) v += (crr * (T)srr[p] + crs * (T)srs[p] + css * (T)sss[p]) * us[e][p];
            v *= (T)a.J[k];
#pragma unroll
            for (int f = 0; f < 3; f++) {
                int jf = -1;  // phi_i on face f: ring positions f*N .. f*N+N (mod 3N)
                if (i < NB) {
                    const int d = (i - f * N + NB) % NB;
                    if (d <= N) jf = d;
                }
#pragma unroll
                for (int g = 0; g < Nfq; g++) {
                    const T dn = ar[e][f] * (T)a.Drf[(size_t)(f * Nfq + g) * Np + i] +
                                 as_[e][f] * (T)a.Dsf[(size_t)(f * Nfq + g) * Np + i];
                    T t = c2[e][f][g] * dn;
                    if (jf >= 0) t += c1[e][f][g] * (T)a.If[g * Nfp + jf];
                    v += t;
                }
            }
            const double out = (double)v;
            y[(size_t)k * Np + i] = out;
            dot += out * u[(size_t)k * Np + i];
        }
        __syncthreads();
    }
    if (part) {
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dot;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0;
            for (int w = 0; w < D::THREADS / 32; w++) s += red[w];
            part[blockIdx.x] = s;
        }
    }
}

// diagonal blocks S_kk (column j = S_kk e_j with neighbours zero), FP64
template <int N>
__global__ void ipdg_diag_kernel(IpdgArgs a, double* __restrict__ blocks) {
    using D = IpDims<N>;
    constexpr int Np = D::Np, Nfp = D::Nfp, Nfq = D::Nfq, NB = 3 * N;
    const int k = blockIdx.x;
    const int j = threadIdx.x;  // column
    if (k >= a.K || j >= Np) return;
    const double* gk = a.geo + (size_t)k * 4;
    const double rx = gk[0], sx = gk[1], ry = gk[2], sy = gk[3];
    const double crr = rx * rx + ry * ry, crs = rx * sx + ry * sy, css = sx * sx + sy * sy;
    double col[Np];
    for (int i = 0; i < Np; i++)
        col[i] = a.J[k] * (crr * a.Srr[i * Np + j] + crs * a.Srs2[i * Np + j] + css * a.Sss[i * Np + j]);
    for (int f = 0; f < 3; f++) {
        double nx, ny, fsc;
        face_normal(f, rx, sx, ry, sy, nx, ny, fsc);
        const double arr = nx * rx + ny * ry, ass = nx * sx + ny * sy;
        const int c = a.conn[(size_t)k * 3 + f];
        double tau;
        if (c >= 0) {
            const int nb = c >> 3, fn = c & 3;
            const double* gn = a.geo + (size_t)nb * 4;
            double nx2, ny2, fsc2;
            face_normal(fn, gn[0], gn[1], gn[2], gn[3], nx2, ny2, fsc2);
            tau = a.tau_coef * (N + 1) * (N + 1) * fmax(fsc, fsc2);
        } else {
            tau = a.tau_coef * (N + 1) * (N + 1) * fsc;
        }
        // u = e_j: own trace / normal derivative at each Gauss point
        int jf = -1;
        if (j < NB) {
            const int d = (j - f * N + NB) % NB;
            if (d <= N) jf = d;
        }
        for (int g = 0; g < Nfq; g++) {
            const double um = jf >= 0 ? a.If[g * Nfp + jf] : 0.0;
            const double dm = arr * a.Drf[(size_t)(f * Nfq + g) * Np + j] + ass * a.Dsf[(size_t)(f * Nfq + g) * Np + j];
            const double up = (c >= 0) ? 0.0 : -um;
            const double dp = (c >= 0) ? 0.0 : dm;
            const double wJ = fsc * a.J[k] * a.fw[g];
            const double jump = um - up, sigma = 0.5 * (dm + dp);
            const double cc1 = wJ * (0.5 * tau * jump - sigma), cc2 = -0.5 * wJ * jump;
            for (int i = 0; i < Np; i++) {
                double t = cc2 * (arr * a.Drf[(size_t)(f * Nfq + g) * Np + i] + ass * a.Dsf[(size_t)(f * Nfq + g) * Np + i]);
                if (i < NB) {
                    const int d = (i - f * N + NB) % NB;
                    if (d <= N) t += cc1 * a.If[g * Nfp + d];
                }
                col[i] += t;
            }
        }
    }
    for (int i = 0; i < Np; i++) blocks[(size_t)k * Np * Np + (size_t)i * Np + j] = col[i];
}

// in-place inverse of each Np x Np block (Gauss-Jordan, partial pivoting); FP64
// result plus an FP32 copy
__global__ void invert_blocks_kernel(double* __restrict__ blocks, float* __restrict__ blocks32, int K, int Np,
                                     int* __restrict__ status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    double* A = blocks + (size_t)k * Np * Np;
    double M[36 * 36];
    double X[36 * 36];
    for (int i = 0; i < Np * Np; i++) { M[i] = A[i]; X[i] = 0.0; }
    for (int i = 0; i < Np; i++) X[i * Np + i] = 1.0;
    for (int c = 0; c < Np; c++) {
        int p = c;
        for (int i = c + 1; i < Np; i++)
            if (fabs(M[i * Np + c]) > fabs(M[p * Np + c])) p = i;
        if (M[p * Np + c] == 0.0) { atomicExch(status, 1); return; }
        if (p != c)
            for (int j = 0; j < Np; j++) {
                double t = M[p * Np + j]; M[p * Np + j] = M[c * Np + j]; M[c * Np + j] = t;
                t = X[p * Np + j]; X[p * Np + j] = X[c * Np + j]; X[c * Np + j] = t;
            }
        const double inv = 1.0 / M[c * Np + c];
        for (int j = 0; j < Np; j++) { M[c * Np + j] *= inv; X[c * Np + j] *= inv; }
        for (int i = 0; i < Np; i++) {
            if (i == c) continue;
            const double f = M[i * Np + c];
            if (f == 0.0) continue;
            for (int j = 0; j < Np; j++) { M[i * Np + j] -= f * M[c * Np + j]; X[i * Np + j] -= f * X[c * Np + j]; }
        }
    }
    for (int i = 0; i < Np * Np; i++) { A[i] = X[i]; blocks32[(size_t)k * Np * Np + i] = (float)X[i]; }
}

// ---------------------------------------------------------------------------
// PCG.  Scalars live on the device; every kernel returns immediately once the
// solve has stopped (S->done), so launches can be issued ahead of the host's
// convergence check.  Dot products: per-CTA partials over a fixed grid G, then
// a fixed-order warp reduction by each consumer (deterministic).  The partial
// r.z is double-buffered by iteration parity so consumers of the old and the
// new value never race.

__device__ __forceinline__ double warp_sum(const double* __restrict__ part, int n) {
    double s = 0;
    for (int i = threadIdx.x & 31; i < n; i += 32) s += part[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

__device__ __forceinline__ void block_sum2(double a, double b, double* oa, double* ob) {
    __shared__ double ra[32], rb[32];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) { ra[threadIdx.x >> 5] = a; rb[threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sa = 0, sb = 0;
        for (int w = 0; w < (int)((blockDim.x + 31) >> 5); w++) { sa += ra[w]; sb += rb[w]; }
        if (oa) *oa = sa;
        if (ob) *ob = sb;
    }
    __syncthreads();  // ra/rb are reused by the next call
}

// element-aligned thread mapping: CTA = EB elements x Np rows (EB*Np <= blockDim)
__device__ __forceinline__ double bj_apply_row(const float* __restrict__ P, const double* __restrict__ r, int Np,
                                               int k, int i) {
    const float* row = P + ((size_t)k * Np + i) * Np;
    const double* rk = r + (size_t)k * Np;
    float s = 0.f;
    for (int j = 0; j < Np; j++) s = fmaf(row[j], (float)rk[j], s);
    return (double)s;
}

__device__ __forceinline__ double bj_apply_row64(const double* __restrict__ P, const double* __restrict__ r, int Np,
                                                 int k, int i) {
    const double* row = P + ((size_t)k * Np + i) * Np;
    const double* rk = r + (size_t)k * Np;
    double s = 0.0;
    for (int j = 0; j < Np; j++) s += row[j] * rk[j];
    return s;
}

__device__ __forceinline__ double bj_apply(const PcgVecs& v, int Np, int k, int i) {
    return v.P64 ? bj_apply_row64(v.P64, v.r, Np, k, i) : bj_apply_row(v.P32, v.r, Np, k, i);
}

// z = P r, p = z, part_rz[1] = r.z, part_rr = r.r   (x, r given)
__global__ void pcg_init_kernel(PcgVecs v, int K, int Np) {
    const int EB = blockDim.x / Np;
    const int e = threadIdx.x / Np, i = threadIdx.x - e * Np;
    double rz = 0, rr = 0;
    const int ngroups = (K + EB - 1) / EB;
    for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const int k = grp * EB + e;
        if (e < EB && k < K) {
            const size_t idx = (size_t)k * Np + i;
            const double z = bj_apply(v, Np, k, i);
            v.z[idx] = z;
            v.p[idx] = z;
            rz += v.r[idx] * z;
            rr += v.r[idx] * v.r[idx];
        }
    }
    block_sum2(rz, rr, v.part_rz + v.G + blockIdx.x, v.part_rr + blockIdx.x);
}

// alpha = rz / pAp; x += alpha p; r -= alpha Ap; z = P r; partials of r.z,
// r.r and r.z_old (flexible / Polak-Ribiere beta)
__global__ void pcg_update_kernel(PcgVecs v, int K, int Np, int parity) {
    if (v.S->done) return;
    __shared__ double s_alpha;
    if (threadIdx.x < 32) {
        const double rz = warp_sum(v.part_rz + (parity ^ 1) * v.G, v.G);
        const double pap = warp_sum(v.part_pap, v.G);
        if (threadIdx.x == 0) s_alpha = rz / pap;
    }
    __syncthreads();
    const double alpha = s_alpha;
    const int EB = blockDim.x / Np;
    const int e = threadIdx.x / Np, i = threadIdx.x - e * Np;
    double rz = 0, rr = 0, rzo = 0;
    const int ngroups = (K + EB - 1) / EB;
    for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const int k = grp * EB + e;
        const bool act = e < EB && k < K;
        const size_t idx = (size_t)k * Np + i;
        if (act) {
            v.x[idx] += alpha * v.p[idx];
            v.r[idx] -= alpha * v.Ap[idx];
        }
        __syncthreads();  // the element's r rows are written by this CTA
        if (act) {
            const double zo = v.z[idx];
            const double z = bj_apply(v, Np, k, i);
            v.z[idx] = z;
            const double ri = v.r[idx];
            rz += ri * z;
            rr += ri * ri;
            rzo += ri * zo;
        }
        __syncthreads();
    }
    block_sum2(rz, rr, v.part_rz + parity * v.G + blockIdx.x, v.part_rr + blockIdx.x);
    block_sum2(rzo, 0.0, v.part_rzo + blockIdx.x, nullptr);
}

// beta = rz_new / rz_old; p = z + beta p; convergence test on r.r
__global__ void pcg_pupdate_kernel(PcgVecs v, size_t n, int parity) {
    if (v.S->done) return;
    __shared__ double s_beta;
    __shared__ int s_stop;
    if (threadIdx.x < 32) {
        const double rz_new = warp_sum(v.part_rz + parity * v.G, v.G);
        const double rz_old = warp_sum(v.part_rz + (parity ^ 1) * v.G, v.G);
        const double rzo = warp_sum(v.part_rzo, v.G);
        const double rr = warp_sum(v.part_rr, v.G);
        if (threadIdx.x == 0) {
            s_beta = (rz_new - rzo) / rz_old;
            int stop = 0;
            if (!(rr == rr) || !(rz_new == rz_new) || rz_old == 0.0) stop = 2;
            else if (rr <= v.S->tol2) stop = 1;
            s_stop = stop;
            if (blockIdx.x == 0) {
                v.S->it += 1;
                if (stop) v.S->done = stop;
            }
        }
    }
    __syncthreads();
    if (s_stop) return;
    const double beta = s_beta;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        v.p[t] = v.z[t] + beta * v.p[t];
}

__global__ void dot_kernel(const double* __restrict__ x, const double* __restrict__ y, size_t n, double* part) {
    double s = 0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        s += x[t] * y[t];
    block_sum2(s, 0.0, part + blockIdx.x, nullptr);
}

__global__ void reduce_to_kernel(const double* __restrict__ part, int G, double* out) {
    if (threadIdx.x < 32) {
        const double s = warp_sum(part, G);
        if (threadIdx.x == 0) *out = s;
    }
}

__global__ void axpy_kernel(double* y, const double* x, double alpha, size_t n) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        y[t] += alpha * x[t];
}

__global__ void xmy_kernel(double* out, const double* b, const double* y, size_t n) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        out[t] = b[t] - y[t];
}

// reference node order <-> ring order for scalar fields (K x Np)
__global__ void permute_kernel(const double* __restrict__ in, double* __restrict__ out, const int* __restrict__ ring,
                               int K, int Np, int to_ring) {
    const size_t n = (size_t)K * Np;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / Np), p = (int)(t - (size_t)k * Np);
        if (to_ring) out[t] = in[(size_t)k * Np + ring[p]];
        else out[(size_t)k * Np + ring[p]] = in[t];
    }
}

// ---------------------------------------------------------------------------
// launchers

template <int N>
static cudaError_t apply_n(const IpdgArgs& a, bool fp32, const double* u, double* y, double* part, int G,
                           const int* done, cudaStream_t s) {
    using D = IpDims<N>;
    const int ntiles = (a.K + D::E - 1) / D::E;
    const int grid = part ? G : (ntiles < 65535 * 8 ? ntiles : 65535 * 8);
    if (fp32) ipdg_apply_kernel<N, float><<<grid, D::THREADS, 0, s>>>(a, u, y, part, done);
    else ipdg_apply_kernel<N, double><<<grid, D::THREADS, 0, s>>>(a, u, y, part, done);
    return cudaGetLastError();
}

static cudaError_t apply_dispatch(const IpdgArgs& a, bool fp32, const double* u, double* y, double* part, int G,
                                  const int* done, cudaStream_t s) {
    switch (a.N) {
        case 1: return apply_n<1>(a, fp32, u, y, part, G, done, s);
        case 2: return apply_n<2>(a, fp32, u, y, part, G, done, s);
        case 3: return apply_n<3>(a, fp32, u, y, part, G, done, s);
        case 4: return apply_n<4>(a, fp32, u, y, part, G, done, s);
        case 5: return apply_n<5>(a, fp32, u, y, part, G, done, s);
        case 6: return apply_n<6>(a, fp32, u, y, part, G, done, s);
        case 7: return apply_n<7>(a, fp32, u, y, part, G, done, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_ipdg_apply(const IpdgArgs& a, bool fp32, const double* u, double* y, double* part, int G,
                              cudaStream_t s) {
    return apply_dispatch(a, fp32, u, y, part, G, nullptr, s);
}

cudaError_t launch_ipdg_diag(const IpdgArgs& a, double* blocks, cudaStream_t s) {
    switch (a.N) {
#define DIAG_CASE(n) \
    case n: ipdg_diag_kernel<n><<<a.K, 64, 0, s>>>(a, blocks); break;
        DIAG_CASE(1) DIAG_CASE(2) DIAG_CASE(3) DIAG_CASE(4) DIAG_CASE(5) DIAG_CASE(6) DIAG_CASE(7)
#undef DIAG_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_invert_blocks(double* blocks, float* blocks32, int K, int Np, int* status, cudaStream_t s) {
    invert_blocks_kernel<<<(K + 63) / 64, 64, 0, s>>>(blocks, blocks32, K, Np, status);
    return cudaGetLastError();
}

// element-aligned CTA size: whole elements of Np rows, rounded up to full
// warps (the extra lanes idle but take part in the warp reductions)
static int rows_block(int Np) {
    int eb = 256 / Np;
    if (eb < 1) eb = 1;
    return (eb * Np + 31) / 32 * 32;
}

cudaError_t launch_pcg_init(const IpdgArgs& a, const PcgVecs& v, cudaStream_t s) {
    pcg_init_kernel<<<v.G, rows_block(a.Np), 0, s>>>(v, a.K, a.Np);
    return cudaGetLastError();
}

cudaError_t launch_pcg_iteration(const IpdgArgs& a, const PcgVecs& v, bool fp32, int parity, cudaStream_t s) {
    cudaError_t e = apply_dispatch(a, fp32, v.p, v.Ap, v.part_pap, v.G, &v.S->done, s);
    if (e != cudaSuccess) return e;
    pcg_update_kernel<<<v.G, rows_block(a.Np), 0, s>>>(v, a.K, a.Np, parity);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    pcg_pupdate_kernel<<<v.G, 256, 0, s>>>(v, (size_t)a.K * a.Np, parity);
    return cudaGetLastError();
}

cudaError_t launch_dot(const double* x, const double* y, size_t n, double* part, int G, cudaStream_t s) {
    dot_kernel<<<G, 256, 0, s>>>(x, y, n, part);
    return cudaGetLastError();
}

cudaError_t launch_reduce_to(const double* part, int G, double* out, cudaStream_t s) {
    reduce_to_kernel<<<1, 32, 0, s>>>(part, G, out);
    return cudaGetLastError();
}

cudaError_t launch_axpy(double* y, const double* x, double alpha, size_t n, cudaStream_t s) {
    axpy_kernel<<<608, 256, 0, s>>>(y, x, alpha, n);
    return cudaGetLastError();
}

cudaError_t launch_xmy(double* out, const double* b, const double* y, size_t n, cudaStream_t s) {
    xmy_kernel<<<608, 256, 0, s>>>(out, b, y, n);
    return cudaGetLastError();
}

cudaError_t launch_permute(const double* in, double* out, const int* perm, int K, int Np, bool to_ring,
                           cudaStream_t s) {
    permute_kernel<<<608, 256, 0, s>>>(in, out, perm, K, Np, to_ring ? 1 : 0);
    return cudaGetLastError();
}

}  // namespace dgk
