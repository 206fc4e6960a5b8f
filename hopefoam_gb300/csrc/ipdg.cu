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
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "../../include/dgcu.h"
#include "dg_ctx.hpp"
#include "euler_flux.cuh"
#include "ipdg.hpp"
#include "lpc.hpp"
#include "mg.hpp"
#include "pcg_reduce.cuh"

namespace dgk {

template <int N>
struct IpDims {
    static constexpr int Np = Dims<N>::Np, Nfp = Dims<N>::Nfp, Nfq = Dims<N>::Nfq;
    static constexpr int THREADS = 256;
    static constexpr int W = (Np > 3 * Nfq) ? Np : 3 * Nfq;  // threads one element needs in either phase
    static constexpr int E = THREADS / W;                    // elements per tile
};

template <typename T>
__device__ __forceinline__ const IpdgOps<T>& ops_of(const IpdgArgs& a);
template <>
__device__ __forceinline__ const IpdgOps<double>& ops_of<double>(const IpdgArgs& a) { return a.o64; }
template <>
__device__ __forceinline__ const IpdgOps<float>& ops_of<float>(const IpdgArgs& a) { return a.o32; }

// Per tile of E elements:
//  (1) staging: the input of the element and of its three face neighbours
//      enters shared memory as offsets from one value per element (its
//      first ring node), formed in FP64 and then rounded to T; the offset
//      between the two elements' values across each face is kept too (FP64
//      difference, rounded to T).  Gradients annihilate constants, so the
//      operator sees only these differences: for a smooth field they are
//      O(h) smaller than the field, and in FP32 arithmetic the apply's error
//      shrinks by that factor (the full field would carry eps32 |u| into
//      every jump and derivative and cost CG its convergence at large
//      condition numbers).  In the PCG the input is the new search direction
//      p = z + beta p_old, formed here in FP64 (and written out for the
//      element's own rows) so that no separate update pass is needed;
//  (2) one thread per (element, face, Gauss point): traces and normal
//      derivatives of both sides, then
//        c1 = wJ (tau/2 [u] - sigma)         multiplies phi_i
//        c2 = -wJ [u] / 2, times n.grad r / n.grad s of the element
//                                            multiply dphi_i/dr, dphi_i/ds;
//  (3) one thread per (element, node): volume term and the face terms.
// Operator tables are read with the thread index running along the
// contiguous dimension (the stiffness parts are symmetric, the face
// derivative tables exist in both layouts), so every warp load is coalesced.
// Persistent CTAs (a few per SM) stride over the tiles; in the PCG each CTA's
// share of p.Ap enters one deterministic grid-wide sum whose last CTA also
// forms alpha (one arrival per CTA, not per tile).
struct ApplyPcg {
    const double* p_old;  // previous search direction (read when beta != 0)
    double* p_new;        // this direction, written for each element's rows
    PcgScalars* S;        // beta in, pap / alpha out; null outside the PCG
    double* part;
    // FP32 offset mirrors (element value minus the element's first-node
    // value) of z and of the search directions; used by the FP32 apply in the
    // PCG so that staging needs no FP64 arithmetic per node
    const float* dz;
    const float* dp_old;
    float* dp_new;
};

template <int N, typename T>
__global__ void __launch_bounds__(256, 4) ipdg_apply_kernel(IpdgArgs a, const double* __restrict__ u,
                                                         double* __restrict__ y, ApplyPcg pc) {
    using D = IpDims<N>;
    constexpr int Np = D::Np, Nfp = D::Nfp, Nfq = D::Nfq, E = D::E, NB = 3 * N, NF = 3 * Nfq;
    const IpdgOps<T>& o = ops_of<T>(a);
    __shared__ T us[E][Np];         // own offsets u - u_k0
    __shared__ T un[E][3][Np];      // neighbour offsets u_nb - u_nb0
    __shared__ T dc[E][3];          // u_k0 - u_nb0 (0 on boundary faces)
    __shared__ T ub0[E];            // u_k0 rounded (Dirichlet jumps)
    __shared__ double pd[E][Np];    // own input in FP64 (offsets, p.Ap)
    __shared__ double stg[E][3][Np];  // neighbour input in FP64 (when not staged from the mirrors)
    __shared__ int nbr[E][3];       // packed neighbour (conn)
    __shared__ T c1[E][NF];
    __shared__ T c2r[E][NF];
    __shared__ T c2s[E][NF];
    double beta = 0.0;
    if (pc.S) {
        if (pc.S->done) return;
        beta = pc.S->beta;
    }
    const double* __restrict__ p_old = pc.p_old;
    const bool mirrors = sizeof(T) == 4 && pc.dz != nullptr;
    const bool has_beta = beta != 0.0;  // uniform: one FP64 compare per thread
    const float betaf = (float)beta;
    const int ntiles = (a.K + E - 1) / E;
    double dot = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int k0 = tile * E;
    const int ne = min(E, a.K - k0);
    // (1) staging.  FP64 work is kept out of divergent branches: a warp
    // instruction occupies the FP64 pipe for its full width whatever its
    // active lanes.  (a) own rows, (b) neighbour rows, (c) per element face.
    for (int t = threadIdx.x; t < ne * Np; t += blockDim.x) {
        const int e = t / Np, p = t - e * Np;
        const size_t i = (size_t)k0 * Np + t;
        const double vp = has_beta ? fma(beta, p_old[i], u[i]) : u[i];
        pd[e][p] = vp;
        if (pc.p_new) pc.p_new[i] = vp;
        if (mirrors) {
            float d = pc.dz[i];
            if (has_beta) d = fmaf(betaf, pc.dp_old[i], d);
            us[e][p] = (T)d;
            pc.dp_new[i] = d;
        }
    }
    for (int t = threadIdx.x; t < ne * 3 * Np; t += blockDim.x) {
        const int e = t / (3 * Np), rem = t - e * 3 * Np, f = rem / Np, p = rem - f * Np;
        const int c = a.conn[(size_t)(k0 + e) * 3 + f];
        if (p == 0) nbr[e][f] = c;
        if (c < 0) continue;
        const size_t i = (size_t)(c >> 3) * Np + p;
        if (mirrors) {
            float d = pc.dz[i];
            if (has_beta) d = fmaf(betaf, pc.dp_old[i], d);
            un[e][f][p] = (T)d;
        } else {
            stg[e][f][p] = has_beta ? fma(beta, p_old[i], u[i]) : u[i];
        }
    }
    __syncthreads();
    if (!mirrors) {
        for (int t = threadIdx.x; t < ne * Np; t += blockDim.x) {
            const int e = t / Np, p = t - e * Np;
            us[e][p] = (T)(pd[e][p] - pd[e][0]);
        }
        for (int t = threadIdx.x; t < ne * 3 * Np; t += blockDim.x) {
            const int e = t / (3 * Np), rem = t - e * 3 * Np, f = rem / Np, p = rem - f * Np;
            if (nbr[e][f] >= 0) un[e][f][p] = (T)(stg[e][f][p] - stg[e][f][0]);
        }
    }
    if (threadIdx.x < ne * 3) {
        const int e = threadIdx.x / 3, f = threadIdx.x - e * 3;
        const int c = nbr[e][f];
        double d = 0.0;
        if (c >= 0) {
            const size_t i0 = (size_t)(c >> 3) * Np;
            d = pd[e][0] - (has_beta ? fma(beta, p_old[i0], u[i0]) : u[i0]);
        }
        dc[e][f] = (T)d;
        if (f == 0) ub0[e] = (T)pd[e][0];
    }
    __syncthreads();
    // (2) face terms
    if (threadIdx.x < ne * NF) {
        const int e = threadIdx.x / NF, fg = threadIdx.x - e * NF, f = fg / Nfq, g = fg - f * Nfq;
        const int k = k0 + e;
        const T* fc = o.fc + ((size_t)k * 3 + f) * kFaceCoef;
        const T arr = fc[0], ass = fc[1];  // n . grad r, n . grad s
        T ur = 0, usd = 0, um = 0;
#pragma unroll
        for (int p = 0; p < Np; p++) {
            ur += o.DrfT[p * NF + fg] * us[e][p];
            usd += o.DsfT[p * NF + fg] * us[e][p];
        }
#pragma unroll
        for (int j = 0; j < Nfp; j++) um += o.If[g * Nfp + j] * us[e][(f * N + j) % NB];
        const T dm = arr * ur + ass * usd;
        T jump, dp;
        const int c = nbr[e][f];
        if (c >= 0) {
            const int fn = c & 3, rot = (c >> 2) & 1;
            const int g2 = rot ? (Nfq - 1 - g) : g;
            const int fg2 = fn * Nfq + g2;
            T vr = 0, vs = 0, up = 0;
#pragma unroll
            for (int p = 0; p < Np; p++) {
                vr += o.DrfT[p * NF + fg2] * un[e][f][p];
                vs += o.DsfT[p * NF + fg2] * un[e][f][p];
            }
#pragma unroll
            for (int j = 0; j < Nfp; j++) {
                const int jj = rot ? (N - j) : j;
                up += o.If[g * Nfp + j] * un[e][f][(fn * N + jj) % NB];
            }
            dp = fc[2] * vr + fc[3] * vs;  // own normal . grad r, s of the neighbour
            jump = (um - up) + dc[e][f];
        } else {
            // Dirichlet face: u+ = -u-, so [u] = 2 u- (offset included)
            jump = (T)2 * (um + ub0[e]);
            dp = dm;
        }
        const T wJ = fc[5] * o.fw[g];
        const T sigma = (T)0.5 * (dm + dp);
        const T cc2 = -(T)0.5 * wJ * jump;
        c1[e][fg] = wJ * (fc[4] * jump - sigma);
        c2r[e][fg] = cc2 * arr;
        c2s[e][fg] = cc2 * ass;
    }
    __syncthreads();
    // (3) element rows
    if (threadIdx.x < ne * Np) {
        const int e = threadIdx.x / Np, i = threadIdx.x - e * Np;
        const int k = k0 + e;
        T A = 0, B = 0, C = 0;
#pragma unroll
        for (int p = 0; p < Np; p++) {
            const T up = us[e][p];
            A += o.Srr[p * Np + i] * up;
            B += o.Srs2[p * Np + i] * up;
            C += o.Sss[p * Np + i] * up;
        }
        T v = o.vc[(size_t)k * 3] * A + o.vc[(size_t)k * 3 + 1] * B + o.vc[(size_t)k * 3 + 2] * C;
        if (a.mass_coef != 0.0) {
            // Helmholtz term mass_coef J M u, u = offsets + the element's first-node value
            T m = o.mrow[i] * ub0[e];
#pragma unroll
            for (int p = 0; p < Np; p++) m += o.Mr[p * Np + i] * us[e][p];
            v += (T)(a.mass_coef * a.J[k]) * m;
        }
#pragma unroll
        for (int fg = 0; fg < NF; fg++) v += c2r[e][fg] * o.Drf[fg * Np + i] + c2s[e][fg] * o.Dsf[fg * Np + i];
        if (i < NB) {
#pragma unroll
            for (int f = 0; f < 3; f++) {
                const int d = (i - f * N + NB) % NB;  // phi_i on face f: ring positions f*N .. f*N+N (mod 3N)
                if (d <= N) {
#pragma unroll
                    for (int g = 0; g < Nfq; g++) v += c1[e][f * Nfq + g] * o.If[g * Nfp + d];
                }
            }
        }
        const double out = (double)v;
        y[(size_t)k * Np + i] = out;
        dot += out * pd[e][i];
    }
    __syncthreads();  // shared tile buffers are refilled by the next tile
    }
    if (pc.S) {
        double val[1] = {dot}, tot[1];
        if (grid_sum<1>(val, pc.part, gridDim.x, &pc.S->counter, tot) && threadIdx.x == 0) {
            const double pap = tot[0];
            pc.S->pap = pap;
            pc.S->alpha = pc.S->rz / pap;
            if (!(pap > 0.0) || !(pc.S->alpha == pc.S->alpha)) pc.S->done = 2;
        }
    }
}

// SIPG apply for the FP32 iterations of the PCG (N <= 5), in two passes with
// one element per lane pair.  Every reference table entry is a
// kernel-parameter (constant-bank) operand of the FMA that uses it, so the
// arithmetic is FMAs plus the element's own loads.  The face terms need, on
// each side of a face, the input's trace and normal derivative at the face's
// Gauss points.  The first pass forms the input p = z + beta p_old (FP64,
// written out for the element's rows, and as FP32 offsets from the element's
// first-node value) and writes, for every element and face, the trace
// (offset form) and the outward normal derivative at the Gauss points in the
// element's own order: LaneFaceRec<N>::R floats per face.  The second pass
// reads its own records and, per interior face, the neighbour's record of
// the shared face (a contiguous 16-byte-aligned run instead of a gather of
// the neighbour's nodes).  The neighbour traverses the shared face the other
// way when rot is set (Gauss point g is its point Nfq-1-g), and its outward
// normal is the negated one of this element, so the neighbour-side
// derivative along this element's normal is minus its own.  The offset
// between the two elements' first-node values enters the jump; each value is
// kept as an FP32 pair (hi, lo) and the offset formed as (hi - hi') + (lo -
// lo') in FP32 (within about one FP32 rounding of the exact difference, with
// no FP64 work per face).  Same operator and outputs as ipdg_apply_kernel; the
// sums run in another order, so results agree to FP32 round-off.
// Both passes run two lanes per element: a CTA of 256 threads covers a tile
// of 128 elements, its warps 0-3 take one half of the work of each element
// (Gauss points in the first pass, output rows in the second) and warps 4-7
// the other, so the half is uniform across a warp and every table entry
// stays a constant-bank operand.
template <int N>
struct LaneFaceRec {
    static constexpr int Nfq = N + 2, R = lane_face_rec(N), ER = 3 * R, SR = ER + 1;  // SR: padded smem stride
    static constexpr int GH = (Nfq + 1) / 2;                 // first pass: Gauss points [0, GH) | [GH, Nfq)
    static constexpr int Np = (N + 1) * (N + 2) / 2, NH = (Np + 1) / 2;  // second pass: rows [0, NH) | [NH, Np)
};

template <int H>
using HalfTag = std::integral_constant<int, H>;

template <int N>
__global__ void __launch_bounds__(256) ipdg_lane_trace_kernel(IpdgArgs a, const __grid_constant__ IpLaneTab<N> T,
                                                              const double* __restrict__ u, ApplyPcg pc) {
    using L = IpLaneTab<N>;
    using FR = LaneFaceRec<N>;
    constexpr int Np = L::Np, Nfp = L::Nfp, Nfq = L::Nfq, NB = 3 * N, R = FR::R, ER = FR::ER, SR = FR::SR,
                  GH = FR::GH;
    if (pc.S->done) return;
    const double beta = pc.S->beta;
    const bool has_beta = beta != 0.0;
    const float betaf = (float)beta;
    const double* __restrict__ p_old = pc.p_old;
    const float* __restrict__ dzv = pc.dz;
    const float* __restrict__ dpo = pc.dp_old;
    double* __restrict__ p_new = pc.p_new;
    float* __restrict__ dp_new = pc.dp_new;
    float* __restrict__ ftr = a.lane_ftr;
    float2* __restrict__ p0 = a.lane_p0;
    __shared__ float sd[128 * Np];
    __shared__ float srec[128 * SR];
    __shared__ double sp0[128];
    const int e = threadIdx.x & 127, h = threadIdx.x >> 7;
    const int ntiles = (a.K + 127) / 128;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int k0 = tile * 128, ne = min(128, a.K - k0), nn = ne * Np;
        const size_t g0 = (size_t)k0 * Np;
        // node-parallel staging in batches of SB nodes per thread, every
        // load of a batch issued before its first use
        constexpr int J = (Np + 1) / 2, SB = 4;
#pragma unroll
        for (int j0 = 0; j0 < J; j0 += SB) {
            double xu[SB], xp[SB];
            float fz[SB], fp[SB];
#pragma unroll
            for (int j = 0; j < SB; j++) {
                const int t = threadIdx.x + 256 * (j0 + j);
                if (j0 + j < J && t < nn) {
                    xu[j] = u[g0 + t];
                    fz[j] = dzv[g0 + t];
                    if (has_beta) {
                        xp[j] = p_old[g0 + t];
                        fp[j] = dpo[g0 + t];
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < SB; j++) {
                const int t = threadIdx.x + 256 * (j0 + j);
                if (j0 + j < J && t < nn) {
                    const double vp = has_beta ? fma(beta, xp[j], xu[j]) : xu[j];
                    if (p_new) p_new[g0 + t] = vp;
                    const int e2 = t / Np;
                    if (t == e2 * Np) sp0[e2] = vp;
                    const float d = has_beta ? fmaf(betaf, fp[j], fz[j]) : fz[j];
                    dp_new[g0 + t] = d;
                    sd[t] = d;
                }
            }
        }
        __syncthreads();
        if (e < ne) {
            const int k = k0 + e;
            if (h == 0) {
                const double v0 = sp0[e];
                const float hi = (float)v0;
                p0[k] = make_float2(hi, (float)(v0 - (double)hi));
            }
            float us[Np];
#pragma unroll
            for (int p = 0; p < Np; p++) us[p] = sd[e * Np + p];
            float* rec = srec + e * SR;
            auto points = [&](auto hc) {
                constexpr int g0h = decltype(hc)::value ? GH : 0, g1h = decltype(hc)::value ? Nfq : GH;
#pragma unroll
                for (int f = 0; f < 3; f++) {
                    const float2 f01 = *reinterpret_cast<const float2*>(a.o32.fc + ((size_t)k * 3 + f) * kFaceCoef);
#pragma unroll
                    for (int g = g0h; g < g1h; g++) {
                        const int fg = f * Nfq + g;
                        float ur = 0.f, usd = 0.f, um = 0.f;
#pragma unroll
                        for (int p = 0; p < Np; p++) {
                            ur = fmaf(T.DrfT[p][fg], us[p], ur);
                            usd = fmaf(T.DsfT[p][fg], us[p], usd);
                        }
#pragma unroll
                        for (int j = 0; j < Nfp; j++) um = fmaf(T.If[g][j], us[(f * N + j) % NB], um);
                        rec[f * R + g] = um;
                        rec[f * R + Nfq + g] = f01.x * ur + f01.y * usd;
                    }
                    if (decltype(hc)::value) {
#pragma unroll
                        for (int q = 2 * Nfq; q < R; q++) rec[f * R + q] = 0.f;
                    }
                }
            };
            if (h == 0) points(HalfTag<0>{});
            else points(HalfTag<1>{});
        }
        __syncthreads();
        // records out, 16 bytes per store (ER is a multiple of 4)
        float4* dst = reinterpret_cast<float4*>(ftr + (size_t)k0 * ER);
        const int n4 = ne * (ER / 4);
#pragma unroll
        for (int j = 0; j < (ER / 4 + 1) / 2; j++) {
            const int t4 = threadIdx.x + 256 * j;
            if (t4 < n4) {
                const int e2 = (4 * t4) / ER;
                const float* src = srec + e2 * SR + (4 * t4 - e2 * ER);
                dst[t4] = make_float4(src[0], src[1], src[2], src[3]);
            }
        }
        __syncthreads();  // the next tile rewrites sd and srec
    }
}

template <int N>
__global__ void __launch_bounds__(256, N <= 4 ? 3 : 2) ipdg_lane_face_apply_kernel(IpdgArgs a,
        const __grid_constant__ IpLaneTab<N> T, double* __restrict__ y, ApplyPcg pc) {
    using L = IpLaneTab<N>;
    using FR = LaneFaceRec<N>;
    constexpr int Np = L::Np, Nfq = L::Nfq, NB = 3 * N, R = FR::R, ER = FR::ER, SR = FR::SR, NH = FR::NH;
    if (pc.S->done) return;
    const bool mass = a.mass_coef != 0.0;
    const double* __restrict__ p_new = pc.p_new;
    const float* __restrict__ dp_new = pc.dp_new;
    const float* __restrict__ ftr = a.lane_ftr;
    const float2* __restrict__ p0 = a.lane_p0;
    __shared__ float sd[128 * Np];
    __shared__ float srec[128 * SR];
    __shared__ float sout[128 * Np];
    const int e = threadIdx.x & 127, h = threadIdx.x >> 7;
    double dot = 0.0;
    const int ntiles = (a.K + 127) / 128;
    constexpr int J = (Np + 1) / 2, J4 = (ER / 4 + 1) / 2;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int k0 = tile * 128, ne = min(128, a.K - k0), nn = ne * Np, n4 = ne * (ER / 4);
        const size_t g0 = (size_t)k0 * Np;
        {
            float xs[J];
            float4 xr[J4];
#pragma unroll
            for (int j = 0; j < J; j++) {
                const int t = threadIdx.x + 256 * j;
                if (t < nn) xs[j] = dp_new[g0 + t];
            }
            const float4* src = reinterpret_cast<const float4*>(ftr + (size_t)k0 * ER);
#pragma unroll
            for (int j = 0; j < J4; j++) {
                const int t4 = threadIdx.x + 256 * j;
                if (t4 < n4) xr[j] = src[t4];
            }
#pragma unroll
            for (int j = 0; j < J; j++) {
                const int t = threadIdx.x + 256 * j;
                if (t < nn) sd[t] = xs[j];
            }
#pragma unroll
            for (int j = 0; j < J4; j++) {
                const int t4 = threadIdx.x + 256 * j;
                if (t4 < n4) {
                    const int e2 = (4 * t4) / ER;
                    float* d = srec + e2 * SR + (4 * t4 - e2 * ER);
                    d[0] = xr[j].x;
                    d[1] = xr[j].y;
                    d[2] = xr[j].z;
                    d[3] = xr[j].w;
                }
            }
        }
        __syncthreads();
        if (e < ne) {
            const int k = k0 + e;
            float us[Np];
#pragma unroll
            for (int p = 0; p < Np; p++) us[p] = sd[e * Np + p];
            const float2 pd0 = p0[k];
            const float ub0 = pd0.x;
            const float* vc = a.o32.vc + (size_t)k * 3;
            const float vrr = vc[0], vrs = vc[1], vss = vc[2];
            const float* rec = srec + e * SR;
            auto rows = [&](auto hc) {
                constexpr int i0 = decltype(hc)::value ? NH : 0, i1 = decltype(hc)::value ? Np : NH;
                float v[NH];
#pragma unroll
                for (int i = i0; i < i1; i++) {
                    float A = 0.f, B = 0.f, C = 0.f;
#pragma unroll
                    for (int p = 0; p < Np; p++) {
                        A = fmaf(T.Srr[i][p], us[p], A);
                        B = fmaf(T.Srs2[i][p], us[p], B);
                        C = fmaf(T.Sss[i][p], us[p], C);
                    }
                    v[i - i0] = vrr * A + vrs * B + vss * C;
                }
                if (mass) {
                    const float mc = (float)(a.mass_coef * a.J[k]);
#pragma unroll
                    for (int i = i0; i < i1; i++) {
                        float m = T.mrow[i] * ub0;
#pragma unroll
                        for (int p = 0; p < Np; p++) m = fmaf(T.Mr[i][p], us[p], m);
                        v[i - i0] = fmaf(mc, m, v[i - i0]);
                    }
                }
#pragma unroll
                for (int f = 0; f < 3; f++) {
                    const int c = a.conn[(size_t)k * 3 + f];
                    const float2* fcp = reinterpret_cast<const float2*>(a.o32.fc + ((size_t)k * 3 + f) * kFaceCoef);
                    const float2 f01 = fcp[0], f45 = fcp[2];
                    const bool interior = c >= 0;
                    const bool rot = (c >> 2) & 1;
                    float nr[R];
                    float dc = 0.f;
                    if (interior) {
                        const int nbk = c >> 3, fn = c & 3;
                        const float4* src = reinterpret_cast<const float4*>(ftr + ((size_t)nbk * 3 + fn) * R);
#pragma unroll
                        for (int q = 0; q < R / 4; q++) {
                            const float4 w = src[q];
                            nr[4 * q] = w.x;
                            nr[4 * q + 1] = w.y;
                            nr[4 * q + 2] = w.z;
                            nr[4 * q + 3] = w.w;
                        }
                        const float2 pn = p0[nbk];
                        dc = (pd0.x - pn.x) + (pd0.y - pn.y);
                    } else {
#pragma unroll
                        for (int q = 0; q < R; q++) nr[q] = 0.f;
                    }
#pragma unroll
                    for (int g = 0; g < Nfq; g++) {
                        const int fg = f * Nfq + g;
                        const float um = rec[f * R + g], dm = rec[f * R + Nfq + g];
                        float jump, dp;
                        if (interior) {
                            const float up = rot ? nr[Nfq - 1 - g] : nr[g];
                            dp = -(rot ? nr[2 * Nfq - 1 - g] : nr[Nfq + g]);
                            jump = (um - up) + dc;
                        } else {
                            // Dirichlet face: u+ = -u-, so [u] = 2 u- (offset included)
                            jump = 2.f * (um + ub0);
                            dp = dm;
                        }
                        const float wJ = f45.y * T.fw[g];
                        const float sigma = 0.5f * (dm + dp);
                        const float cc2 = -0.5f * wJ * jump;
                        const float c1 = wJ * (f45.x * jump - sigma);
                        const float c2r = cc2 * f01.x, c2s = cc2 * f01.y;
#pragma unroll
                        for (int i = i0; i < i1; i++)
                            v[i - i0] = fmaf(c2r, T.DrfT[i][fg], fmaf(c2s, T.DsfT[i][fg], v[i - i0]));
#pragma unroll
                        for (int d = 0; d <= N; d++) {
                            const int i = (f * N + d) % NB;
                            if (i >= i0 && i < i1) v[i - i0] = fmaf(c1, T.If[g][d], v[i - i0]);
                        }
                    }
                }
#pragma unroll
                for (int i = i0; i < i1; i++) sout[e * Np + i] = v[i - i0];
            };
            if (h == 0) rows(HalfTag<0>{});
            else rows(HalfTag<1>{});
        }
        __syncthreads();
        {
            double xp[J];
#pragma unroll
            for (int j = 0; j < J; j++) {
                const int t = threadIdx.x + 256 * j;
                if (t < nn) xp[j] = p_new[g0 + t];
            }
#pragma unroll
            for (int j = 0; j < J; j++) {
                const int t = threadIdx.x + 256 * j;
                if (t < nn) {
                    const double out = (double)sout[t];
                    y[g0 + t] = out;
                    dot += out * xp[j];
                }
            }
        }
        __syncthreads();  // the next tile rewrites sd and srec
    }
    double val[1] = {dot}, tot[1];
    if (grid_sum<1>(val, pc.part, gridDim.x, &pc.S->counter, tot) && threadIdx.x == 0) {
        const double pap = tot[0];
        pc.S->pap = pap;
        pc.S->alpha = pc.S->rz / pap;
        if (!(pap > 0.0) || !(pc.S->alpha == pc.S->alpha)) pc.S->done = 2;
    }
}

// diagonal blocks S_kk (column j = S_kk e_j with neighbours zero), FP64
template <int N>
__global__ void ipdg_diag_kernel(IpdgArgs a, double* __restrict__ blocks) {
    using D = IpDims<N>;
    constexpr int Np = D::Np, Nfp = D::Nfp, Nfq = D::Nfq, NB = 3 * N;
    const IpdgOps<double>& o = a.o64;
    const int k = blockIdx.x;
    const int j = threadIdx.x;  // column
    if (k >= a.K || j >= Np) return;
    const double vrr = o.vc[(size_t)k * 3], vrs = o.vc[(size_t)k * 3 + 1], vss = o.vc[(size_t)k * 3 + 2];
    double col[Np];
    const double mc = a.mass_coef * a.J[k];
    for (int i = 0; i < Np; i++)
        col[i] = vrr * o.Srr[i * Np + j] + vrs * o.Srs2[i * Np + j] + vss * o.Sss[i * Np + j] + mc * o.Mr[i * Np + j];
    for (int f = 0; f < 3; f++) {
        const double* fc = o.fc + ((size_t)k * 3 + f) * kFaceCoef;
        const double arr = fc[0], ass = fc[1];
        const int c = a.conn[(size_t)k * 3 + f];
        // u = e_j: own trace / normal derivative at each Gauss point
        int jf = -1;
        if (j < NB) {
            const int d = (j - f * N + NB) % NB;
            if (d <= N) jf = d;
        }
        for (int g = 0; g < Nfq; g++) {
            const double um = jf >= 0 ? o.If[g * Nfp + jf] : 0.0;
            const double dm = arr * o.Drf[(f * Nfq + g) * Np + j] + ass * o.Dsf[(f * Nfq + g) * Np + j];
            const double up = (c >= 0) ? 0.0 : -um;
            const double dp = (c >= 0) ? 0.0 : dm;
            const double wJ = fc[5] * o.fw[g];
            const double jump = um - up, sigma = 0.5 * (dm + dp);
            const double cc1 = wJ * (fc[4] * jump - sigma), cc2 = -0.5 * wJ * jump;
            for (int i = 0; i < Np; i++) {
                double t = cc2 * (arr * o.Drf[(f * Nfq + g) * Np + i] + ass * o.Dsf[(f * Nfq + g) * Np + i]);
                if (i < NB) {
                    const int d = (i - f * N + NB) % NB;
                    if (d <= N) t += cc1 * o.If[g * Nfp + d];
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
    for (int i = 0; i < Np * Np; i++) {
        A[i] = X[i];
        if (blocks32) blocks32[(size_t)k * Np * Np + i] = (float)X[i];
    }
}

// ---------------------------------------------------------------------------
// PCG.  Scalars live on the device (PcgScalars); every kernel returns at once
// when the solve has stopped (S->done), so launches are issued ahead of the
// host's convergence check.  Dot products are deterministic grid-wide sums
// (pcg_reduce.cuh); the last CTA of each sum forms the scalars that the next
// kernel needs (alpha after the apply, beta and the stop test after the
// update), so an iteration is two launches: apply (with p = z + beta p_old
// fused in) and update.

// standalone partial sums (host-side dot products): per-CTA partials over a
// fixed grid, reduced in fixed order by reduce_to_kernel
__device__ __forceinline__ void block_sum1(double a, double* oa) {
    __shared__ double ra[32];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) ra[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sa = 0;
        for (int w = 0; w < (int)((blockDim.x + 31) >> 5); w++) sa += ra[w];
        *oa = sa;
    }
}

// Element-aligned kernels: a group of EB = 256 / Np whole elements, one
// thread per (element, row), Np a compile-time constant so that the block
// products unroll (Np independent loads in flight per thread).  Persistent
// CTAs (a few per SM) stride over the groups, so each grid-wide sum has one
// arrival per CTA.  The inverse diagonal blocks are stored grouped: for group
// g and column j the EB x Np entries (element, row) are contiguous,
//   Pg[((g Np + j) EB + e) Np + i] = P_{g EB + e}[i][j],
// so the CTA's loads for one column form a single contiguous read.
//
// Up to Np = 32 (N <= 6) an element's rows never straddle a warp: each warp
// holds EW = 32 / Np whole elements (WA), so the rows of an element exchange
// their values by warp shuffles and the kernels need no CTA barrier per
// group.  N = 7 (Np = 36) keeps one shared-memory exchange per group.
template <int NP>
struct RowDims {
    static constexpr bool WA = NP <= 32;
    static constexpr int EW = WA ? 32 / NP : 0;  // elements per warp
    static constexpr int EB = WA ? 8 * EW : 256 / NP;
    static constexpr int THREADS = WA ? 256 : (EB * NP + 31) / 32 * 32;  // extra lanes idle but join the reductions
};

// this thread's (element in the group, row) and its slot in the grouped layout
template <int NP>
__device__ __forceinline__ void row_of(int& e, int& i) {
    if constexpr (RowDims<NP>::WA) {
        const int lane = threadIdx.x & 31;
        e = (threadIdx.x >> 5) * RowDims<NP>::EW + lane / NP;
        i = lane % NP;
        if (lane >= RowDims<NP>::EW * NP) e = RowDims<NP>::EB;  // idle lane
    } else {
        e = threadIdx.x / NP;
        i = threadIdx.x - e * NP;
    }
}

__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }

// FP32 offset mirror of z (value minus the element's row-0 value, lane lb of
// the warp-aligned layout).  With FP32 blocks z is an FP32 product widened to
// FP64, and the difference of two FP32 values rounded once to FP32 equals the
// FP32 subtraction: no FP64 work.  Warp-uniform flags (every lane shuffles).
__device__ __forceinline__ float mirror_offset(bool want, bool fp64_blocks, double z, float zf, int lb) {
    if (!want) return 0.f;
    if (fp64_blocks) return (float)(z - __shfl_sync(0xffffffffu, z, lb));
    return zf - __shfl_sync(0xffffffffu, zf, lb);
}

// this thread's row of its element's inverse block (grouped layout), loaded
// ahead of the residual it multiplies
template <int NP, typename PT>
__device__ __forceinline__ void bj_row_load(const PT* __restrict__ P, int grp, PT (&row)[NP]) {
    constexpr int EBNP = RowDims<NP>::EB * NP;
    int e, i;
    row_of<NP>(e, i);
    const PT* col = P + (size_t)grp * NP * EBNP + e * NP + i;
#pragma unroll
    for (int j = 0; j < NP; j++) row[j] = __ldg(col + j * EBNP);
}

template <int NP, typename PT, typename RT>
__device__ __forceinline__ double bj_row_apply(const PT (&row)[NP], const RT* rs) {
    PT s = 0;
#pragma unroll
    for (int j = 0; j < NP; j++) s = fma_t(row[j], (PT)rs[j], s);
    return (double)s;
}

template <int NP, typename PT, typename RT>
__device__ __forceinline__ double bj_rowg(const PT* __restrict__ P, const RT* rs, int grp) {
    constexpr int EBNP = RowDims<NP>::EB * NP;
    int e, i;
    row_of<NP>(e, i);
    const PT* col = P + (size_t)grp * NP * EBNP + e * NP + i;
    PT s = 0;
#pragma unroll
    for (int j = 0; j < NP; j++) s = fma_t(col[j * EBNP], (PT)rs[j], s);
    return (double)s;
}

// mode 0 (init):    z = P r; S->rz = r.z, S->rr = r.r, beta = 0 (first p = z)
// mode 1 (refresh): the same, beta kept (residual replacement)
// Learned mode (v.zb): zb = P r and S->rr only; the learned kernel forms z, r.z.
template <int NP>
__global__ void __launch_bounds__(RowDims<NP>::THREADS) pcg_init_kernel(PcgVecs v, int K, int mode) {
    constexpr int EB = RowDims<NP>::EB;
    int e, i;
    row_of<NP>(e, i);
    const int ngroups = (K + EB - 1) / EB;
    double rz = 0, rr = 0;
    if constexpr (RowDims<NP>::WA) {
        const int lb = (threadIdx.x & 31) - i;  // lane of the element's row 0
        for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
            const int k = grp * EB + e;
            const bool act = e < EB && k < K;
            const size_t idx = (size_t)k * NP + i;
            const double ri = act ? v.r[idx] : 0.0;
            const float r32 = (float)ri;
            double z = 0;
            float zf = 0.f;  // the FP32 product (FP32 blocks)
            if (v.P64) {
                double s = 0;
                const double* col = v.P64 + (size_t)grp * NP * EB * NP + e * NP + i;
#pragma unroll
                for (int j = 0; j < NP; j++) {
                    const double rj = __shfl_sync(0xffffffffu, ri, lb + j);
                    if (act) s = fma(__ldg(col + (size_t)j * EB * NP), rj, s);
                }
                z = s;
            } else {
                float prow[NP];
                if (act) bj_row_load<NP>(v.P32, grp, prow);
                float s = 0.f;
#pragma unroll
                for (int j = 0; j < NP; j++) {
                    const float rj = __shfl_sync(0xffffffffu, r32, lb + j);
                    if (act) s = fmaf(prow[j], rj, s);
                }
                z = (double)s;
                zf = s;
            }
            const float dzi = mirror_offset(v.dz != nullptr, v.P64 != nullptr, z, zf, lb);
            if (act) {
                if (v.zb) v.zb[idx] = z;
                else {
                    v.z[idx] = z;
                    rz += ri * z;
                }
                if (v.r32) v.r32[idx] = r32;
                if (v.dz) v.dz[idx] = dzi;  // learned mode: the mirror of P r
                rr += ri * ri;
            }
        }
    } else {
        __shared__ double rs[EB][NP];
        __shared__ float rs32[EB][NP];
        __shared__ double zs0[EB];
        for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
            const int k = grp * EB + e;
            const bool act = e < EB && k < K;
            const size_t idx = (size_t)k * NP + i;
            double ri = 0, z = 0;
            if (act) {
                ri = v.r[idx];
                rs[e][i] = ri;
                rs32[e][i] = (float)ri;
            }
            __syncthreads();
            if (act) {
                z = v.P64 ? bj_rowg<NP>(v.P64, rs[e], grp) : bj_rowg<NP>(v.P32, rs32[e], grp);
                if (v.zb) v.zb[idx] = z;
                else {
                    v.z[idx] = z;
                    rz += ri * z;
                }
                if (i == 0) zs0[e] = z;
                if (v.r32) v.r32[idx] = rs32[e][i];
                rr += ri * ri;
            }
            if (v.dz) {  // learned mode: the mirror of P r, completed by the learned kernel
                __syncthreads();
                if (act) v.dz[idx] = (float)(z - zs0[e]);
            }
            __syncthreads();
        }
    }
    double val[2] = {rz, rr}, tot[2];
    if (grid_sum<2>(val, v.part, gridDim.x, &v.S->counter, tot) && threadIdx.x == 0) {
        v.S->rr = tot[1];
        if (!v.zb) v.S->rz = tot[0];
        if (mode == 0) {
            v.S->beta = 0.0;
            if (tot[1] <= v.S->tol2) v.S->done = 1;
        }
    }
}

// z = P r over all elements (FP32 blocks)
template <int NP>
__global__ void __launch_bounds__(RowDims<NP>::THREADS) bj_kernel(const float* __restrict__ P32,
                                                                  const double* __restrict__ r,
                                                                  double* __restrict__ z, int K) {
    constexpr int EB = RowDims<NP>::EB;
    int e, i;
    row_of<NP>(e, i);
    const int ngroups = (K + EB - 1) / EB;
    if constexpr (RowDims<NP>::WA) {
        const int lb = (threadIdx.x & 31) - i;
        for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
            const int k = grp * EB + e;
            const bool act = e < EB && k < K;
            const float r32 = act ? (float)r[(size_t)k * NP + i] : 0.f;
            float prow[NP];
            if (act) bj_row_load<NP>(P32, grp, prow);
            float s = 0.f;
#pragma unroll
            for (int j = 0; j < NP; j++) {
                const float rj = __shfl_sync(0xffffffffu, r32, lb + j);
                if (act) s = fmaf(prow[j], rj, s);
            }
            if (act) z[(size_t)k * NP + i] = (double)s;
        }
    } else {
        __shared__ float rs32[EB][NP];
        for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
            const int k = grp * EB + e;
            const bool act = e < EB && k < K;
            if (act) rs32[e][i] = (float)r[(size_t)k * NP + i];
            __syncthreads();
            if (act) z[(size_t)k * NP + i] = bj_rowg<NP>(P32, rs32[e], grp);
            __syncthreads();
        }
    }
}

// x += alpha p; r -= alpha Ap; z = P r; then beta = r.z / r_old.z_old and the
// stop test (learned mode: zb = P r and r.r only; the learned kernel uses the
// flexible beta)
template <int NP>
__global__ void __launch_bounds__(RowDims<NP>::THREADS) pcg_update_kernel(PcgVecs v, int K, int parity) {
    constexpr int EB = RowDims<NP>::EB;
    if (v.S->done) return;
    const double alpha = v.S->alpha;
    const double* __restrict__ p = v.p[parity ^ 1];
    int e, i;
    row_of<NP>(e, i);
    const int ngroups = (K + EB - 1) / EB;
    double rz = 0, rr = 0, rzo = 0;
    if constexpr (RowDims<NP>::WA) {
        // no CTA barrier: the element's residual reaches its rows by shuffles
        const int lb = (threadIdx.x & 31) - i;
        for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
            const int k = grp * EB + e;
            const bool act = e < EB && k < K;
            const size_t idx = (size_t)k * NP + i;
            // the block row is loaded with the vectors (one memory phase per group)
            float prow[NP];
            if (act && !v.P64) bj_row_load<NP>(v.P32, grp, prow);
            double ri = 0;
            if (act) {
                v.x[idx] += alpha * p[idx];
                ri = v.r[idx] - alpha * v.Ap[idx];
                v.r[idx] = ri;
            }
            const float r32 = (float)ri;
            double z = 0;
            float zf = 0.f;  // the FP32 product (FP32 blocks)
            if (v.P64) {
                double s = 0;
                const double* col = v.P64 + (size_t)grp * NP * EB * NP + e * NP + i;
#pragma unroll
                for (int j = 0; j < NP; j++) {
                    const double rj = __shfl_sync(0xffffffffu, ri, lb + j);
                    if (act) s = fma(__ldg(col + (size_t)j * EB * NP), rj, s);
                }
                z = s;
            } else {
                float s = 0.f;
#pragma unroll
                for (int j = 0; j < NP; j++) {
                    const float rj = __shfl_sync(0xffffffffu, r32, lb + j);
                    if (act) s = fmaf(prow[j], rj, s);
                }
                z = (double)s;
                zf = s;
            }
            const float dzi = mirror_offset(v.dz != nullptr, v.P64 != nullptr, z, zf, lb);
            if (act) {
                rr += ri * ri;
                if (v.r32) v.r32[idx] = r32;
                if (v.zb) {
                    v.zb[idx] = z;  // the learned kernel forms z and finishes the iteration
                } else {
                    // block Jacobi is a fixed linear preconditioner: the standard
                    // (Fletcher-Reeves) beta needs no r.z_old
                    v.z[idx] = z;
                    rz += ri * z;
                }
                if (v.dz) v.dz[idx] = dzi;  // learned mode: the mirror of P r
            }
        }
    } else {
        __shared__ double rs[EB][NP];
        __shared__ float rs32[EB][NP];
        __shared__ double zs0[EB];
        for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
            const int k = grp * EB + e;
            const bool act = e < EB && k < K;
            const size_t idx = (size_t)k * NP + i;
            double ri = 0, z = 0;
            float prow[NP];
            if (act && !v.P64) bj_row_load<NP>(v.P32, grp, prow);
            if (act) {
                v.x[idx] += alpha * p[idx];
                ri = v.r[idx] - alpha * v.Ap[idx];
                v.r[idx] = ri;
                if (v.P64) rs[e][i] = ri;
                if (!v.P64 || v.r32) rs32[e][i] = (float)ri;
            }
            __syncthreads();
            if (act) {
                z = v.P64 ? bj_rowg<NP>(v.P64, rs[e], grp) : bj_row_apply<NP>(prow, rs32[e]);
                rr += ri * ri;
                if (v.r32) v.r32[idx] = rs32[e][i];
                if (v.zb) v.zb[idx] = z;
                else {
                    v.z[idx] = z;
                    rz += ri * z;
                }
                if (i == 0) zs0[e] = z;
            }
            if (v.dz) {
                __syncthreads();
                if (act) v.dz[idx] = (float)(z - zs0[e]);
            }
            __syncthreads();
        }
    }
    double val[3] = {rz, rr, rzo}, tot[3];
    if (grid_sum<3>(val, v.part, gridDim.x, &v.S->counter, tot) && threadIdx.x == 0) {
        if (v.zb) v.S->rr = tot[1];
        else pcg_finish(v.S, tot[0], tot[2], tot[1]);
    }
}

// inverse blocks (row-major per element) -> grouped layout (zero padding)
template <int NP>
__global__ void group_blocks_kernel(const double* __restrict__ blk, double* __restrict__ P64,
                                    float* __restrict__ P32, int K) {
    constexpr int EB = RowDims<NP>::EB;
    const int ngroups = (K + EB - 1) / EB;
    const size_t total = (size_t)ngroups * NP * EB * NP;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % NP);
        const int e = (int)((t / NP) % EB);
        const int j = (int)((t / ((size_t)NP * EB)) % NP);
        const int grp = (int)(t / ((size_t)NP * EB * NP));
        const int k = grp * EB + e;
        const double val = k < K ? blk[(size_t)k * NP * NP + (size_t)i * NP + j] : 0.0;
        P64[t] = val;
        P32[t] = (float)val;
    }
}

__global__ void dot_kernel(const double* __restrict__ x, const double* __restrict__ y, size_t n, double* part) {
    double s = 0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        s += x[t] * y[t];
    block_sum1(s, part + blockIdx.x);
}

__global__ void reduce_to_kernel(const double* __restrict__ part, int G, double* out) {
    if (threadIdx.x < 32) {
        double s = 0;
        for (int i = threadIdx.x; i < G; i += 32) s += part[i];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
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

// persistent grid: CTAs per SM that fit (64 registers x 256 threads: 4), at most one per tile
template <int N>
static int apply_grid(const IpdgArgs& a) {
    const int ntiles = (a.K + IpDims<N>::E - 1) / IpDims<N>::E;
    return std::max(1, std::min(ntiles, 4 * a.sms));
}

template <int N>
static cudaError_t apply_n(const IpdgArgs& a, bool fp32, const double* u, double* y, const ApplyPcg& pc,
                           cudaStream_t s) {
    using D = IpDims<N>;
    if constexpr (N <= 5) {
        if (fp32 && pc.dz && pc.S && pc.p_new && a.lane_tab && a.lane_ftr && a.lane_p0) {
            const int grid = std::max(1, std::min((a.K + 127) / 128, pcg_max_grid(a.K, N, a.sms)));
            const IpLaneTab<N>& tab = *static_cast<const IpLaneTab<N>*>(a.lane_tab);
            ipdg_lane_trace_kernel<N><<<grid, 256, 0, s>>>(a, tab, u, pc);
            const cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
            ipdg_lane_face_apply_kernel<N><<<grid, 256, 0, s>>>(a, tab, y, pc);
            return cudaGetLastError();
        }
    }
    const int grid = apply_grid<N>(a);
    if (fp32) ipdg_apply_kernel<N, float><<<grid, D::THREADS, 0, s>>>(a, u, y, pc);
    else ipdg_apply_kernel<N, double><<<grid, D::THREADS, 0, s>>>(a, u, y, pc);
    return cudaGetLastError();
}

static cudaError_t apply_dispatch(const IpdgArgs& a, bool fp32, const double* u, double* y, const ApplyPcg& pc,
                                  cudaStream_t s) {
    switch (a.N) {
        case 1: return apply_n<1>(a, fp32, u, y, pc, s);
        case 2: return apply_n<2>(a, fp32, u, y, pc, s);
        case 3: return apply_n<3>(a, fp32, u, y, pc, s);
        case 4: return apply_n<4>(a, fp32, u, y, pc, s);
        case 5: return apply_n<5>(a, fp32, u, y, pc, s);
        case 6: return apply_n<6>(a, fp32, u, y, pc, s);
        case 7: return apply_n<7>(a, fp32, u, y, pc, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_ipdg_apply(const IpdgArgs& a, bool fp32, const double* u, double* y, cudaStream_t s) {
    ApplyPcg pc{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    return apply_dispatch(a, fp32, u, y, pc, s);
}

int pcg_max_grid(int K, int N, int sms) {
    (void)K;
    (void)N;
    return std::max(8 * sms, 1024);  // element kernels: up to 8 CTAs per SM; apply: 4; learned kernel: 608
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

// element-aligned launches, dispatched on the order
#define ROWS_DISPATCH(Np_, CALL)                         \
    switch (Np_) {                                       \
        case 3: { constexpr int NP = 3; CALL; } break;   \
        case 6: { constexpr int NP = 6; CALL; } break;   \
        case 10: { constexpr int NP = 10; CALL; } break; \
        case 15: { constexpr int NP = 15; CALL; } break; \
        case 21: { constexpr int NP = 21; CALL; } break; \
        case 28: { constexpr int NP = 28; CALL; } break; \
        case 36: { constexpr int NP = 36; CALL; } break; \
        default: return cudaErrorInvalidValue;           \
    }

template <int NP>
static int rows_grid(const IpdgArgs& a) {
    const int ngroups = (a.K + RowDims<NP>::EB - 1) / RowDims<NP>::EB;
    return std::max(1, std::min(ngroups, 8 * a.sms));  // 256 threads x 32 registers: 8 CTAs per SM
}

template <int NP>
static size_t grouped_size(int K) {
    const size_t ngroups = (K + RowDims<NP>::EB - 1) / RowDims<NP>::EB;
    return ngroups * NP * RowDims<NP>::EB * NP;
}

size_t grouped_blocks_size(int K, int Np) {
    switch (Np) {
        case 3: return grouped_size<3>(K);
        case 6: return grouped_size<6>(K);
        case 10: return grouped_size<10>(K);
        case 15: return grouped_size<15>(K);
        case 21: return grouped_size<21>(K);
        case 28: return grouped_size<28>(K);
        case 36: return grouped_size<36>(K);
        default: return 0;
    }
}

cudaError_t launch_group_blocks(const IpdgArgs& a, const double* blocks, double* P64, float* P32, cudaStream_t s) {
    ROWS_DISPATCH(a.Np, (group_blocks_kernel<NP><<<4 * a.sms, 256, 0, s>>>(blocks, P64, P32, a.K)));
    return cudaGetLastError();
}

// mode 0 init, 1 refresh; learned mode adds the learned kernel
static cudaError_t pcg_precondition(const IpdgArgs& a, const PcgVecs& v, const LpcNet* lpc, const LpcFeatArgs* fa,
                                    int mode, cudaStream_t s) {
    ROWS_DISPATCH(a.Np, (pcg_init_kernel<NP><<<rows_grid<NP>(a), RowDims<NP>::THREADS, 0, s>>>(v, a.K, mode)));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !v.zb) return e;
    const int lmode = mode == 0 ? LPC_PCG_INIT : LPC_PCG_REFRESH;
    if (v.mg && v.zl && lpc && lpc->sw) {
        // learned local stage into zl, then the coarse-space correction forms z
        e = launch_schwarz_local(*lpc->sw, v.r, v.r32, lpc->U, nullptr, s);
        if (e == cudaSuccess)
            e = launch_schwarz_collect(*lpc->sw, v.zb, lpc->U, nullptr, v.zl, v.dz, LPC_APPLY, v.S, v.part, s);
        if (e != cudaSuccess) return e;
        return launch_mg_correction(*v.mg, v.r, v.zl, v.z, v.dz, lmode, v.S, v.part, v.nmax, nullptr, s);
    }
    if (v.mg) return launch_mg_correction(*v.mg, v.r, v.zb, v.z, v.dz, lmode, v.S, v.part, v.nmax, nullptr, s);
    if (lpc->sw) {
        e = launch_schwarz_local(*lpc->sw, v.r, v.r32, lpc->U, nullptr, s);
        if (e != cudaSuccess) return e;
        return launch_schwarz_collect(*lpc->sw, v.zb, lpc->U, v.r, v.z, v.dz, lmode, v.S, v.part, s);
    }
    return launch_lpc_precond(*lpc, *fa, v.r, v.z, lmode, v.S, v.part, v.dz, s);
}

cudaError_t launch_pcg_init(const IpdgArgs& a, const PcgVecs& v, const LpcNet* lpc, const LpcFeatArgs* fa,
                            cudaStream_t s) {
    return pcg_precondition(a, v, lpc, fa, 0, s);
}

cudaError_t launch_pcg_refresh(const IpdgArgs& a, const PcgVecs& v, const LpcNet* lpc, const LpcFeatArgs* fa,
                               cudaStream_t s) {
    return pcg_precondition(a, v, lpc, fa, 1, s);
}

cudaError_t launch_pcg_iteration(const IpdgArgs& a, const PcgVecs& v, bool fp32, int parity, const LpcNet* lpc,
                                 const LpcFeatArgs* fa, cudaStream_t s) {
    ApplyPcg pc{v.p[parity], v.p[parity ^ 1], v.S, v.part, v.dz, v.dp[parity], v.dp[parity ^ 1]};
    cudaError_t e = apply_dispatch(a, fp32, v.z, v.Ap, pc, s);
    if (e != cudaSuccess) return e;
    ROWS_DISPATCH(a.Np,
                  (pcg_update_kernel<NP><<<rows_grid<NP>(a), RowDims<NP>::THREADS, 0, s>>>(v, a.K, parity)));
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (v.zb && v.mg && v.zl && lpc && lpc->sw) {
        e = launch_schwarz_local(*lpc->sw, v.r, v.r32, lpc->U, &v.S->done, s);
        if (e == cudaSuccess)
            e = launch_schwarz_collect(*lpc->sw, v.zb, lpc->U, nullptr, v.zl, v.dz, LPC_APPLY, v.S, v.part, s);
        if (e == cudaSuccess)
            e = launch_mg_correction(*v.mg, v.r, v.zl, v.z, v.dz, LPC_PCG_ITERATION, v.S, v.part, v.nmax, nullptr, s);
    } else if (v.zb && v.mg) {
        e = launch_mg_correction(*v.mg, v.r, v.zb, v.z, v.dz, LPC_PCG_ITERATION, v.S, v.part, v.nmax, nullptr, s);
    } else if (v.zb) {
        if (lpc->sw) {
            e = launch_schwarz_local(*lpc->sw, v.r, v.r32, lpc->U, &v.S->done, s);
            if (e == cudaSuccess)
                e = launch_schwarz_collect(*lpc->sw, v.zb, lpc->U, v.r, v.z, v.dz, LPC_PCG_ITERATION, v.S, v.part, s);
        } else {
            e = launch_lpc_precond(*lpc, *fa, v.r, v.z, LPC_PCG_ITERATION, v.S, v.part, v.dz, s);
        }
    }
    return e;
}

cudaError_t launch_bj(const IpdgArgs& a, const float* P32, const double* r, double* z, cudaStream_t s) {
    ROWS_DISPATCH(a.Np, (bj_kernel<NP><<<rows_grid<NP>(a), RowDims<NP>::THREADS, 0, s>>>(P32, r, z, a.K)));
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
