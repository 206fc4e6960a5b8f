// ipdg_tc.cu -- the SIPG apply of the FP32 PCG iterations on the tcgen05
// tensor cores (kind::tf32, 3-pass split products, FP32 accumulation in
// tensor memory), orders N <= 4 (sm_103a).
//
// Same operator, staging and outputs as ipdg_apply_kernel (ipdg.cu): per
// element the input offsets u (FP32 mirrors, p = z + beta p_old formed and
// written here), and for each face the neighbour's offsets read in its
// relabelled numbering (the shared face is its face 0, traversed in this
// element's direction), so that one set of face-0 tables serves every face.
// Tiles of 128 elements, one tensor-memory lane per element:
//
//   GEMM1  D1[e][n] = sum_p u[e][p] B1[n][p]   n: per face f the traces and
//          reference derivatives at its Gauss points (d/dr, d/ds, value;
//          8 columns each), then the volume parts Srr u, Srs2 u, Sss u and
//          the mass part Mr u (16 columns each)
//   GEMM2  D2_f[e][n] = sum_p nb_f[e][p] B2[n][p]  the neighbour's d/dr,
//          d/ds and value at the Gauss points of its face 0, per face f
//   combine (one thread per element and face): jump, average normal flux and
//          penalty give c1, c2r, c2s per Gauss point (SIMT, FP32)
//   GEMM3  D3[e][i] = sum_k c[e][k] B3[i][k]   the face terms lifted onto the
//          nodes: c2r Drf + c2s Dsf + c1 If
//   output y_i = J (c_rr Srr + c_rs Srs2 + c_ss Sss) u + alpha J M u + D3,
//          staged through shared memory for coalesced FP64 stores, and the
//          CTA's share of p.Ap for the PCG's grid-wide sum
//
// Each FP32 operand enters as TF32 hi + lo and each table as TF32 hi + lo
// (hi*hi + lo*hi + hi*lo), so the products carry FP32-level error, as the
// SIMT FP32 apply does.  Persistent CTAs of 256 threads, one per SM; every
// mbarrier wait is bounded and reports a timeout in the status word.
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/dgcu.h"
#include "dg_ctx.hpp"
#include "ipdg.hpp"
#include "pcg_reduce.cuh"
#include "umma.cuh"

namespace dgk {

namespace {

constexpr uint32_t kIpTcWait = 1u << 22;

template <int N>
struct IpTcDims {
    static constexpr int Np = (N + 1) * (N + 2) / 2, Nfp = N + 1, Nfq = N + 2, NB = 3 * N;
    static_assert(Np <= 16 && Nfq <= 8, "the tensor-core apply covers N <= 4");
    static constexpr int E = 128, THREADS = 256;
    static constexpr int KP = (Np + 7) / 8 * 8;  // GEMM1/2 K
    static constexpr int FB = 24;                // per face: [d/dr 8 | d/ds 8 | value 8]
    static constexpr int VOL = 3 * FB;           // volume blocks start (Srr, Srs2, Sss, Mr; 16 each)
    static constexpr int N1 = ((VOL + 4 * 16) + 15) / 16 * 16;
    static constexpr int N2 = 32;
    static constexpr int K3 = 3 * FB;            // lift operand: per face [c2r 8 | c2s 8 | c1 8]
    static constexpr int N3 = 16;
    static constexpr int COL2 = N1, COL3 = N1 + 3 * N2;
    static constexpr int TMEM_COLS = 256;
    static_assert(COL3 + N3 <= TMEM_COLS, "tensor memory layout");
    static constexpr int al(int x) { return (x + 1023) / 1024 * 1024; }
    static constexpr int SZ_B1 = 2 * N1 * KP * 4, SZ_B2 = 2 * N2 * KP * 4, SZ_B3 = 2 * N3 * K3 * 4;
    static constexpr int SZ_A1 = 2 * E * KP * 4, SZ_A3 = 2 * E * K3 * 4;
    static constexpr int OFF_B1 = 0;
    static constexpr int OFF_B2 = OFF_B1 + al(SZ_B1);
    static constexpr int OFF_B3 = OFF_B2 + al(SZ_B2);
    static constexpr int OFF_A1 = OFF_B3 + al(SZ_B3);
    static constexpr int OFF_A2 = OFF_A1 + al(SZ_A1);  // three faces
    static constexpr int A2_STRIDE = al(SZ_A1);
    static constexpr int OFF_A3 = OFF_A2 + 3 * A2_STRIDE;
    static constexpr int OFF_Y = OFF_A3 + al(SZ_A3);   // FP64 output rows (coalesced stores)
    static constexpr int OFF_PD = OFF_Y + E * Np * 8;   // FP64 first-node value per element
    static constexpr int OFF_DC = OFF_PD + E * 8;      // FP32 offset differences across faces
    static constexpr int OFF_CN = OFF_DC + E * 3 * 4;  // face links
    static constexpr int OFF_BAR = OFF_CN + E * 3 * 4;
    static constexpr int SMEM = OFF_BAR + 64;
    static_assert(SMEM <= 232448, "shared memory budget");
};

__device__ __forceinline__ void put_split(float* buf, uint32_t lo_floats, uint32_t off, float x) {
    float hi, lo;
    umma::split_tf32(x, hi, lo);
    buf[off] = hi;
    buf[off + lo_floats] = lo;
}

}  // namespace

template <int N>
__global__ void __launch_bounds__(256, 1) ipdg_apply_tc_kernel(IpdgArgs a, const double* __restrict__ u,
                                                              double* __restrict__ y, ApplyPcg pc) {
    using D = IpTcDims<N>;
    constexpr int Np = D::Np, Nfq = D::Nfq, E = D::E, KP = D::KP, FB = D::FB, K3 = D::K3;
    extern __shared__ __align__(1024) unsigned char smem[];
    if (pc.S && pc.S->done) return;
    float* sB1 = reinterpret_cast<float*>(smem + D::OFF_B1);
    float* sB2 = reinterpret_cast<float*>(smem + D::OFF_B2);
    float* sB3 = reinterpret_cast<float*>(smem + D::OFF_B3);
    float* sA1 = reinterpret_cast<float*>(smem + D::OFF_A1);
    float* sA3 = reinterpret_cast<float*>(smem + D::OFF_A3);
    double* sY = reinterpret_cast<double*>(smem + D::OFF_Y);
    double* sPD = reinterpret_cast<double*>(smem + D::OFF_PD);
    float* sDC = reinterpret_cast<float*>(smem + D::OFF_DC);
    int* sCN = reinterpret_cast<int*>(smem + D::OFF_CN);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + D::OFF_BAR);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
    auto sA2 = [&](int f) { return reinterpret_cast<float*>(smem + D::OFF_A2 + f * D::A2_STRIDE); };
    constexpr uint32_t LO_A = E * KP, LO_A3 = E * K3;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const double beta = pc.S ? pc.S->beta : 0.0;
    const bool has_beta = beta != 0.0;
    const float betaf = (float)beta;
    const double* __restrict__ p_old = pc.p_old;
    const float* __restrict__ dzv = pc.dz;
    const float* __restrict__ dpo = pc.dp_old;
    const IpdgOps<float>& o = a.o32;
    const int ntiles = (a.K + E - 1) / E;

    // constant operands, zero operand buffers (padding columns stay zero)
    {
        const int4* src = reinterpret_cast<const int4*>(a.tc_b);
        int4* dst = reinterpret_cast<int4*>(smem + D::OFF_B1);
        for (int i = tid; i < D::SZ_B1 / 16; i += blockDim.x) dst[i] = src[i];
        src += D::SZ_B1 / 16;
        dst = reinterpret_cast<int4*>(smem + D::OFF_B2);
        for (int i = tid; i < D::SZ_B2 / 16; i += blockDim.x) dst[i] = src[i];
        src += D::SZ_B2 / 16;
        dst = reinterpret_cast<int4*>(smem + D::OFF_B3);
        for (int i = tid; i < D::SZ_B3 / 16; i += blockDim.x) dst[i] = src[i];
        float* z0 = reinterpret_cast<float*>(smem + D::OFF_A1);
        const int nz = (D::OFF_Y - D::OFF_A1) / 4;
        for (int i = tid; i < nz; i += blockDim.x) z0[i] = 0.f;
    }
    if (tid == 0) {
        umma::mbar_init(bar, 1);
        umma::fence_mbar_init();
    }
    if (warp == 0) {
        umma::tmem_alloc(tmem_slot, D::TMEM_COLS);
        umma::tmem_relinquish();
    }
    umma::fence_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const uint32_t aB1 = umma::smem_u32(sB1), aB2 = umma::smem_u32(sB2), aB3 = umma::smem_u32(sB3);
    const uint32_t aA1 = umma::smem_u32(sA1), aA3 = umma::smem_u32(sA3);
    const uint32_t aA2 = umma::smem_u32(smem + D::OFF_A2);
    const uint32_t id1 = umma::idesc_tf32(128, D::N1), id2 = umma::idesc_tf32(128, D::N2),
                   id3 = umma::idesc_tf32(128, D::N3);
    constexpr uint32_t SBO = (KP / 4) * 128, SBO3 = (K3 / 4) * 128;
    constexpr uint32_t LOB1 = D::N1 * KP * 4, LOB2 = D::N2 * KP * 4, LOB3 = D::N3 * K3 * 4;
    uint32_t ph = 0;
    bool failed = false, pend = false;
    const int qd = warp & 3, half = warp >> 2;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * qd) << 16);
    double dot = 0.0;

    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const int k0 = tile * E, ne = min(E, a.K - k0);
        const size_t g0 = (size_t)k0 * Np;
        // ---- staging: own input (p = z + beta p_old written out; FP32 offsets)
        for (int t = tid; t < ne * Np; t += blockDim.x) {
            const int e = t / Np, p = t - e * Np;
            const size_t i = g0 + t;
            const double vp = has_beta ? fma(beta, p_old[i], u[i]) : u[i];
            if (pc.p_new) pc.p_new[i] = vp;
            if (p == 0) sPD[e] = vp;
            float d = dzv[i];
            if (has_beta) d = fmaf(betaf, dpo[i], d);
            pc.dp_new[i] = d;
            put_split(sA1, LO_A, umma::kmajor_offset(e, p, KP) >> 2, d);
        }
        for (int t = tid; t < ne * 3; t += blockDim.x) sCN[t] = a.conn[(size_t)k0 * 3 + t];
        __syncthreads();
        // neighbours in their relabelled numbering, and the FP64 offset differences
        for (int t = tid; t < ne * 3 * Np; t += blockDim.x) {
            const int e = t / (3 * Np), rem = t - e * 3 * Np, f = rem / Np, p = rem - f * Np;
            const int c = sCN[e * 3 + f];
            float d = 0.f;
            if (c >= 0) {
                const size_t j = (size_t)(c >> 3) * Np + a.nperm[2 * (c & 3) + ((c >> 2) & 1)][p];
                d = dzv[j];
                if (has_beta) d = fmaf(betaf, dpo[j], d);
            }
            put_split(sA2(f), LO_A, umma::kmajor_offset(e, p, KP) >> 2, d);
        }
        for (int t = tid; t < ne * 3; t += blockDim.x) {
            const int c = sCN[t];
            float dcv = 0.f;
            if (c >= 0) {
                const size_t j = (size_t)(c >> 3) * Np;
                dcv = (float)(sPD[t / 3] - (has_beta ? fma(beta, p_old[j], u[j]) : u[j]));
            }
            sDC[t] = dcv;
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        // ---- GEMM1 and the three GEMM2s
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < KP / 8; s++) {
                const uint64_t bh = umma::smem_desc(aB1 + s * 256, 128, SBO), bl = umma::smem_desc(aB1 + LOB1 + s * 256, 128, SBO);
                const uint64_t ah = umma::smem_desc(aA1 + s * 256, 128, SBO), al = umma::smem_desc(aA1 + LO_A * 4 + s * 256, 128, SBO);
                umma::mma_tf32(tmem, ah, bh, id1, s > 0);
                umma::mma_tf32(tmem, al, bh, id1, 1);
                umma::mma_tf32(tmem, ah, bl, id1, 1);
            }
#pragma unroll
            for (int f = 0; f < 3; f++) {
                const uint32_t aF = aA2 + f * D::A2_STRIDE;
#pragma unroll
                for (int s = 0; s < KP / 8; s++) {
                    const uint64_t bh = umma::smem_desc(aB2 + s * 256, 128, SBO), bl = umma::smem_desc(aB2 + LOB2 + s * 256, 128, SBO);
                    const uint64_t ah = umma::smem_desc(aF + s * 256, 128, SBO), al = umma::smem_desc(aF + LO_A * 4 + s * 256, 128, SBO);
                    const uint32_t dcol = tmem + D::COL2 + f * D::N2;
                    umma::mma_tf32(dcol, ah, bh, id2, s > 0);
                    umma::mma_tf32(dcol, al, bh, id2, 1);
                    umma::mma_tf32(dcol, ah, bl, id2, 1);
                }
            }
            umma::commit(bar);
            pend = true;
        }
        {
            const bool ok = umma::mbar_wait(bar, ph, kIpTcWait);
            ph ^= 1;
            if (tid == 0 && ok) pend = false;
            if (__syncthreads_or(!ok)) { failed = true; break; }
        }
        umma::fence_after_sync();
        // ---- combine: one thread per (element, face); warps of half 0 take faces 0, 2, half 1 face 1
        {
            const int e = 32 * qd + lane;
            const bool act = e < ne;
            const int k = k0 + (act ? e : 0);
            const float ub0 = (float)sPD[act ? e : 0];
            for (int f = half; f < 3; f += 2) {
                float ur[8], us_[8], um[8], vr[8], vs[8], up[8];
                umma::tmem_ld8(lane_base + f * FB, ur);
                umma::tmem_ld8(lane_base + f * FB + 8, us_);
                umma::tmem_ld8(lane_base + f * FB + 16, um);
                umma::tmem_ld8(lane_base + D::COL2 + f * D::N2, vr);
                umma::tmem_ld8(lane_base + D::COL2 + f * D::N2 + 8, vs);
                umma::tmem_ld8(lane_base + D::COL2 + f * D::N2 + 16, up);
                umma::tmem_ld_wait();
                if (act) {
                    const float2* fcp = reinterpret_cast<const float2*>(a.fcl + ((size_t)k * 3 + f) * kFaceCoef);
                    const float2 f01 = fcp[0], f23 = fcp[1], f45 = fcp[2];
                    const bool interior = sCN[e * 3 + f] >= 0;
                    const float dc = sDC[e * 3 + f];
#pragma unroll
                    for (int g = 0; g < Nfq; g++) {
                        const float dm = f01.x * ur[g] + f01.y * us_[g];
                        float jump, dp;
                        if (interior) {
                            dp = f23.x * vr[g] + f23.y * vs[g];
                            jump = (um[g] - up[g]) + dc;
                        } else {
                            jump = 2.f * (um[g] + ub0);  // Dirichlet face: u+ = -u-
                            dp = dm;
                        }
                        const float wJ = f45.y * o.fw[g];
                        const float sigma = 0.5f * (dm + dp);
                        const float cc2 = -0.5f * wJ * jump;
                        put_split(sA3, LO_A3, umma::kmajor_offset(e, f * FB + g, K3) >> 2, cc2 * f01.x);
                        put_split(sA3, LO_A3, umma::kmajor_offset(e, f * FB + 8 + g, K3) >> 2, cc2 * f01.y);
                        put_split(sA3, LO_A3, umma::kmajor_offset(e, f * FB + 16 + g, K3) >> 2,
                                  wJ * (f45.x * jump - sigma));
                    }
                }
            }
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        // ---- GEMM3: the face terms lifted onto the nodes
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < K3 / 8; s++) {
                const uint64_t bh = umma::smem_desc(aB3 + s * 256, 128, SBO3), bl = umma::smem_desc(aB3 + LOB3 + s * 256, 128, SBO3);
                const uint64_t ah = umma::smem_desc(aA3 + s * 256, 128, SBO3), al = umma::smem_desc(aA3 + LO_A3 * 4 + s * 256, 128, SBO3);
                umma::mma_tf32(tmem + D::COL3, ah, bh, id3, s > 0);
                umma::mma_tf32(tmem + D::COL3, al, bh, id3, 1);
                umma::mma_tf32(tmem + D::COL3, ah, bl, id3, 1);
            }
            umma::commit(bar);
            pend = true;
        }
        {
            const bool ok = umma::mbar_wait(bar, ph, kIpTcWait);
            ph ^= 1;
            if (tid == 0 && ok) pend = false;
            if (__syncthreads_or(!ok)) { failed = true; break; }
        }
        umma::fence_after_sync();
        // ---- outputs: rows 8 half .. 8 half + 7 of each element into shared memory
        {
            const int e = 32 * qd + lane;
            const bool act = e < ne;
            const int k = k0 + (act ? e : 0);
            float A[8], B[8], C[8], M[8], Lf[8];
            const int c0 = 8 * half;
            umma::tmem_ld8(lane_base + D::VOL + c0, A);
            umma::tmem_ld8(lane_base + D::VOL + 16 + c0, B);
            umma::tmem_ld8(lane_base + D::VOL + 32 + c0, C);
            umma::tmem_ld8(lane_base + D::VOL + 48 + c0, M);
            umma::tmem_ld8(lane_base + D::COL3 + c0, Lf);
            umma::tmem_ld_wait();
            if (act) {
                const float vrr = o.vc[(size_t)k * 3], vrs = o.vc[(size_t)k * 3 + 1], vss = o.vc[(size_t)k * 3 + 2];
                const bool mass = a.mass_coef != 0.0;
                const float mc = mass ? (float)(a.mass_coef * a.J[k]) : 0.f;
                const float ub0 = (float)sPD[e];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int i = c0 + j;
                    if (i < Np) {
                        float v = vrr * A[j] + vrs * B[j] + vss * C[j] + Lf[j];
                        if (mass) v = fmaf(mc, fmaf(o.mrow[i], ub0, M[j]), v);
                        sY[e * Np + i] = (double)v;
                    }
                }
            }
        }
        umma::fence_before_sync();
        __syncthreads();
        // coalesced FP64 stores and this CTA's share of p.Ap
        for (int t = tid; t < ne * Np; t += blockDim.x) {
            const double v = sY[t];
            y[g0 + t] = v;
            const double pv = pc.p_new ? pc.p_new[g0 + t] : (has_beta ? fma(beta, p_old[g0 + t], u[g0 + t]) : u[g0 + t]);
            dot += v * pv;
        }
        __syncthreads();  // sY and the operands are rewritten by the next tile
    }
    if (failed && tid == 0 && a.tc_status) atomicExch(a.tc_status, 1);
    if (tid == 0 && pend) umma::mbar_wait(bar, ph, kIpTcWait);  // MMAs in flight after a timeout
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, D::TMEM_COLS);
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

// ---------------------------------------------------------------------------
// host: operand images and launch

static inline float tf32_rna_host(float x) {
    uint32_t v;
    memcpy(&v, &x, 4);
    v = (v + 0x1000u) & 0xFFFFE000u;
    float r;
    memcpy(&r, &v, 4);
    return r;
}

// canonical K-major image (hi part, then lo part) of a rows x KP operand
template <typename F>
static void tc_image(int rows, int KP, F f, std::vector<float>& out) {
    std::vector<float> img((size_t)2 * rows * KP, 0.f);
    const size_t lo = (size_t)rows * KP;
    for (int r = 0; r < rows; r++)
        for (int k = 0; k < KP; k++) {
            const double x = f(r, k);
            const float hi = tf32_rna_host((float)x);
            const size_t off = umma::kmajor_offset(r, k, KP) >> 2;
            img[off] = hi;
            img[lo + off] = (float)(x - (double)hi);
        }
    out.insert(out.end(), img.begin(), img.end());
}

template <int N>
static std::vector<float> tc_images_n(const std::vector<double>& DrfT, const std::vector<double>& DsfT,
                                      const std::vector<double>& If, const std::vector<double>& Srr,
                                      const std::vector<double>& Srs2, const std::vector<double>& Sss,
                                      const std::vector<double>& Mr) {
    using D = IpTcDims<N>;
    constexpr int Np = D::Np, Nfp = D::Nfp, Nfq = D::Nfq, NB = D::NB, NF = 3 * Nfq, FB = D::FB, KP = D::KP;
    // value of basis function p at face f's Gauss point g (face f's nodes are ring positions (f N + j) mod 3N)
    auto trace = [&](int f, int g, int p) {
        for (int j = 0; j < Nfp; j++)
            if ((f * N + j) % NB == p) return If[(size_t)g * Nfp + j];
        return 0.0;
    };
    std::vector<float> out;
    tc_image(D::N1, KP, [&](int n, int p) -> double {
        if (p >= Np) return 0.0;
        if (n < D::VOL) {
            const int f = n / FB, w = n % FB, q = w / 8, g = w % 8;
            if (g >= Nfq) return 0.0;
            if (q == 0) return DrfT[(size_t)p * NF + f * Nfq + g];
            if (q == 1) return DsfT[(size_t)p * NF + f * Nfq + g];
            return trace(f, g, p);
        }
        const int blk = (n - D::VOL) / 16, i = (n - D::VOL) % 16;
        if (blk >= 4 || i >= Np) return 0.0;
        const std::vector<double>& S = blk == 0 ? Srr : blk == 1 ? Srs2 : blk == 2 ? Sss : Mr;
        return S[(size_t)i * Np + p];
    }, out);
    tc_image(D::N2, KP, [&](int n, int p) -> double {
        if (p >= Np || n >= FB) return 0.0;
        const int q = n / 8, g = n % 8;
        if (g >= Nfq) return 0.0;
        if (q == 0) return DrfT[(size_t)p * NF + g];
        if (q == 1) return DsfT[(size_t)p * NF + g];
        return trace(0, g, p);
    }, out);
    tc_image(D::N3, D::K3, [&](int i, int kk) -> double {
        if (i >= Np) return 0.0;
        const int f = kk / FB, w = kk % FB, q = w / 8, g = w % 8;
        if (g >= Nfq) return 0.0;
        if (q == 0) return DrfT[(size_t)i * NF + f * Nfq + g];
        if (q == 1) return DsfT[(size_t)i * NF + f * Nfq + g];
        return trace(f, g, i);
    }, out);
    return out;
}

std::vector<float> ipdg_tc_images(int N, const std::vector<double>& DrfT, const std::vector<double>& DsfT,
                                  const std::vector<double>& If, const std::vector<double>& Srr,
                                  const std::vector<double>& Srs2, const std::vector<double>& Sss,
                                  const std::vector<double>& Mr) {
    switch (N) {
        case 1: return tc_images_n<1>(DrfT, DsfT, If, Srr, Srs2, Sss, Mr);
        case 2: return tc_images_n<2>(DrfT, DsfT, If, Srr, Srs2, Sss, Mr);
        case 3: return tc_images_n<3>(DrfT, DsfT, If, Srr, Srs2, Sss, Mr);
        case 4: return tc_images_n<4>(DrfT, DsfT, If, Srr, Srs2, Sss, Mr);
        default: return {};
    }
}

template <int N>
static cudaError_t launch_tc_n(const IpdgArgs& a, const double* u, double* y, const ApplyPcg& pc, cudaStream_t s) {
    using D = IpTcDims<N>;
    const int ntiles = (a.K + D::E - 1) / D::E;
    const int grid = std::max(1, std::min(ntiles, a.sms));
    ipdg_apply_tc_kernel<N><<<grid, D::THREADS, D::SMEM, s>>>(a, u, y, pc);
    return cudaGetLastError();
}

// shared-memory opt-in, on the current device (dg_ipdg_setup)
cudaError_t setup_ipdg_tc(int N) {
    switch (N) {
        case 1: return cudaFuncSetAttribute(ipdg_apply_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, IpTcDims<1>::SMEM);
        case 2: return cudaFuncSetAttribute(ipdg_apply_tc_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, IpTcDims<2>::SMEM);
        case 3: return cudaFuncSetAttribute(ipdg_apply_tc_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, IpTcDims<3>::SMEM);
        case 4: return cudaFuncSetAttribute(ipdg_apply_tc_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, IpTcDims<4>::SMEM);
        default: return cudaErrorNotSupported;
    }
}

cudaError_t launch_ipdg_apply_tc(const IpdgArgs& a, const double* u, double* y, const ApplyPcg& pc, cudaStream_t s) {
    switch (a.N) {
        case 1: return launch_tc_n<1>(a, u, y, pc, s);
        case 2: return launch_tc_n<2>(a, u, y, pc, s);
        case 3: return launch_tc_n<3>(a, u, y, pc, s);
        case 4: return launch_tc_n<4>(a, u, y, pc, s);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace dgk
