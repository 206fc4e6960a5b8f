// schwarz_mlp.cu -- tensor-core (tcgen05, kind::f16 with BF16 operands) kernels of
// the two-layer learned additive-Schwarz preconditioner
//
//   M r = P r + sum_m G_m^T W^T act(W G_m r),   W: 128 x F (F = 4 Np), BF16,
//   act(h) = max(h, slope h), slope in [0, 1] (0: relu)
//
// G_m gathers the residual on element m and on its three face neighbours
// (each rotated so that the shared face is its face 0).  The two layers share
// W (tied weights), so every term satisfies (G_m r) . W^T act(W G_m r) =
// sum_j h_j act(h_j) >= 0: r . M(r) > 0 for every r != 0, and the flexible
// PCG's step lengths stay positive.
//
// Local stage (inference and the training forward pass), tiles of 128
// patches, one TMEM lane row per patch:
//   GEMM1  Hd[128][128] = X[128][KP] . W^T       (X as BF16 hi + lo: two passes)
//   GEMM2  U[128][KP]   = act(Hd)[128][128] . W  (act(Hd) as BF16 hi + lo)
// Weight gradient of the energy loss (training), per tile:
//   P  = X . W^T, then P = A . W^T in the same TMEM columns (X = G r, A = G g)
//   Gw[128][KP] += h^T . A + (D (W a))^T . X     (h = act(X W^T), D = act')
// with X, A, h and D W a rounded to BF16 once, FP32 accumulation over every
// patch of the CTA in TMEM; one partial per CTA, summed by a second kernel.
// Operands use the canonical no-swizzle K-major layout of umma.cuh.  Every
// mbarrier wait is bounded and reports a timeout in *status.
#include <cuda_bf16.h>

#include "lpc.hpp"
#include "umma.cuh"

namespace dgk {

namespace {

constexpr uint32_t kMlpWaitLimit = 1u << 22;

template <int NP>
struct MlpDims {
    static constexpr int H = kSchwarzMlpH;
    static constexpr int F = 4 * NP;
    static constexpr int KP = (F + 15) / 16 * 16;  // GEMM1 K, GEMM2 N, gradient N
    static constexpr int al(int x) { return (x + 1023) / 1024 * 1024; }
    static constexpr int SZ_W1 = H * KP * 2;  // W as the B operand of X W^T: rows j, K = feature
    static constexpr int SZ_W2 = KP * H * 2;  // W^T as the B operand of h W: rows i, K = hidden
    static constexpr int SZ_X = 2 * 128 * KP * 2;
    static constexpr int SZ_H = 2 * 128 * H * 2;
    static constexpr int OFF_W1 = 0;
    static constexpr int OFF_W2 = OFF_W1 + al(SZ_W1);
    static constexpr int OFF_X = OFF_W2 + al(SZ_W2);
    static constexpr int OFF_H = OFF_X + al(SZ_X);
    static constexpr int OFF_BAR = OFF_H + al(SZ_H);
    static constexpr int SMEM = OFF_BAR + 64;
    static_assert(128 * F * 4 <= SZ_H, "the U rows are staged in the hidden-layer buffer");
    static_assert(SMEM <= 232448, "shared memory budget");
    // weight gradient
    static constexpr int SZ_ROWS = 128 * KP * 2;  // X or A rows (A operand of P = . W^T)
    static constexpr int SZ_HT = H * 128 * 2;     // h^T or (D W a)^T: rows j, K = patch
    static constexpr int SZ_CT = KP * 128 * 2;    // A^T or X^T: rows i, K = patch
    static constexpr int G_W1 = 0;
    static constexpr int G_XA = G_W1 + al(SZ_W1);
    static constexpr int G_AA = G_XA + al(SZ_ROWS);
    static constexpr int G_HT = G_AA + al(SZ_ROWS);
    static constexpr int G_BT = G_HT + al(SZ_HT);
    static constexpr int G_AT = G_BT + al(SZ_HT);
    static constexpr int G_XT = G_AT + al(SZ_CT);
    static constexpr int G_BAR = G_XT + al(SZ_CT);
    static constexpr int GSMEM = G_BAR + 64;
    static_assert(GSMEM <= 232448, "shared memory budget");
    static constexpr int TMEM_COLS = 256;  // 128 hidden columns + KP <= 112 output columns
};

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo_half, __nv_bfloat16 hi_half) {
    __nv_bfloat162 v = __halves2bfloat162(lo_half, hi_half);
    return *reinterpret_cast<uint32_t*>(&v);
}

// the residual patch of element m (own block, then the three rotated
// neighbour blocks; zero across a boundary) as FP32
template <int NP>
__device__ __forceinline__ void mlp_gather(const SchwarzArgs& a, const float* __restrict__ v32,
                                           const double* __restrict__ v, int m, bool act, float* x) {
    if (!act) {
#pragma unroll
        for (int i = 0; i < 4 * NP; i++) x[i] = 0.f;
        return;
    }
    if (v32) {
        const float* vm = v32 + (size_t)m * NP;
#pragma unroll
        for (int i = 0; i < NP; i++) x[i] = vm[i];
    } else {
        const double* vm = v + (size_t)m * NP;
#pragma unroll
        for (int i = 0; i < NP; i++) x[i] = (float)vm[i];
    }
#pragma unroll
    for (int f = 0; f < 3; f++) {
        const int c = a.conn[(size_t)m * 3 + f];
        const int* pm = a.perm + (c & 3) * NP;
        const size_t nb = (size_t)(c >= 0 ? (c >> 3) : 0) * NP;
#pragma unroll
        for (int i = 0; i < NP; i++) {
            float val = 0.f;
            if (c >= 0) val = v32 ? v32[nb + pm[i]] : (float)v[nb + pm[i]];
            x[(f + 1) * NP + i] = val;
        }
    }
}

// BF16 images of W for the two B operands (zero padding beyond F)
template <int NP>
__device__ __forceinline__ void mlp_stage_weights(const __nv_bfloat16* __restrict__ W, unsigned char* sW1,
                                                  unsigned char* sW2) {
    using D = MlpDims<NP>;
    constexpr int H = D::H, F = D::F, KP = D::KP;
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int t = threadIdx.x; t < H * KP; t += blockDim.x) {
        const int j = t / KP, i = t - j * KP;
        *reinterpret_cast<__nv_bfloat16*>(sW1 + umma::kmajor_offset_b16(j, i, KP)) = i < F ? W[j * F + i] : zero;
    }
    if (sW2)
        for (int t = threadIdx.x; t < KP * H; t += blockDim.x) {
            const int i = t / H, j = t - i * H;
            *reinterpret_cast<__nv_bfloat16*>(sW2 + umma::kmajor_offset_b16(i, j, H)) = i < F ? W[j * F + i] : zero;
        }
}

}  // namespace

template <int NP>
__global__ void __launch_bounds__(128, 1) schwarz_mlp_local_kernel(SchwarzArgs a, const float* __restrict__ r32,
                                                                   const double* __restrict__ r,
                                                                   float* __restrict__ U, const int* __restrict__ done,
                                                                   int* status) {
    using D = MlpDims<NP>;
    constexpr int H = D::H, F = D::F, KP = D::KP;
    extern __shared__ __align__(1024) unsigned char smem[];
    if (done && *done) return;
    unsigned char* sW1 = smem + D::OFF_W1;
    unsigned char* sW2 = smem + D::OFF_W2;
    unsigned char* sX = smem + D::OFF_X;
    unsigned char* sH = smem + D::OFF_H;
    uint64_t* bar1 = reinterpret_cast<uint64_t*>(smem + D::OFF_BAR);
    uint64_t* bar2 = bar1 + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar1 + 2);
    const int tid = threadIdx.x, warp = tid >> 5;

    const float slope = a.slope;
    mlp_stage_weights<NP>(a.W, sW1, sW2);
    if (tid == 0) {
        umma::mbar_init(bar1, 1);
        umma::mbar_init(bar2, 1);
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
    const uint32_t tD1 = tmem, tD2 = tmem + H;
    const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
    const uint32_t idesc1 = umma::idesc_bf16(128, H);
    const uint32_t idesc2 = umma::idesc_bf16(128, KP);
    const uint32_t aW1 = umma::smem_u32(sW1), aW2 = umma::smem_u32(sW2);
    const uint32_t aX = umma::smem_u32(sX), aH = umma::smem_u32(sH);
    constexpr uint32_t LOX = 128 * KP * 2, LOH = 128 * H * 2;
    constexpr uint32_t SBO1 = (KP / 8) * 128, SBO2 = (H / 8) * 128;
    uint32_t ph = 0;
    bool failed = false;
    const int ntiles = (a.K + 127) / 128;

    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const int m = tile * 128 + tid;
        // (1) X row of patch m as BF16 hi + lo
        {
            float x[F];
            mlp_gather<NP>(a, r32, r, m, m < a.K, x);
#pragma unroll
            for (int i8 = 0; i8 < KP / 8; i8++) {
                uint32_t hw[4], lw[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int i0 = i8 * 8 + 2 * q;
                    const float x0 = i0 < F ? x[i0] : 0.f, x1 = i0 + 1 < F ? x[i0 + 1] : 0.f;
                    const __nv_bfloat16 h0 = __float2bfloat16(x0), h1 = __float2bfloat16(x1);
                    hw[q] = pack_bf16(h0, h1);
                    lw[q] = pack_bf16(__float2bfloat16(x0 - __bfloat162float(h0)),
                                      __float2bfloat16(x1 - __bfloat162float(h1)));
                }
                const uint32_t off = umma::kmajor_offset_b16(tid, i8 * 8, KP);
                *reinterpret_cast<uint4*>(sX + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4*>(sX + LOX + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < KP / 16; s++) {
                const uint64_t ah = umma::smem_desc(aX + s * 256, 128, SBO1);
                const uint64_t al = umma::smem_desc(aX + LOX + s * 256, 128, SBO1);
                const uint64_t b = umma::smem_desc(aW1 + s * 256, 128, SBO1);
                umma::mma_bf16(tD1, ah, b, idesc1, s > 0);
                umma::mma_bf16(tD1, al, b, idesc1, 1);
            }
            umma::commit(bar1);
        }
        bool ok = umma::mbar_wait(bar1, ph, kMlpWaitLimit);
        if (__syncthreads_or(!ok)) { failed = true; break; }
        umma::fence_after_sync();
        // (2) act(Hd) row as BF16 hi + lo
#pragma unroll 2
        for (int c8 = 0; c8 < H / 8; c8++) {
            float h[8];
            umma::tmem_ld8(tD1 + lane_base + c8 * 8, h);
            umma::tmem_ld_wait();
            uint32_t hw[4], lw[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float v0 = fmaxf(h[2 * q], slope * h[2 * q]), v1 = fmaxf(h[2 * q + 1], slope * h[2 * q + 1]);
                const __nv_bfloat16 h0 = __float2bfloat16(v0), h1 = __float2bfloat16(v1);
                hw[q] = pack_bf16(h0, h1);
                lw[q] = pack_bf16(__float2bfloat16(v0 - __bfloat162float(h0)),
                                  __float2bfloat16(v1 - __bfloat162float(h1)));
            }
            const uint32_t off = umma::kmajor_offset_b16(tid, c8 * 8, H);
            *reinterpret_cast<uint4*>(sH + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
            *reinterpret_cast<uint4*>(sH + LOH + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < H / 16; s++) {
                const uint64_t ah = umma::smem_desc(aH + s * 256, 128, SBO2);
                const uint64_t al = umma::smem_desc(aH + LOH + s * 256, 128, SBO2);
                const uint64_t b = umma::smem_desc(aW2 + s * 256, 128, SBO2);
                umma::mma_bf16(tD2, ah, b, idesc2, s > 0);
                umma::mma_bf16(tD2, al, b, idesc2, 1);
            }
            umma::commit(bar2);
        }
        ok = umma::mbar_wait(bar2, ph, kMlpWaitLimit);
        ph ^= 1;
        if (__syncthreads_or(!ok)) { failed = true; break; }
        umma::fence_after_sync();
        // (3) U rows: TMEM -> shared memory (the hidden buffer is free: GEMM2 has
        //     completed) -> coalesced float4 stores of the tile's contiguous rows
        float* sU = reinterpret_cast<float*>(sH);  // 128 x F floats, row-major
#pragma unroll
        for (int c8 = 0; c8 < KP / 8; c8++) {
            float u[8];
            umma::tmem_ld8(tD2 + lane_base + c8 * 8, u);
            umma::tmem_ld_wait();
#pragma unroll
            for (int q4 = 0; q4 < 2; q4++)
                if (c8 * 8 + 4 * q4 < F)
                    *reinterpret_cast<float4*>(sU + tid * F + c8 * 8 + 4 * q4) =
                        make_float4(u[4 * q4], u[4 * q4 + 1], u[4 * q4 + 2], u[4 * q4 + 3]);
        }
        umma::fence_before_sync();
        __syncthreads();
        {
            const int rows = min(128, a.K - tile * 128);
            const float4* src = reinterpret_cast<const float4*>(sU);
            float4* dst = reinterpret_cast<float4*>(U + (size_t)tile * 128 * F);  // F % 4 == 0: 16-byte aligned
            for (int t = tid; t < rows * F / 4; t += blockDim.x) dst[t] = src[t];
        }
        __syncthreads();  // X and the hidden buffer are rewritten by the next tile
    }
    if (failed && tid == 0) atomicExch(status, 1);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, D::TMEM_COLS);
}

template <int NP>
__global__ void __launch_bounds__(128, 1) schwarz_mlp_wgrad_kernel(SchwarzArgs a, const double* __restrict__ r,
                                                                   const double* __restrict__ g,
                                                                   float* __restrict__ part, int* status) {
    using D = MlpDims<NP>;
    constexpr int H = D::H, F = D::F, KP = D::KP;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sW1 = smem + D::G_W1;
    unsigned char* sXA = smem + D::G_XA;
    unsigned char* sAA = smem + D::G_AA;
    unsigned char* sHT = smem + D::G_HT;
    unsigned char* sBT = smem + D::G_BT;
    unsigned char* sAT = smem + D::G_AT;
    unsigned char* sXT = smem + D::G_XT;
    uint64_t* bar1 = reinterpret_cast<uint64_t*>(smem + D::G_BAR);
    uint64_t* bar2 = bar1 + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar1 + 2);
    const int tid = threadIdx.x, warp = tid >> 5;

    const float slope = a.slope;
    mlp_stage_weights<NP>(a.W, sW1, nullptr);
    if (tid == 0) {
        umma::mbar_init(bar1, 1);
        umma::mbar_init(bar2, 1);
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
    const uint32_t tP = tmem, tG = tmem + H;
    const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
    const uint32_t idescP = umma::idesc_bf16(128, H);
    const uint32_t idescG = umma::idesc_bf16(128, KP);
    const uint32_t aW1 = umma::smem_u32(sW1), aXA = umma::smem_u32(sXA), aAA = umma::smem_u32(sAA);
    const uint32_t aHT = umma::smem_u32(sHT), aBT = umma::smem_u32(sBT);
    const uint32_t aAT = umma::smem_u32(sAT), aXT = umma::smem_u32(sXT);
    constexpr uint32_t SBO1 = (KP / 8) * 128, SBOT = (128 / 8) * 128;
    uint32_t ph1 = 0, ph2 = 0;
    bool failed = false, any = false;
    const int ntiles = (a.K + 127) / 128;

    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        if (any) {  // the previous tile's gradient MMAs read the transposed operands
            const bool ok = umma::mbar_wait(bar2, ph2, kMlpWaitLimit);
            ph2 ^= 1;
            if (__syncthreads_or(!ok)) { failed = true; break; }
            umma::fence_after_sync();
        }
        const int m = tile * 128 + tid;
        // (1) x = G_m r and a = G_m g, rounded to BF16: rows for P, columns for Gw
        {
            float x[F], av[F];
            mlp_gather<NP>(a, nullptr, r, m, m < a.K, x);
            mlp_gather<NP>(a, nullptr, g, m, m < a.K, av);
#pragma unroll
            for (int i8 = 0; i8 < KP / 8; i8++) {
                uint32_t xw[4], aw[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int i0 = i8 * 8 + 2 * q;
                    const __nv_bfloat16 x0 = __float2bfloat16(i0 < F ? x[i0] : 0.f);
                    const __nv_bfloat16 x1 = __float2bfloat16(i0 + 1 < F ? x[i0 + 1] : 0.f);
                    const __nv_bfloat16 a0 = __float2bfloat16(i0 < F ? av[i0] : 0.f);
                    const __nv_bfloat16 a1 = __float2bfloat16(i0 + 1 < F ? av[i0 + 1] : 0.f);
                    xw[q] = pack_bf16(x0, x1);
                    aw[q] = pack_bf16(a0, a1);
                    *reinterpret_cast<__nv_bfloat16*>(sXT + umma::kmajor_offset_b16(i0, tid, 128)) = x0;
                    *reinterpret_cast<__nv_bfloat16*>(sXT + umma::kmajor_offset_b16(i0 + 1, tid, 128)) = x1;
                    *reinterpret_cast<__nv_bfloat16*>(sAT + umma::kmajor_offset_b16(i0, tid, 128)) = a0;
                    *reinterpret_cast<__nv_bfloat16*>(sAT + umma::kmajor_offset_b16(i0 + 1, tid, 128)) = a1;
                }
                const uint32_t off = umma::kmajor_offset_b16(tid, i8 * 8, KP);
                *reinterpret_cast<uint4*>(sXA + off) = make_uint4(xw[0], xw[1], xw[2], xw[3]);
                *reinterpret_cast<uint4*>(sAA + off) = make_uint4(aw[0], aw[1], aw[2], aw[3]);
            }
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        // (2) P = X W^T -> h = act(P) (column tid of h^T) and the mask bits P > 0
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < KP / 16; s++)
                umma::mma_bf16(tP, umma::smem_desc(aXA + s * 256, 128, SBO1), umma::smem_desc(aW1 + s * 256, 128, SBO1),
                               idescP, s > 0);
            umma::commit(bar1);
        }
        bool ok = umma::mbar_wait(bar1, ph1, kMlpWaitLimit);
        ph1 ^= 1;
        if (__syncthreads_or(!ok)) { failed = true; break; }
        umma::fence_after_sync();
        uint32_t mask[H / 32];
#pragma unroll
        for (int w = 0; w < H / 32; w++) mask[w] = 0u;
#pragma unroll
        for (int c8 = 0; c8 < H / 8; c8++) {
            float v[8];
            umma::tmem_ld8(tP + lane_base + c8 * 8, v);
            umma::tmem_ld_wait();
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int j = c8 * 8 + q;
                if (v[q] > 0.f) mask[j >> 5] |= 1u << (j & 31);
                *reinterpret_cast<__nv_bfloat16*>(sHT + umma::kmajor_offset_b16(j, tid, 128)) =
                    __float2bfloat16(fmaxf(v[q], slope * v[q]));
            }
        }
        umma::fence_before_sync();
        __syncthreads();  // every row of P has been read before it is overwritten
        umma::fence_after_sync();
        // (3) P = A W^T -> D (W a) (column tid of its transpose)
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < KP / 16; s++)
                umma::mma_bf16(tP, umma::smem_desc(aAA + s * 256, 128, SBO1), umma::smem_desc(aW1 + s * 256, 128, SBO1),
                               idescP, s > 0);
            umma::commit(bar1);
        }
        ok = umma::mbar_wait(bar1, ph1, kMlpWaitLimit);
        ph1 ^= 1;
        if (__syncthreads_or(!ok)) { failed = true; break; }
        umma::fence_after_sync();
#pragma unroll
        for (int c8 = 0; c8 < H / 8; c8++) {
            float v[8];
            umma::tmem_ld8(tP + lane_base + c8 * 8, v);
            umma::tmem_ld_wait();
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int j = c8 * 8 + q;
                const float bm = (mask[j >> 5] >> (j & 31)) & 1u ? v[q] : slope * v[q];
                *reinterpret_cast<__nv_bfloat16*>(sBT + umma::kmajor_offset_b16(j, tid, 128)) = __float2bfloat16(bm);
            }
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        // (4) Gw += h^T A + (D W a)^T X over this tile's 128 patches
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < 128 / 16; s++)
                umma::mma_bf16(tG, umma::smem_desc(aHT + s * 256, 128, SBOT), umma::smem_desc(aAT + s * 256, 128, SBOT),
                               idescG, (any || s > 0) ? 1u : 0u);
#pragma unroll
            for (int s = 0; s < 128 / 16; s++)
                umma::mma_bf16(tG, umma::smem_desc(aBT + s * 256, 128, SBOT), umma::smem_desc(aXT + s * 256, 128, SBOT),
                               idescG, 1u);
            umma::commit(bar2);
        }
        any = true;
    }
    if (!failed && any) {
        const bool ok = umma::mbar_wait(bar2, ph2, kMlpWaitLimit);
        if (__syncthreads_or(!ok)) failed = true;
        umma::fence_after_sync();
    }
    // partial of this CTA: row j = hidden unit (TMEM lane), columns = features
    float* out = part + (size_t)blockIdx.x * H * F;
    const int j = 32 * warp + (tid & 31);
    if (!failed && any) {
#pragma unroll
        for (int c8 = 0; c8 < KP / 8; c8++) {
            float v[8];
            umma::tmem_ld8(tG + lane_base + c8 * 8, v);
            umma::tmem_ld_wait();
#pragma unroll
            for (int q = 0; q < 8; q++)
                if (c8 * 8 + q < F) out[(size_t)j * F + c8 * 8 + q] = v[q];
        }
    } else {
        for (int i = 0; i < F; i++) out[(size_t)j * F + i] = 0.f;
    }
    if (failed && tid == 0) atomicExch(status, 1);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, D::TMEM_COLS);
}

// gW = (2 a / b) * sum over the CTA partials (fixed order), a and b each the
// sum of G partials
__global__ void schwarz_mlp_wreduce_kernel(const float* __restrict__ part, int nparts, int n,
                                           const double* __restrict__ part_a, const double* __restrict__ part_b, int G,
                                           float* __restrict__ gW) {
    __shared__ float s_scale;
    if (threadIdx.x < 32) {
        double aa = 0, bb = 0;
        for (int i = threadIdx.x; i < G; i += 32) { aa += part_a[i]; bb += part_b[i]; }
        for (int o = 16; o > 0; o >>= 1) {
            aa += __shfl_xor_sync(0xffffffffu, aa, o);
            bb += __shfl_xor_sync(0xffffffffu, bb, o);
        }
        if (threadIdx.x == 0) s_scale = bb > 0 ? (float)(2.0 * aa / bb) : 0.f;
    }
    __syncthreads();
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        float acc = 0.f;
        for (int c = 0; c < nparts; c++) acc += part[(size_t)c * n + t];
        gW[t] = s_scale * acc;
    }
}

namespace {

template <int NP>
cudaError_t mlp_local_np(const SchwarzArgs& a, const double* r, const float* r32, float* U, const int* done,
                         int* status, cudaStream_t st) {
    using D = MlpDims<NP>;
    static bool attr = false;  // per process: the attribute is a property of the function
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(schwarz_mlp_local_kernel<NP>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, D::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int ntiles = (a.K + 127) / 128;
    const int grid = ntiles < a.sms ? ntiles : a.sms;
    schwarz_mlp_local_kernel<NP><<<grid, 128, D::SMEM, st>>>(a, r32, r, U, done, status);
    return cudaGetLastError();
}

template <int NP>
cudaError_t mlp_wgrad_np(const SchwarzArgs& a, const double* r, const double* g, float* part, int* status,
                         cudaStream_t st) {
    using D = MlpDims<NP>;
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(schwarz_mlp_wgrad_kernel<NP>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, D::GSMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    schwarz_mlp_wgrad_kernel<NP><<<schwarz_mlp_wgrad_ctas(a), 128, D::GSMEM, st>>>(a, r, g, part, status);
    return cudaGetLastError();
}

}  // namespace

#define MLP_NP_DISPATCH(NPV, CALL)              \
    switch (NPV) {                              \
        case 3: { constexpr int NP = 3; return CALL; }   \
        case 6: { constexpr int NP = 6; return CALL; }   \
        case 10: { constexpr int NP = 10; return CALL; } \
        case 15: { constexpr int NP = 15; return CALL; } \
        case 21: { constexpr int NP = 21; return CALL; } \
        case 28: { constexpr int NP = 28; return CALL; } \
        default: return cudaErrorNotSupported;  \
    }

cudaError_t launch_schwarz_mlp_local(const SchwarzArgs& a, const double* r, const float* r32, float* U,
                                     const int* done, int* status, cudaStream_t st) {
    if (a.H != kSchwarzMlpH || !status) return cudaErrorNotSupported;
    MLP_NP_DISPATCH(a.Np, (mlp_local_np<NP>(a, r, r32, U, done, status, st)))
}

int schwarz_mlp_wgrad_ctas(const SchwarzArgs& a) {
    const int ntiles = (a.K + 127) / 128;
    return ntiles < a.sms ? ntiles : a.sms;
}

cudaError_t launch_schwarz_mlp_wgrad(const SchwarzArgs& a, const double* r, const double* g, float* part,
                                     int* status, cudaStream_t st) {
    if (a.H != kSchwarzMlpH || !status) return cudaErrorNotSupported;
    MLP_NP_DISPATCH(a.Np, (mlp_wgrad_np<NP>(a, r, g, part, status, st)))
}

cudaError_t launch_schwarz_mlp_wreduce(const float* part, int nparts, int H, int F, const double* part_a,
                                       const double* part_b, int G, float* gW, cudaStream_t st) {
    const int n = H * F;
    schwarz_mlp_wreduce_kernel<<<(n + 255) / 256, 256, 0, st>>>(part, nparts, n, part_a, part_b, G, gW);
    return cudaGetLastError();
}

}  // namespace dgk
