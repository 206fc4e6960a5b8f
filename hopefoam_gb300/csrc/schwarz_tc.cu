// schwarz_tc.cu -- tensor-core (tcgen05, kind::tf32) local stage of the learned
// additive-Schwarz preconditioner: U_m = W^T (W G_m r) for tiles of 128
// elements (one TMEM lane row per element).
//
//   GEMM1  Hd[128][32]  = X[128][F -> KP1] . W^T        (B1 = W, K-major rows j)
//   GEMM2  Ud[128][NF2] = Hd[128][32]      . W          (B2 = W^T, K-major rows i)
//
// W is stored in BF16, so its TF32 image is exact and a single pass of W
// suffices; the FP32 activations X and Hd enter as TF32 hi + lo (two passes),
// which keeps the products at FP32 accuracy: M stays linear to FP32 round-off.
// Operands use the canonical no-swizzle K-major layout of umma.cuh; the second
// A operand (Hd) overwrites the first (X) after GEMM1 has completed. Every
// mbarrier wait is bounded and reports a timeout in *status.
#include <cuda_bf16.h>

#include "lpc.hpp"
#include "umma.cuh"

namespace dgk {

namespace {

constexpr uint32_t kTcWaitLimit = 1u << 22;

template <int NP>
struct SchwarzTcDims {
    static constexpr int H = 32;
    static constexpr int F = 4 * NP;
    static constexpr int KP1 = (F + 7) / 8 * 8;       // GEMM1 K
    static constexpr int NF2 = (F + 15) / 16 * 16;    // GEMM2 N (M = 128 needs N % 16 == 0)
    static constexpr int KP2 = H;                     // GEMM2 K
    static constexpr int KA = KP1 > KP2 ? KP1 : KP2;  // A buffer width (X, then Hd)
    static constexpr int al(int x) { return (x + 1023) / 1024 * 1024; }
    static constexpr int SZ_B1 = H * KP1 * 4;
    static constexpr int SZ_B2 = NF2 * KP2 * 4;
    static constexpr int SZ_A = 2 * 128 * KA * 4;     // hi | lo
    static constexpr int OFF_B1 = 0;
    static constexpr int OFF_B2 = OFF_B1 + al(SZ_B1);
    static constexpr int OFF_A = OFF_B2 + al(SZ_B2);
    static constexpr int OFF_BAR = OFF_A + al(SZ_A);
    static constexpr int SMEM = OFF_BAR + 64;
    static constexpr int TMEM_COLS = (H + NF2) <= 128 ? 128 : 256;
    static_assert(SMEM <= 232448, "shared memory budget");
};

// X row of element m: the residual on the element and its three rotated
// neighbours (zero for m >= K and across a boundary)
template <int NP>
__device__ __forceinline__ void tc_gather(const SchwarzArgs& a, const float* __restrict__ r32,
                                          const double* __restrict__ r, int m, float* x) {
    if (m >= a.K) {
#pragma unroll
        for (int i = 0; i < 4 * NP; i++) x[i] = 0.f;
        return;
    }
    if (r32) {
        const float* vm = r32 + (size_t)m * NP;
#pragma unroll
        for (int i = 0; i < NP; i++) x[i] = vm[i];
    } else {
        const double* vm = r + (size_t)m * NP;
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
            float v = 0.f;
            if (c >= 0) v = r32 ? r32[nb + pm[i]] : (float)r[nb + pm[i]];
            x[(f + 1) * NP + i] = v;
        }
    }
}

}  // namespace

template <int NP>
__global__ void __launch_bounds__(128, 1) schwarz_local_tc_kernel(SchwarzArgs a, const float* __restrict__ r32,
                                                                  const double* __restrict__ r, float* __restrict__ U,
                                                                  const int* __restrict__ done, int* status) {
    using D = SchwarzTcDims<NP>;
    constexpr int H = D::H, F = D::F, KP1 = D::KP1, NF2 = D::NF2, KP2 = D::KP2;
    extern __shared__ __align__(1024) unsigned char smem[];
    if (done && *done) return;
    float* sB1 = reinterpret_cast<float*>(smem + D::OFF_B1);
    float* sB2 = reinterpret_cast<float*>(smem + D::OFF_B2);
    float* sA = reinterpret_cast<float*>(smem + D::OFF_A);
    uint64_t* bar1 = reinterpret_cast<uint64_t*>(smem + D::OFF_BAR);
    uint64_t* bar2 = bar1 + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar1 + 2);
    volatile int* fail_flag = reinterpret_cast<volatile int*>(bar1 + 3);
    const int tid = threadIdx.x, warp = tid >> 5;

    // B images from the BF16 weights (exact in TF32), zero padding
    for (int t = tid; t < H * KP1; t += blockDim.x) {
        const int j = t / KP1, i = t - j * KP1;
        sB1[umma::kmajor_offset(j, i, KP1) >> 2] = i < F ? __bfloat162float(a.W[j * F + i]) : 0.f;
    }
    for (int t = tid; t < NF2 * KP2; t += blockDim.x) {
        const int i = t / KP2, j = t - i * KP2;
        sB2[umma::kmajor_offset(i, j, KP2) >> 2] = i < F ? __bfloat162float(a.W[j * F + i]) : 0.f;
    }
    if (tid == 0) {
        *fail_flag = 0;
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
    const uint32_t idesc1 = umma::idesc_tf32(128, H);
    const uint32_t idesc2 = umma::idesc_tf32(128, NF2);
    const uint32_t aB1 = umma::smem_u32(sB1), aB2 = umma::smem_u32(sB2), aA = umma::smem_u32(sA);
    constexpr uint32_t LO1 = 128 * KP1 * 4, LO2 = 128 * KP2 * 4;
    uint32_t ph = 0;
    bool failed = false;
    const int ntiles = (a.K + 127) / 128;

    // X rows are gathered one tile ahead: the next tile's loads are in flight
    // while this tile's MMAs, activations and stores run
    float x[F];
    if (blockIdx.x < ntiles) tc_gather<NP>(a, r32, r, blockIdx.x * 128 + tid, x);
    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        // (1) X row of element tile * 128 + tid as TF32 hi + lo
        {
            // four consecutive k per 16-byte store: eight threads of a phase
            // write 128 contiguous bytes (no bank conflicts)
#pragma unroll
            for (int i4 = 0; i4 < KP1 / 4; i4++) {
                float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (4 * i4 + q < F) umma::split_tf32(x[4 * i4 + q], hi[q], lo[q]);
                const uint32_t off = umma::kmajor_offset(tid, 4 * i4, KP1) >> 2;
                *reinterpret_cast<float4*>(sA + off) = make_float4(hi[0], hi[1], hi[2], hi[3]);
                *reinterpret_cast<float4*>(sA + off + LO1 / 4) = make_float4(lo[0], lo[1], lo[2], lo[3]);
            }
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < KP1 / 8; s++) {
                const uint64_t ah = umma::smem_desc(aA + s * 256, 128, (KP1 / 4) * 128);
                const uint64_t al = umma::smem_desc(aA + LO1 + s * 256, 128, (KP1 / 4) * 128);
                const uint64_t b = umma::smem_desc(aB1 + s * 256, 128, (KP1 / 4) * 128);
                umma::mma_tf32(tD1, ah, b, idesc1, s > 0);
                umma::mma_tf32(tD1, al, b, idesc1, 1);
            }
            umma::commit(bar1);
        }
        if (tile + (int)gridDim.x < ntiles) tc_gather<NP>(a, r32, r, (tile + gridDim.x) * 128 + tid, x);
        bool ok = umma::mbar_wait(bar1, ph, kTcWaitLimit);
        if (__syncthreads_or(!ok)) { failed = true; break; }
        umma::fence_after_sync();
        // (2) Hd row -> A2 (hi, lo), written over X (GEMM1 has completed)
#pragma unroll
        for (int c8 = 0; c8 < H / 8; c8++) {
            float h[8];
            umma::tmem_ld8(tD1 + lane_base + c8 * 8, h);
            umma::tmem_ld_wait();
#pragma unroll
            for (int q4 = 0; q4 < 2; q4++) {
                float hi[4], lo[4];
#pragma unroll
                for (int q = 0; q < 4; q++) umma::split_tf32(h[4 * q4 + q], hi[q], lo[q]);
                const uint32_t off = umma::kmajor_offset(tid, c8 * 8 + 4 * q4, KP2) >> 2;
                *reinterpret_cast<float4*>(sA + off) = make_float4(hi[0], hi[1], hi[2], hi[3]);
                *reinterpret_cast<float4*>(sA + off + LO2 / 4) = make_float4(lo[0], lo[1], lo[2], lo[3]);
            }
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < KP2 / 8; s++) {
                const uint64_t ah = umma::smem_desc(aA + s * 256, 128, (KP2 / 4) * 128);
                const uint64_t al = umma::smem_desc(aA + LO2 + s * 256, 128, (KP2 / 4) * 128);
                const uint64_t b = umma::smem_desc(aB2 + s * 256, 128, (KP2 / 4) * 128);
                umma::mma_tf32(tD2, ah, b, idesc2, s > 0);
                umma::mma_tf32(tD2, al, b, idesc2, 1);
            }
            umma::commit(bar2);
        }
        ok = umma::mbar_wait(bar2, ph, kTcWaitLimit);
        ph ^= 1;
        if (__syncthreads_or(!ok)) { failed = true; break; }
        umma::fence_after_sync();
        // (3) U rows: TMEM -> shared memory (the A buffer is free: GEMM2 has
        //     completed) -> coalesced float4 stores of the tile's contiguous rows
        float* sU = sA;  // 128 x F floats, row-major
#pragma unroll
        for (int c8 = 0; c8 < NF2 / 8; c8++) {
            float u[8];
            umma::tmem_ld8(tD2 + lane_base + c8 * 8, u);
            umma::tmem_ld_wait();
            // F % 4 == 0: whole float4 groups (rows of F / 4 groups; the 16-byte
            // stride of F floats between threads spreads a phase over all banks)
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
        __syncthreads();  // A is rewritten by the next tile
    }
    if (failed && tid == 0) atomicExch(status, 1);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, D::TMEM_COLS);
}

template <int NP>
static cudaError_t schwarz_tc_np(const SchwarzArgs& a, const double* r, const float* r32, float* U,
                                 const int* done, int* status, cudaStream_t st) {
    using D = SchwarzTcDims<NP>;
    static bool attr = false;  // per process: the attribute is a property of the function
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(schwarz_local_tc_kernel<NP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             D::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int ntiles = (a.K + 127) / 128;
    const int grid = ntiles < 2 * a.sms ? ntiles : 2 * a.sms;
    schwarz_local_tc_kernel<NP><<<grid, 128, D::SMEM, st>>>(a, r32, r, U, done, status);
    return cudaGetLastError();
}

cudaError_t launch_schwarz_local_tc(const SchwarzArgs& a, const double* r, const float* r32, float* U,
                                    const int* done, int* status, cudaStream_t st) {
    if (a.H != 32) return cudaErrorNotSupported;
    switch (a.Np) {
        case 3: return schwarz_tc_np<3>(a, r, r32, U, done, status, st);
        case 6: return schwarz_tc_np<6>(a, r, r32, U, done, status, st);
        case 10: return schwarz_tc_np<10>(a, r, r32, U, done, status, st);
        case 15: return schwarz_tc_np<15>(a, r, r32, U, done, status, st);
        case 21: return schwarz_tc_np<21>(a, r, r32, U, done, status, st);
        case 28: return schwarz_tc_np<28>(a, r, r32, U, done, status, st);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace dgk
