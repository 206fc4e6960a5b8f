// euler_split_pipe.cu -- the split-precision fused DG Euler stage for orders
// N <= 6, software-pipelined across tiles (sm_103a).
//
// Same arithmetic, operands, tensor-memory layout and results as
// euler_stage_split_kernel (euler_split.cu, which documents them); only the
// order of the work per CTA differs.  There, every phase of a tile runs
// between two CTA barriers, so the FP64-pipe work of staging (one FP64
// subtraction and conversion per staged value; GB300 retires two FP64
// operations per clock per SM) and the memory latency of the epilogue leave
// the other pipes idle.  Here tile t+1's phases are interleaved with tile t's:
//
//   prologue:  stage(t0), GEMM1(t0), faces(t0)
//   per tile t (t+1 = the CTA's next tile):
//     wait GEMM1(t); request t+1's neighbour traces (cp.async)
//     volume passes of t (TMEM -> FP32 flux -> chunk operand -> GEMM2 MMAs),
//       with stage(t+1) in slices between them: pass 0 forms t+1's
//       reference state and metrics (after its FP64 tile copy has landed),
//       the later passes its FP32 deltas and TF32 operand
//     issue the bulk copy of t+2's FP64 tile and GEMM1(t+1)
//     wait GEMM2(t); R(t) TMEM -> shared
//     epilogue(t) (LSERK update, global stores) and faces(t+1) with no
//       barrier between them
//
// The reference state, its FP64 copy and the metrics are double-buffered by
// tile parity; the FP64 tile buffer, the FP32 deltas, the GEMM1 operand and
// the neighbour traces are single-buffered because their readers (faces and
// GEMM1 of t) have finished before stage(t+1) writes them.  The stage input
// is re-read from L2 in the epilogue.  Every mbarrier wait is bounded; a
// timeout sets the status word, and the CTA waits for its copies and MMAs in
// flight before it frees tensor memory and returns.
#include <algorithm>
#include <cstdio>

#include "../../include/dgcu.h"
#include "euler_flux.cuh"
#include "euler_split.cuh"
#include "f64split.cuh"
#include "umma.cuh"

namespace dgk {

template <int N>
struct PipeDims {
    using S = SplitDims<N>;
    static_assert(!S::STREAM, "the pipelined stage covers N <= 6");
    static constexpr int al(int x) { return (x + 1023) / 1024 * 1024; }  // tensor-core operands
    static constexpr int a128(int x) { return (x + 127) / 128 * 128; }    // everything else
    static constexpr int OFF_B1 = 0;
    static constexpr int OFF_B2 = OFF_B1 + al(S::SZ_B1);
    static constexpr int OFF_A1 = OFF_B2 + al(S::SZ_B2);
    static constexpr int OFF_AC = OFF_A1 + al(S::SZ_A1);
    static constexpr int OFF_AF = OFF_AC + S::NBUF * S::AL_AC;
    static constexpr int OFF_QF = OFF_AF + al(S::SZ_AF);
    static constexpr int OFF_Q64 = OFF_QF + a128(S::SZ_QF);
    // per tile parity: reference state FP32 [ROWS], FP64 [ROWS], metrics FP32 [E][4]
    static constexpr int SZ_QB = S::ROWS * 4 + S::ROWS * 8 + S::E * 16;
    static constexpr int QB_STRIDE = (SZ_QB + 127) / 128 * 128;
    static constexpr int OFF_QB = OFF_Q64 + a128(S::SZ_Q64);
    static constexpr int OFF_NB = OFF_QB + 2 * QB_STRIDE;
    static constexpr bool GATHER = OFF_NB + a128(S::SZ_NB_FULL) + 64 <= 232448;
    static constexpr int SZ_NB = GATHER ? S::SZ_NB_FULL : 0;
    static constexpr int OFF_BAR = OFF_NB + a128(SZ_NB);
    static constexpr int SMEM = OFF_BAR + 64;
    static_assert(SMEM <= 232448, "shared memory budget");
    // volume passes (two chunks per pass where there are two chunk buffers)
    static constexpr int NPASS = S::PAIR ? (S::NCH + 1) / 2 : S::NCH;
    // FP32 deltas of a tile per thread, and how they are spread over the passes
    // one core matrix of the GEMM1 operand per warp and step: warp w holds
    // rows 8w .. 8w + 7, lane = 4 (row % 8) + (k % 4), KP1 / 4 steps along K
    static constexpr int NDQ = S::KP1 / 4;
    static_assert(S::THREADS == 512 && S::ROWS == 128, "16 warps x 8 rows");
    static constexpr int DQ_SLICES = NPASS > 1 ? NPASS - 1 : 1;
    static constexpr int DQ_PER = (NDQ + DQ_SLICES - 1) / DQ_SLICES;
};

// The stage for the tiles bid, bid + nblk, ... of one context (a CTA of 512
// threads); the single-context kernel runs it with its own block index and
// grid size, the mixed-order batch kernel with its share of the grid.
template <int N>
__device__ __forceinline__ void pipe_body(const SplitArgs& sa, const int bid, const int nblk) {
    using S = SplitDims<N>;
    using D = PipeDims<N>;
    constexpr int Np = S::Np, Ng = S::Ng, Nfp = S::Nfp, Nfq = S::Nfq, E = S::E;
    constexpr int KP1 = S::KP1, NG = S::NG, NF = S::NF, NP2 = S::NP2, KP2 = S::KP2, CH = S::CH, KC = S::KC;
    constexpr int NB = 3 * N;
    extern __shared__ __align__(1024) unsigned char smem[];
    float* sB1 = reinterpret_cast<float*>(smem + D::OFF_B1);
    float* sB2 = reinterpret_cast<float*>(smem + D::OFF_B2);
    float* sA1 = reinterpret_cast<float*>(smem + D::OFF_A1);
    float* sAF = reinterpret_cast<float*>(smem + D::OFF_AF);
    float* sQF = reinterpret_cast<float*>(smem + D::OFF_QF);
    double* sQ64 = reinterpret_cast<double*>(smem + D::OFF_Q64);
    double* sNB = reinterpret_cast<double*>(smem + D::OFF_NB);
    float* sRS = reinterpret_cast<float*>(smem + D::OFF_AC);  // after GEMM2 completed
    uint64_t* bar1 = reinterpret_cast<uint64_t*>(smem + D::OFF_BAR);
    uint64_t* bar2 = bar1 + 1;  // [NBUF]
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar1 + 3);
    uint64_t* bq = bar1 + 4;  // the FP64 tile copy has landed
    // N = 3 (kArrive): every thread's operand writes of a volume pass after the
    // first, or of the next tile's staging, are done -- every thread arrives,
    // only the MMA-issuing thread waits, the other warps go on into the next
    // pass (measured: N = 3 1.14 -> 1.05 ms per step; no change at N = 2;
    // slower at N = 4, 5, where the warps that run ahead delay the issuing one)
    // (each part alone at N = 4, 5 measured slower too: passes 1.39 -> 1.43 and
    // 1.79 -> 1.85 ms per step, end of staging 1.39 -> 1.40 and 1.79 -> 1.80)
    constexpr bool kArrive = N == 3;      // the later volume passes
    constexpr bool kArrivePost = N == 3;  // the end of the next tile's staging
    uint64_t* bready = bar1 + 5;
    volatile int* sfail = reinterpret_cast<volatile int*>(bar1 + 6);  // a wait of that path timed out
    // reference state / metrics of tile parity b
    auto qbf = [&](int b) { return reinterpret_cast<float*>(smem + D::OFF_QB + b * D::QB_STRIDE); };
    auto qbd = [&](int b) {
        return reinterpret_cast<double*>(smem + D::OFF_QB + b * D::QB_STRIDE + S::ROWS * 4);
    };
    auto geo = [&](int b) {
        return reinterpret_cast<float*>(smem + D::OFF_QB + b * D::QB_STRIDE + S::ROWS * 12);
    };

    const EulerArgs& a = sa.e;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ntiles = (a.K + E - 1) / E;
    const float gamma = (float)a.gamma;
    const int G = nblk;

    uint32_t pq = 0;       // bq phase parity
    bool qpend = false;    // a tile copy in flight (thread 0)
    bool g1pend = false;   // a GEMM1 in flight whose completion nobody waited for (thread 0)
    auto issue_q = [&](int t) {
        const int k0t = t * E;
        const uint32_t bytes = (uint32_t)min(E, a.K - k0t) * 4u * (uint32_t)Np * 8u;
        umma::mbar_arrive_expect_tx(bq, bytes);
        umma::bulk_g2s(sQ64, a.qin + (size_t)k0t * 4 * Np, bytes, bq);
        qpend = true;
    };

    // neighbour traces of a tile's faces into sNB by 8-byte asynchronous copies
    // (the neighbour element's node in its own face order with the rotation
    // applied, or the boundary slot's trace); cn[j]: the face link of this
    // thread's task j, loaded ahead
    constexpr int GT = (3 * E * Nfp + S::THREADS - 1) / S::THREADS;
    int cn[GT];
    auto load_links = [&](int t) {
#pragma unroll
        for (int j = 0; j < GT; j++) {
            const int i = tid + j * S::THREADS;
            cn[j] = (t < ntiles && i < 3 * min(E, a.K - t * E) * Nfp) ? __ldg(a.conn + (size_t)t * E * 3 + i / Nfp) : 0;
        }
    };
    auto gather = [&](int t) {
        const int kt = t * E;
        const int nt = 3 * min(E, a.K - kt) * Nfp;
#pragma unroll
        for (int j = 0; j < GT; j++) {
            const int i = tid + j * S::THREADS;
            if (i >= nt) break;
            const int ef = i / Nfp, ii = i - ef * Nfp;
            const int c = cn[j];
            const double* src;
            int vstride;
            if (c >= 0) {
                const int nb = c >> 3, fn = c & 3, rot = (c >> 2) & 1;
                const int jj = rot ? (N - ii) : ii;
                src = a.qin + (size_t)nb * 4 * Np + (fn * N + jj) % NB;
                vstride = Np;
            } else {
                src = a.btrace + (size_t)(-1 - c) * 4 * Nfp + ii;
                vstride = Nfp;
            }
            double* dst = sNB + (size_t)i * 4;
#pragma unroll
            for (int v = 0; v < 4; v++) umma::cp_async8(dst + v, src + v * vstride);
        }
    };

    // stage, part 1: the reference state (mean of the three vertex values,
    // FP32 and its FP64 copy) and FP32 metrics of tile t into parity b; the
    // tile's FP64 copy must have landed
    auto stage_ref = [&](int t, int b) {
        const int k0t = t * E, net = min(E, a.K - k0t);
        if (tid < S::ROWS) {
            const int e = tid >> 2, v = tid & 3;
            float qb = 1.f;
            if (e < net) {
                const double* row = sQ64 + e * 4 * Np + v * Np;  // ring order: vertices at 0, N, 2N
                qb = (float)((row[0] + row[N] + row[2 * N]) * (1.0 / 3.0));
            }
            qbf(b)[tid] = qb;
            qbd(b)[tid] = (double)qb;
        } else if (tid < S::ROWS + 4 * E) {
            const int e = (tid - S::ROWS) >> 2, c = (tid - S::ROWS) & 3;
            geo(b)[tid - S::ROWS] = e < net ? (float)a.geo[(size_t)(k0t + e) * 4 + c] : 0.f;
        }
    };
    // stage, part 2: FP32 deltas (this thread's items j0 <= j < j1) into sQF and
    // their TF32 hi / lo into the GEMM1 operand
    constexpr uint32_t LO_A1 = 128 * KP1 * 4;
    // the rows and K offsets of this thread in the core-matrix mapping
    const int cm_r = 8 * warp + (lane >> 2), cm_k = lane & 3;
    auto stage_dq = [&](int t, int b, int j0, int j1) {
        const int net = min(E, a.K - t * E);
        if (cm_r >= 4 * net) return;  // rows of a missing element (tail tile)
        const double qr = qbd(b)[cm_r];
        const double* src = sQ64 + cm_r * Np + cm_k;
        float* qf = sQF + cm_r * Np + cm_k;
        float* dst = sA1 + (warp * (KP1 / 4)) * 32 + lane;
#pragma unroll
        for (int j = j0; j < j1; j++) {
            if (j < D::NDQ && 4 * j + cm_k < Np) {
                const float d = (float)(src[4 * j] - qr);
                qf[4 * j] = d;
                float hi, lo;
                umma::split_tf32(d, hi, lo);
                dst[32 * j] = hi;
                dst[32 * j + LO_A1 / 4] = lo;
            }
        }
    };

    // constant operands and zero padding, once per CTA
    {
        const int4* src1 = reinterpret_cast<const int4*>(sa.b1);
        int4* dst1 = reinterpret_cast<int4*>(sB1);
        for (int i = tid; i < S::SZ_B1 / 16; i += blockDim.x) dst1[i] = src1[i];
        const int4* src2 = reinterpret_cast<const int4*>(sa.b2);
        int4* dst2 = reinterpret_cast<int4*>(sB2);
        for (int i = tid; i < S::SZ_B2 / 16; i += blockDim.x) dst2[i] = src2[i];
        for (int i = tid; i < S::SZ_A1 / 4; i += blockDim.x) sA1[i] = 0.f;
        for (int i = tid; i < S::SZ_AF / 4; i += blockDim.x) sAF[i] = 0.f;
    }
    const int t0 = bid;
    if (tid == 0) {
        umma::mbar_init(bar1, 1);
        for (int b = 0; b < S::NBUF; b++) umma::mbar_init(bar2 + b, 1);
        umma::mbar_init(bq, 1);
        umma::mbar_init(bready, S::THREADS);
        *sfail = 0;
        umma::fence_mbar_init();
        if (t0 < ntiles) issue_q(t0);
    }
    if (warp == 0) {
        umma::tmem_alloc(tmem_slot, S::TMEM_COLS);
        umma::tmem_relinquish();
    }
    umma::fence_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const uint32_t tD1 = tmem, tD2 = tmem + S::D2_COL;
    const uint32_t idesc1 = umma::idesc_tf32(128, NG);
    const uint32_t idesc2 = umma::idesc_tf32(128, NP2);
    const uint32_t aB1 = umma::smem_u32(sB1), aB2 = umma::smem_u32(sB2);
    const uint32_t aA1 = umma::smem_u32(sA1), aAF = umma::smem_u32(sAF);
    const uint32_t aAC = umma::smem_u32(smem + D::OFF_AC);
    constexpr uint32_t LO_B1 = NG * KP1 * 4, LO_B2 = S::SZ_B2 / 2, LO_AC = 128 * KC * 4, LO_AF = 128 * NF * 4,
                       STRIDE_AC = S::AL_AC;
    uint32_t ph1 = 0;
    uint32_t ph2 = 0;  // bit b: phase parity of chunk buffer b's MMA barrier
    uint32_t phr = 0;  // phase parity of bready
    bool failed = false;
    const int qd = warp & 3, sub = warp >> 2;
    const int my_e = 8 * qd + (lane >> 2), my_v = lane & 3;

    // thread 0: GEMM1 of the tile staged in sA1, completion on bar1
    auto issue_gemm1 = [&]() {
#pragma unroll
        for (int s = 0; s < KP1 / 8; s++) {
            const uint64_t ah = umma::smem_desc(aA1 + s * 256, 128, (KP1 / 4) * 128);
            const uint64_t al = umma::smem_desc(aA1 + LO_A1 + s * 256, 128, (KP1 / 4) * 128);
            const uint64_t bh = umma::smem_desc(aB1 + s * 256, 128, (KP1 / 4) * 128);
            const uint64_t bl = umma::smem_desc(aB1 + LO_B1 + s * 256, 128, (KP1 / 4) * 128);
            umma::mma_tf32(tD1, ah, bh, idesc1, s > 0);
            umma::mma_tf32(tD1, al, bh, idesc1, 1);
            umma::mma_tf32(tD1, ah, bl, idesc1, 1);
        }
        umma::commit(bar1);
        g1pend = true;
    };

    // face fluxes of tile t (reference state / metrics of parity b) into the
    // lift operand sAF; the neighbour traces are in sNB (GATHER) or are loaded
    // here
    auto faces = [&](int t, int b) {
        const int k0 = t * E, ne = min(E, a.K - k0);
        const float* sQB = qbf(b);
        const double* sQBd = qbd(b);
        const float* sGeo = geo(b);
        if constexpr (S::FP == 2) {
            // N = 4..6: one (element, face) per segment of FW = ceil(Nfq / 2)
            // lanes; lane li = face nodes li, li + FW and Gauss points li, li + FW
            constexpr int FW = S::FW, FPW = S::FPW;
            const int seg = lane / FW, li = lane - seg * FW;  // lanes with seg >= FPW idle
            const int sbase = (seg < FPW ? seg : 0) * FW;
            const int Gf = warp * FPW + seg;
            const bool gok = seg < FPW && Gf < 3 * E;
            const int Gc = gok ? Gf : warp * FPW;
            const int e = Gc / 3, f = Gc - 3 * e;
            const bool valid = gok && e < ne;
            const int k = k0 + (valid ? e : 0);
            float qbv[4];
            double qbdv[4];
#pragma unroll
            for (int v = 0; v < 4; v++) {
                qbv[v] = sQB[4 * (valid ? e : 0) + v];
                qbdv[v] = sQBd[4 * (valid ? e : 0) + v];
            }
            float own[2][4], nbr[2][4];
#pragma unroll
            for (int sl = 0; sl < 2; sl++) {
                const int i = li + sl * FW;
#pragma unroll
                for (int v = 0; v < 4; v++) own[sl][v] = nbr[sl][v] = 0.f;
                if (valid && i < Nfp) {
                    const int pos = (f * N + i) % NB;
#pragma unroll
                    for (int v = 0; v < 4; v++) own[sl][v] = sQF[e * 4 * Np + v * Np + pos];
                    if constexpr (D::GATHER) {
                        const double* nv = sNB + (size_t)((3 * e + f) * Nfp + i) * 4;
#pragma unroll
                        for (int v = 0; v < 4; v++) nbr[sl][v] = f64s::minus_f32(nv[v], qbv[v]);
                    } else {
                        const int c = __ldg(a.conn + (size_t)k * 3 + f);
                        const double* src;
                        int vs;
                        if (c >= 0) {
                            const int nb = c >> 3, fn = c & 3, rot = (c >> 2) & 1;
                            const int jj = rot ? (N - i) : i;
                            src = a.qin + (size_t)nb * 4 * Np + (fn * N + jj) % NB;
                            vs = Np;
                        } else {
                            src = a.btrace + (size_t)(-1 - c) * 4 * Nfp + i;
                            vs = Nfp;
                        }
#pragma unroll
                        for (int v = 0; v < 4; v++) nbr[sl][v] = (float)(__ldg(src + v * vs) - qbdv[v]);
                    }
                }
            }
            float dm[2][4], dp[2][4];
            int gi[2];
#pragma unroll
            for (int sl = 0; sl < 2; sl++) {
                gi[sl] = (li + sl * FW < Nfq) ? li + sl * FW : 0;
#pragma unroll
                for (int v = 0; v < 4; v++) dm[sl][v] = dp[sl][v] = 0.f;
            }
#pragma unroll
            for (int jn = 0; jn < Nfp; jn++) {
                const int src = sbase + jn % FW;
                const float w0 = __ldg(sa.If32 + gi[0] * Nfp + jn);
                const float w1 = __ldg(sa.If32 + gi[1] * Nfp + jn);
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    const float om = __shfl_sync(0xffffffffu, own[jn / FW][v], src);
                    const float op = __shfl_sync(0xffffffffu, nbr[jn / FW][v], src);
                    dm[0][v] = fmaf(w0, om, dm[0][v]);
                    dp[0][v] = fmaf(w0, op, dp[0][v]);
                    dm[1][v] = fmaf(w1, om, dm[1][v]);
                    dp[1][v] = fmaf(w1, op, dp[1][v]);
                }
            }
            const float* gk = sGeo + 4 * (valid ? e : 0);
            float nx, ny, fsc;
            face_normal_f(f, gk[0], gk[1], gk[2], gk[3], nx, ny, fsc);
            const RefState rb = make_ref(gamma, qbv);
            DeltaPrim pm[2], pp[2];
#pragma unroll
            for (int sl = 0; sl < 2; sl++) {
                pm[sl] = delta_prim(gamma, rb, dm[sl]);
                pp[sl] = delta_prim(gamma, rb, dp[sl]);
            }
            float F[2][4];
            if (a.flux == 1) {
#pragma unroll
                for (int sl = 0; sl < 2; sl++) roe_flux_delta(gamma, nx, ny, rb, dm[sl], pm[sl], dp[sl], pp[sl], F[sl]);
            } else {
                float lam = 0.f;
#pragma unroll
                for (int sl = 0; sl < 2; sl++)
                    if (li + sl * FW < Nfq)
                        lam = fmaxf(lam, fmaxf(wave_speed_delta(gamma, nx, ny, rb, pm[sl]),
                                               wave_speed_delta(gamma, nx, ny, rb, pp[sl])));
                float m = lam;
#pragma unroll
                for (int j = 0; j < FW; j++) m = fmaxf(m, __shfl_sync(0xffffffffu, lam, sbase + j));
#pragma unroll
                for (int sl = 0; sl < 2; sl++) lf_flux_delta(nx, ny, m, rb, dm[sl], pm[sl], dp[sl], pp[sl], F[sl]);
            }
#pragma unroll
            for (int sl = 0; sl < 2; sl++) {
                const int g = li + sl * FW;
                if (valid && g < Nfq) {
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        float hi, lo;
                        umma::split_tf32(-fsc * F[sl][v], hi, lo);
                        const uint32_t off = umma::kmajor_offset(g2row(e, v), f * Nfq + g, NF) >> 2;
                        sAF[off] = hi;
                        sAF[off + LO_AF / 4] = lo;
                    }
                }
            }
        } else {
            // one (element, face) per segment of SW lanes, lane i = face node i
            // (gather) and face Gauss point i (flux)
            constexpr int SW = S::SW, SPW = S::SPW;
            const int seg = lane / SW, i = lane - seg * SW;  // lanes with seg >= SPW idle
            const int sbase = (seg < SPW ? seg : 0) * SW;
#pragma unroll 1
            for (int gbase = warp * SPW; gbase < 3 * E; gbase += (S::THREADS / 32) * SPW) {
                const int Gf = gbase + seg;
                const bool gok = seg < SPW && Gf < 3 * E;
                const int Gc = gok ? Gf : gbase;
                const int e = Gc / 3, f = Gc - 3 * e;
                const bool valid = gok && e < ne;
                const int k = k0 + (valid ? e : 0);
                float own[4] = {0.f, 0.f, 0.f, 0.f}, nbr[4] = {0.f, 0.f, 0.f, 0.f};
                float qbv[4];
                double qbdv[4];
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    qbv[v] = sQB[4 * (valid ? e : 0) + v];
                    qbdv[v] = sQBd[4 * (valid ? e : 0) + v];
                }
                if (valid && i < Nfp) {
                    const int pos = (f * N + i) % NB;
#pragma unroll
                    for (int v = 0; v < 4; v++) own[v] = sQF[e * 4 * Np + v * Np + pos];
                    if constexpr (D::GATHER) {
                        const double* nv = sNB + (size_t)((3 * e + f) * Nfp + i) * 4;
#pragma unroll
                        for (int v = 0; v < 4; v++) nbr[v] = f64s::minus_f32(nv[v], qbv[v]);
                    } else {
                        const int c = __ldg(a.conn + (size_t)k * 3 + f);
                        if (c >= 0) {
                            const int nb = c >> 3, fn = c & 3, rot = (c >> 2) & 1;
                            const int jj = rot ? (N - i) : i;
                            const double* qn = a.qin + (size_t)nb * 4 * Np + (fn * N + jj) % NB;
#pragma unroll
                            for (int v = 0; v < 4; v++) nbr[v] = (float)(__ldg(qn + v * Np) - qbdv[v]);
                        } else {
                            const double* bt = a.btrace + (size_t)(-1 - c) * 4 * Nfp + i;
#pragma unroll
                            for (int v = 0; v < 4; v++) nbr[v] = (float)(__ldg(bt + v * Nfp) - qbdv[v]);
                        }
                    }
                }
                float dm[4] = {0.f, 0.f, 0.f, 0.f}, dp[4] = {0.f, 0.f, 0.f, 0.f};
                const int gi = i < Nfq ? i : 0;
#pragma unroll
                for (int jn = 0; jn < Nfp; jn++) {
                    const float w = __ldg(sa.If32 + gi * Nfp + jn);
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        if constexpr (S::PACKED) {
                            dm[v] = fmaf(w, __shfl_sync(0xffffffffu, own[v], sbase + jn), dm[v]);
                            dp[v] = fmaf(w, __shfl_sync(0xffffffffu, nbr[v], sbase + jn), dp[v]);
                        } else {
                            dm[v] = fmaf(w, __shfl_sync(0xffffffffu, own[v], jn, SW), dm[v]);
                            dp[v] = fmaf(w, __shfl_sync(0xffffffffu, nbr[v], jn, SW), dp[v]);
                        }
                    }
                }
                const float* gk = sGeo + 4 * (valid ? e : 0);
                float nx, ny, fsc;
                face_normal_f(f, gk[0], gk[1], gk[2], gk[3], nx, ny, fsc);
                const RefState rb = make_ref(gamma, qbv);
                const DeltaPrim pm = delta_prim(gamma, rb, dm), pp = delta_prim(gamma, rb, dp);
                float F[4];
                if (a.flux == 1) {
                    roe_flux_delta(gamma, nx, ny, rb, dm, pm, dp, pp, F);
                } else {
                    float lam = (i < Nfq) ? fmaxf(wave_speed_delta(gamma, nx, ny, rb, pm),
                                                  wave_speed_delta(gamma, nx, ny, rb, pp))
                                          : 0.f;
                    if constexpr (S::PACKED) {
                        float m = lam;
#pragma unroll
                        for (int j = 0; j < Nfq; j++) m = fmaxf(m, __shfl_sync(0xffffffffu, lam, sbase + j));
                        lam = m;
                    } else {
#pragma unroll
                        for (int o = 1; o < SW; o <<= 1) lam = fmaxf(lam, __shfl_xor_sync(0xffffffffu, lam, o, SW));
                    }
                    lf_flux_delta(nx, ny, lam, rb, dm, pm, dp, pp, F);
                }
                if (valid && i < Nfq) {
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        float hi, lo;
                        umma::split_tf32(-fsc * F[v], hi, lo);
                        const uint32_t off = umma::kmajor_offset(g2row(e, v), f * Nfq + i, NF) >> 2;
                        sAF[off] = hi;
                        sAF[off + LO_AF / 4] = lo;
                    }
                }
            }
        }
    };

    // ---- prologue: stage, GEMM1 and face fluxes of the first tile
    if (t0 < ntiles) {
        if constexpr (D::GATHER) {
            load_links(t0);
            gather(t0);
            load_links(t0 + G);
        }
        const bool okq = umma::mbar_wait(bq, pq, kWaitLimit);
        pq ^= 1;
        if (tid == 0 && okq) qpend = false;
        if (__syncthreads_or(!okq)) failed = true;
        if (!failed) {
            stage_ref(t0, 0);
            __syncthreads();
            stage_dq(t0, 0, 0, D::NDQ);
            if constexpr (D::GATHER) umma::cp_async_wait_all();
            umma::fence_async_smem();
            umma::fence_before_sync();
            __syncthreads();
            umma::fence_after_sync();
            if (tid == 0) {
                if (t0 + G < ntiles) issue_q(t0 + G);
                issue_gemm1();
            }
            faces(t0, 0);
        }
    }

    int par = 0;  // parity of the current tile's reference-state buffer
    for (int tile = t0; tile < ntiles && !failed; tile += G, par ^= 1) {
        const int k0 = tile * E;
        const int ne = min(E, a.K - k0);
        const int tn = tile + G;  // this CTA's next tile
        const bool has_next = tn < ntiles;
        // ---- wait for GEMM1(t); the face phase of t is complete after this barrier
        const bool ok1 = umma::mbar_wait(bar1, ph1, kWaitLimit);
        ph1 ^= 1;
        if (tid == 0 && ok1) g1pend = false;
        if (__syncthreads_or(!ok1)) { failed = true; break; }
        umma::fence_after_sync();
        if constexpr (D::GATHER) {
            // every warp has read sNB: request the next tile's traces (they land
            // during the volume phase), then the links of the tile after it
            if (has_next) {
                gather(tn);
                load_links(tn + G);
            }
        }
        // per-thread element data for the volume flux
        float qbe[4];
#pragma unroll
        for (int v = 0; v < 4; v++) qbe[v] = qbf(par)[4 * my_e + v];
        const RefState bref = make_ref(gamma, qbe);
        const float* gcur = geo(par);
        const float rx = gcur[4 * my_e], sx = gcur[4 * my_e + 1], ry = gcur[4 * my_e + 2], sy = gcur[4 * my_e + 3];

        auto vol_flux = [&](const float* x, int ch, float* fr, float* fs) {
            // the 4 variables at point (sub*4 + my_v): a 4 x 4 transpose across the
            // element's 4 lanes in two butterfly stages (lane bit 1, then bit 0)
            float dq[4] = {x[0], x[1], x[2], x[3]};
            {
                const bool bb = (my_v & 2) != 0;
                const float r0 = __shfl_xor_sync(0xffffffffu, bb ? dq[0] : dq[2], 2);
                const float r1 = __shfl_xor_sync(0xffffffffu, bb ? dq[1] : dq[3], 2);
                dq[0] = bb ? r0 : dq[0];
                dq[1] = bb ? r1 : dq[1];
                dq[2] = bb ? dq[2] : r0;
                dq[3] = bb ? dq[3] : r1;
            }
            {
                const bool bb = (my_v & 1) != 0;
                const float r0 = __shfl_xor_sync(0xffffffffu, bb ? dq[0] : dq[1], 1);
                const float r1 = __shfl_xor_sync(0xffffffffu, bb ? dq[2] : dq[3], 1);
                dq[0] = bb ? r0 : dq[0];
                dq[2] = bb ? r1 : dq[2];
                dq[1] = bb ? dq[1] : r0;
                dq[3] = bb ? dq[3] : r1;
            }
            const int g = ch * CH + sub * 4 + my_v;
            if (g < Ng && my_e < ne) {
                const DeltaPrim d = delta_prim(gamma, bref, dq);
                float fx[4], fy[4];
                flux_delta(bref, dq, d, fx, fy);
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    fr[v] = rx * fx[v] + ry * fy[v];
                    fs[v] = sx * fx[v] + sy * fy[v];
                }
            } else {
#pragma unroll
                for (int v = 0; v < 4; v++) fr[v] = fs[v] = 0.f;
            }
        };
        // this thread's slots in a chunk operand: rows g2row(my_e, v) are one
        // 8-row group apart per v (KC * 8 floats), the Fs columns CH / 4 core
        // matrices after the Fr ones, so every store is a fixed offset from one base
        float* const sAC0 =
            reinterpret_cast<float*>(smem + D::OFF_AC) + (umma::kmajor_offset(g2row(my_e, 0), sub * 4 + my_v, KC) >> 2);
        auto store_chunk = [&](int buf, const float* fr, const float* fs) {
            constexpr int VSTR = KC * 8, FSO = CH * 8, LO = LO_AC / 4;
            float* const b = sAC0 + buf * (STRIDE_AC / 4);
#pragma unroll
            for (int v = 0; v < 4; v++) {
                float hi, lo;
                umma::split_tf32(fr[v], hi, lo);
                b[v * VSTR] = hi;
                b[v * VSTR + LO] = lo;
                umma::split_tf32(fs[v], hi, lo);
                b[v * VSTR + FSO] = hi;
                b[v * VSTR + FSO + LO] = lo;
            }
        };
        auto issue_mma = [&](int ch, int buf) {
            constexpr uint32_t sboA = (KC / 4) * 128, sboB = (KP2 / 4) * 128;
            const uint32_t aC = aAC + buf * STRIDE_AC;
#pragma unroll
            for (int s = 0; s < KC / 8; s++) {
                const uint64_t ah = umma::smem_desc(aC + s * 256, 128, sboA);
                const uint64_t al = umma::smem_desc(aC + LO_AC + s * 256, 128, sboA);
                const int kb = (s < CH / 8) ? (ch * CH + 8 * s) : (NG + ch * CH + 8 * (s - CH / 8));
                const uint64_t bh = umma::smem_desc(aB2 + kb * 32, 128, sboB);
                const uint64_t bl = umma::smem_desc(aB2 + LO_B2 + kb * 32, 128, sboB);
                const uint32_t acc = (ch > 0 || s > 0) ? 1u : 0u;
                umma::mma_tf32(tD2, ah, bh, idesc2, acc);
                umma::mma_tf32(tD2, al, bh, idesc2, 1);
                umma::mma_tf32(tD2, ah, bl, idesc2, 1);
            }
            if (ch == S::NCH - 1) {
                constexpr uint32_t sboF = (NF / 4) * 128;
#pragma unroll
                for (int s = 0; s < NF / 8; s++) {
                    const int kb = 2 * NG + 8 * s;
                    const uint64_t ah = umma::smem_desc(aAF + s * 256, 128, sboF);
                    const uint64_t al = umma::smem_desc(aAF + LO_AF + s * 256, 128, sboF);
                    const uint64_t bh = umma::smem_desc(aB2 + kb * 32, 128, sboB);
                    const uint64_t bl = umma::smem_desc(aB2 + LO_B2 + kb * 32, 128, sboB);
                    umma::mma_tf32(tD2, ah, bh, idesc2, 1);
                    umma::mma_tf32(tD2, al, bh, idesc2, 1);
                    umma::mma_tf32(tD2, ah, bl, idesc2, 1);
                }
            }
            umma::commit(bar2 + buf);
        };
        // the slice of stage(tn) that goes with volume pass p
        const int pn = par ^ 1;
        auto stage_slice = [&](int p) {
            if (!has_next) return;
            if (p == 0) {
                // tn's FP64 tile (issued after stage(t)) has landed by now
                const bool okq = umma::mbar_wait(bq, pq, kWaitLimit);
                if (!okq) failed = true;
                stage_ref(tn, pn);
            } else if (D::NPASS > 1) {
                const int j0 = (p - 1) * D::DQ_PER;
                const int j1 = min(D::NDQ, j0 + D::DQ_PER);
                if (j0 < j1) stage_dq(tn, pn, j0, j1);
            }
        };

        // ---- (C) volume phase of t, stage(tn) in slices
        if constexpr (S::PAIR) {
            int prev_n = 0;
#pragma unroll 1
            for (int p = 0; p < D::NPASS; p++) {
                const int ch0 = 2 * p;
                const int n = (S::NCH - ch0 >= 2) ? 2 : 1;
                float x0[4], x1[4];
                umma::tmem_ld4(tD1 + ((uint32_t)(32 * qd) << 16) + ch0 * CH + sub * 4, x0);
                if (n == 2) umma::tmem_ld4(tD1 + ((uint32_t)(32 * qd) << 16) + (ch0 + 1) * CH + sub * 4, x1);
                umma::tmem_ld_wait();
                float fr0[4], fs0[4], fr1[4], fs1[4];
                vol_flux(x0, ch0, fr0, fs0);
                if (n == 2) vol_flux(x1, ch0 + 1, fr1, fs1);
                stage_slice(p);
                bool okw = !failed;
                for (int b = 0; b < prev_n; b++) {
                    okw = umma::mbar_wait(bar2 + b, (ph2 >> b) & 1u, kWaitLimit) && okw;
                    ph2 ^= 1u << b;
                }
                store_chunk(0, fr0, fs0);
                if (n == 2) store_chunk(1, fr1, fs1);
                umma::fence_async_smem();
                umma::fence_before_sync();
                if (!kArrive || p == 0) {
                    // (pass 0 staged tn's reference state, which every thread's later
                    // slices read: always a CTA barrier)
                    if (__syncthreads_or(!okw)) { failed = true; break; }
                    umma::fence_after_sync();
                    if (tid == 0) {
                        issue_mma(ch0, 0);
                        if (n == 2) issue_mma(ch0 + 1, 1);
                    }
                } else {
                    if (!okw) *sfail = 1;
                    umma::mbar_arrive(bready);
                    if (tid == 0) {
                        const bool okr = umma::mbar_wait(bready, phr, kWaitLimit);
                        if (okr && !*sfail) {
                            umma::fence_after_sync();
                            issue_mma(ch0, 0);
                            if (n == 2) issue_mma(ch0 + 1, 1);
                        } else {
                            *sfail = 1;
                        }
                    }
                    phr ^= 1u;
                    __syncwarp();
                }
                prev_n = n;
            }
        } else {
            // one chunk buffer: each pass waits for the previous pass's MMAs
#pragma unroll 1
            for (int ch = 0; ch < S::NCH; ch++) {
                float x[4];
                umma::tmem_ld4(tD1 + ((uint32_t)(32 * qd) << 16) + ch * CH + sub * 4, x);
                umma::tmem_ld_wait();
                float fr[4], fs[4];
                vol_flux(x, ch, fr, fs);
                stage_slice(ch);
                bool okw = !failed;
                if (ch >= 1) {
                    okw = umma::mbar_wait(bar2, ph2 & 1u, kWaitLimit) && okw;
                    ph2 ^= 1u;
                }
                if (__syncthreads_or(!okw)) { failed = true; break; }
                store_chunk(0, fr, fs);
                umma::fence_async_smem();
                umma::fence_before_sync();
                __syncthreads();
                umma::fence_after_sync();
                if (tid == 0) issue_mma(ch, 0);
            }
        }
        if (failed) break;
        // the rest of stage(tn): with one volume pass the deltas follow here
        if (has_next) {
            if constexpr (D::NPASS == 1) {
                __syncthreads();  // tn's reference state
                stage_dq(tn, pn, 0, D::NDQ);
            }
        }
        if constexpr (D::GATHER) umma::cp_async_wait_all();  // tn's neighbour traces (this thread's copies)
        umma::fence_async_smem();
        umma::fence_before_sync();
        if constexpr (kArrivePost && S::PAIR && D::NPASS > 1) {
            // the issuing thread waits until every thread's staging of tn is written
            // and its reads of D1 are done (sQ64 was read in pass 0, before its barrier)
            umma::mbar_arrive(bready);
            if (has_next) pq ^= 1;  // every thread waited for tn's tile copy in pass 0
            if (tid == 0) {
                const bool okr = umma::mbar_wait(bready, phr, kWaitLimit);
                if (okr && !*sfail) {
                    umma::fence_after_sync();
                    if (has_next) {
                        qpend = false;
                        if (tn + G < ntiles) issue_q(tn + G);
                        issue_gemm1();
                    }
                } else {
                    *sfail = 1;
                }
            }
            phr ^= 1u;
            __syncwarp();
        } else {
            __syncthreads();
            umma::fence_after_sync();
            if (has_next) {
                pq ^= 1;  // every thread waited for tn's tile copy in pass 0
                if (tid == 0) {
                    qpend = false;
                    if (tn + G < ntiles) issue_q(tn + G);  // sQ64 has been read by stage(tn)
                    issue_gemm1();                         // D1 has been read by the volume phase of t
                }
            }
        }
        // the epilogue's RK register values and stage input (L2), loaded while the last MMAs run
        constexpr int EPI = S::EPI;
        const bool first = sa.first != 0;
        const double* qtile = a.qin + (size_t)k0 * 4 * Np;
        float resp[EPI];
        double q0v[EPI];
        {
            const size_t base = (size_t)k0 * 4 * Np;
            const bool need = a.mode == MODE_LSERK && !first;
            const bool needq = a.mode != MODE_RHS;
#pragma unroll
            for (int j = 0; j < EPI; j++) {
                const int i = tid + j * S::THREADS;
                resp[j] = (need && i < ne * 4 * Np) ? __ldg(sa.res32 + base + i) : 0.f;
                q0v[j] = (needq && i < ne * 4 * Np) ? __ldg(qtile + i) : 0.0;
            }
        }
        // outstanding GEMM2 commits
        {
            bool okw = true;
            if constexpr (S::PAIR) {
                constexpr int last_n = (S::NCH % 2 == 0) ? 2 : 1;
#pragma unroll
                for (int b = 0; b < last_n; b++) {
                    okw = umma::mbar_wait(bar2 + b, (ph2 >> b) & 1u, kWaitLimit) && okw;
                    ph2 ^= 1u << b;
                }
            } else {
                okw = umma::mbar_wait(bar2, ph2 & 1u, kWaitLimit);
                ph2 ^= 1u;
            }
            if (__syncthreads_or(!okw || *sfail)) { failed = true; break; }
        }
        umma::fence_after_sync();
        // ---- (D) R (tensor memory) -> staging
        {
            const int e2 = 8 * qd + (lane & 7), v2 = lane >> 3;  // this lane's GEMM2 row (g2row)
#pragma unroll
            for (int col = sub * 8; col < NP2; col += 32) {
                float val[8];
                umma::tmem_ld8(tD2 + ((uint32_t)(32 * qd) << 16) + col, val);
                umma::tmem_ld_wait();
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int p = col + j;
                    if (p < Np && e2 < ne) sRS[(4 * e2 + v2) * Np + p] = val[j];
                }
            }
        }
        umma::fence_before_sync();
        __syncthreads();
        // ---- epilogue of t
        {
            const size_t base = (size_t)k0 * 4 * Np;
            const float rka = sa.rkaf, dtf0 = sa.dtf, rkb = sa.rkbf;
            const int nv = ne * 4 * Np;
            if (a.mode == MODE_LSERK && !sa.dtk32) {
#pragma unroll
                for (int j = 0; j < EPI; j++) {
                    const int i = tid + j * S::THREADS;
                    if (i < nv) {
                        const float R = sRS[i];
                        const float r = first ? dtf0 * R : fmaf(rka, resp[j], dtf0 * R);
                        sa.res32_out[base + i] = r;
                        a.qout[base + i] = q0v[j] + (double)(rkb * r);
                    }
                }
            } else {
#pragma unroll
                for (int j = 0; j < EPI; j++) {
                    const int i = tid + j * S::THREADS;
                    if (i >= nv) break;
                    const float R = sRS[i];
                    const double q0 = q0v[j];
                    const size_t idx = base + i;
                    const float dtf = sa.dtk32 ? dtf0 * sa.dtk32[k0 + i / (4 * Np)] : dtf0;
                    switch (a.mode) {
                        case MODE_RHS: a.rhs[idx] = (double)R; break;
                        case MODE_LSERK: {
                            const float r = first ? dtf * R : fmaf(rka, resp[j], dtf * R);
                            sa.res32_out[idx] = r;
                            a.qout[idx] = q0 + (double)(rkb * r);
                        } break;
                        case MODE_EULER: a.qout[idx] = q0 + (double)(dtf * R); break;
                        default: a.qout[idx] = 0.5 * a.qold[idx] + 0.5 * (q0 + (double)(dtf * R)); break;
                    }
                }
            }
        }
        // ---- face fluxes of tn (no barrier: warps move on as their stores issue)
        if (has_next) faces(tn, pn);
    }
    if (failed && tid == 0) atomicExch(sa.status, 1);
    // let this CTA's asynchronous work in flight complete before it exits
    if (tid == 0) {
        if (qpend) umma::mbar_wait(bq, pq, kWaitLimit);
        if (g1pend) umma::mbar_wait(bar1, ph1, kWaitLimit);
    }
    if constexpr (D::GATHER) umma::cp_async_wait_all();
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, S::TMEM_COLS);
}

template <int N>
__global__ void __launch_bounds__(512, 1) euler_stage_split_pipe_kernel(SplitArgs sa) {
    pipe_body<N>(sa, blockIdx.x, gridDim.x);
}

// One stage of several contexts of orders 1..6 in one launch: blocks
// [cta_end[g-1], cta_end[g]) run group g's tiles with its order's body.
__global__ void __launch_bounds__(512, 1) euler_stage_split_batch_kernel(const __grid_constant__ SplitBatchArgs P) {
    int g = 0;
    while (g + 1 < P.ngroups && (int)blockIdx.x >= P.cta_end[g]) g++;
    const int begin = g ? P.cta_end[g - 1] : 0;
    const int bid = (int)blockIdx.x - begin, nblk = P.cta_end[g] - begin;
    switch (P.order[g]) {
        case 1: pipe_body<1>(P.sa[g], bid, nblk); break;
        case 2: pipe_body<2>(P.sa[g], bid, nblk); break;
        case 3: pipe_body<3>(P.sa[g], bid, nblk); break;
        case 4: pipe_body<4>(P.sa[g], bid, nblk); break;
        case 5: pipe_body<5>(P.sa[g], bid, nblk); break;
        case 6: pipe_body<6>(P.sa[g], bid, nblk); break;
        default: break;
    }
}

static int batch_smem(int N) {
    switch (N) {
        case 1: return PipeDims<1>::SMEM;
        case 2: return PipeDims<2>::SMEM;
        case 3: return PipeDims<3>::SMEM;
        case 4: return PipeDims<4>::SMEM;
        case 5: return PipeDims<5>::SMEM;
        case 6: return PipeDims<6>::SMEM;
        default: return 0;
    }
}

cudaError_t setup_split_batch() {
    int smax = 0;
    for (int n = 1; n <= 6; n++) smax = std::max(smax, batch_smem(n));
    return cudaFuncSetAttribute(euler_stage_split_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
}

cudaError_t launch_split_batch(const SplitBatchArgs& P, cudaStream_t s) {
    if (P.ngroups < 1 || P.ngroups > SplitBatchArgs::MAXG) return cudaErrorInvalidValue;
    int smax = 0;
    for (int g = 0; g < P.ngroups; g++) {
        const int sm = batch_smem(P.order[g]);
        if (sm == 0) return cudaErrorInvalidValue;
        smax = std::max(smax, sm);
    }
    euler_stage_split_batch_kernel<<<P.cta_end[P.ngroups - 1], 512, smax, s>>>(P);
    return cudaGetLastError();
}

template <int N>
cudaError_t setup_split_pipe() {
    return cudaFuncSetAttribute(euler_stage_split_pipe_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                PipeDims<N>::SMEM);
}

template <int N>
cudaError_t launch_split_pipe(const SplitArgs& sa, int grid, cudaStream_t s) {
    euler_stage_split_pipe_kernel<N><<<grid, SplitDims<N>::THREADS, PipeDims<N>::SMEM, s>>>(sa);
    return cudaGetLastError();
}

template cudaError_t setup_split_pipe<1>();
template cudaError_t setup_split_pipe<2>();
template cudaError_t setup_split_pipe<3>();
template cudaError_t setup_split_pipe<4>();
template cudaError_t setup_split_pipe<5>();
template cudaError_t setup_split_pipe<6>();
template cudaError_t launch_split_pipe<1>(const SplitArgs&, int, cudaStream_t);
template cudaError_t launch_split_pipe<2>(const SplitArgs&, int, cudaStream_t);
template cudaError_t launch_split_pipe<3>(const SplitArgs&, int, cudaStream_t);
template cudaError_t launch_split_pipe<4>(const SplitArgs&, int, cudaStream_t);
template cudaError_t launch_split_pipe<5>(const SplitArgs&, int, cudaStream_t);
template cudaError_t launch_split_pipe<6>(const SplitArgs&, int, cudaStream_t);

}  // namespace dgk
