// euler_split.cu -- split-precision fused DG Euler stage on the tcgen05 tensor
// cores (sm_103a).
//
// Arithmetic: the two contractions of the quadrature-form DG right-hand side
// run as TF32 GEMMs with 3-pass split products (hi*hi + lo*hi + hi*lo) and
// FP32 accumulation in tensor memory, on deltas against a per-element
// reference state qb (the row mean):
//   GEMM1 (cubature interpolation, dgGaussField.C:193-202):
//     dQg[r][g] = sum_p dQ[r][p] Vg[g][p],      M = 128 rows r = 4 e + v
//                                               (32 elements x 4 variables),
//                                               N = Ng padded, K = Np padded
//   GEMM2 (volume term + surface lift with the affine mass inverse folded in,
//          defaultConvectionScheme.C:79-128, defaultGrad.C:120-165,
//          defaultDivScheme.C:118-165):
//     R[r][p] = sum_g dFr[r][g] Sr[p][g] + dFs[r][g] Ss[p][g]
//             + sum_c (-sJ/J dF*)[r][c] Lift[p][c],   N = Np padded
// with dF = F(qb + dQ) - F(qb) and dF* = n.F*(q-, q+) - n.F(qb) evaluated
// point-wise in FP32 in cancellation-free product-rule form (euler_flux.cuh).
// Because the weak divergence of a constant flux cancels against its own
// surface term, R is unchanged by the shift, but the FP32 round-off now
// scales with the variation inside an element instead of with |F| N^2 / h.
// The state q stays FP64 in HBM; dQ = q - qb (and the neighbour traces' deltas)
// is one FP64 subtraction and conversion per value (at N = 7 it is formed from
// q's bits with integer and FP32 operations, f64split.cuh); the low-storage RK
// register is FP32 (it carries dt*R, whose own precision is FP32); q += b*res
// is the only other FP64 arithmetic per value.
//
// Structure: persistent CTAs (one per SM, 512 threads), 32 elements per tile.
// Per tile: stage q (FP64 tile in shared memory, reference state, FP32 deltas,
// TF32 hi/lo in the canonical no-swizzle K-major layout, see umma.cuh) ->
// GEMM1 (issued by one thread, completion on an mbarrier) -> face fluxes in
// lane segments, one per (element, face) (gather, Gauss interpolation and
// wave-speed max by shuffles) while GEMM1 runs -> per chunk of 16 cubature
// points: tensor memory ->
// registers, the 4 variables of a point exchanged by a two-stage butterfly of
// warp shuffles within the element's 4 lanes -> FP32 delta flux -> TF32 split into a
// double-buffered chunk operand -> GEMM2 MMAs for that K chunk -> epilogue:
// tensor memory -> shared -> coalesced LSERK update.  At N = 7 the volume
// operator is streamed from L2 per chunk and the tile is not copied to shared
// memory (SplitDims::STREAM).  All mbarrier waits are bounded; a timeout sets
// the status word, the CTA waits for its bulk copies in flight, frees tensor
// memory and returns.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/dgcu.h"
#include "dg_ctx.hpp"
#include "euler_flux.cuh"
#include "euler_split.cuh"
#include "f64split.cuh"
#include "umma.cuh"

namespace dgk {

template <int N>
__global__ void __launch_bounds__(512, 1) euler_stage_split_kernel(SplitArgs sa) {
    using D = SplitDims<N>;
    constexpr int Np = D::Np, Ng = D::Ng, Nfp = D::Nfp, Nfq = D::Nfq, E = D::E;
    constexpr int KP1 = D::KP1, NG = D::NG, NF = D::NF, NP2 = D::NP2, KP2 = D::KP2, CH = D::CH, KC = D::KC;
    constexpr int NB = 3 * N;
    extern __shared__ __align__(1024) unsigned char smem[];
    float* sB1 = reinterpret_cast<float*>(smem + D::OFF_B1);
    float* sB2 = reinterpret_cast<float*>(smem + D::OFF_B2);
    float* sA1 = reinterpret_cast<float*>(smem + D::OFF_A1);
    float* sAF = reinterpret_cast<float*>(smem + D::OFF_AF);
    float* sQF = reinterpret_cast<float*>(smem + D::OFF_QF);
    double* sQ64 = reinterpret_cast<double*>(smem + D::OFF_Q64);
    float* sQB = reinterpret_cast<float*>(smem + D::OFF_QB);                      // [ROWS]
    double* sQBd = reinterpret_cast<double*>(smem + D::OFF_QB + D::ROWS * 4);    // FP64 copy (resident path)
    float* sGeo = reinterpret_cast<float*>(smem + D::OFF_QB + D::OFF_GEO_IN_QB);  // [E][rx, sx, ry, sy]
    double* sNB = reinterpret_cast<double*>(smem + D::OFF_NB);                   // gathered neighbour traces
    float* sRS = reinterpret_cast<float*>(smem + D::OFF_AC);  // after GEMM2 completed
    uint64_t* bar1 = reinterpret_cast<uint64_t*>(smem + D::OFF_BAR);
    uint64_t* bar2 = bar1 + 1;  // [NBUF]
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar1 + 3);
    volatile int* fail_flag = reinterpret_cast<volatile int*>(bar1 + 4);  // set by thread 0, read after a barrier
    uint64_t* bfull = bar1 + 5;  // [NBUF] streamed operand buffer filled (N = 7)
    uint64_t* bq = bar1 + 7;     // N <= 6: the FP64 tile copy has landed

    const EulerArgs& a = sa.e;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ntiles = (a.K + E - 1) / E;
    const float gamma = (float)a.gamma;
    // streamed [Sr|Ss] chunks (N = 7): thread 0 issues the bulk copies and
    // tracks the buffers' phases and copies in flight
    const float* bsrc = sa.b2 + D::SZ_B2 / 4;
    uint32_t pb = 0, pend = 0;  // bit b: buffer b's phase parity / a copy in flight
    auto issue_chunk = [&](int c, int b) {
        umma::mbar_arrive_expect_tx(bfull + b, D::SZ_BC);
        umma::bulk_g2s(smem + D::OFF_BC + b * D::AL_BC, bsrc + (size_t)c * (D::SZ_BC / 4), D::SZ_BC, bfull + b);
        pend |= 1u << b;
    };
    // N <= 6: the next tile's FP64 state is copied into sQ64 by one bulk copy,
    // issued as soon as the current tile's staging has read sQ64 (the
    // epilogue reads the stage input from L2), so it lands during the face
    // and volume phases
    uint32_t pq = 0;
    bool qpend = false;
    // the neighbour side of every face node of a tile (interior: the neighbour
    // element's node in its own face order, rotation applied; boundary: the
    // slot's trace) into sNB by 8-byte asynchronous copies; cnv[j] holds the
    // face link of this thread's task j (loaded by the caller, 0 = the first
    // tile, whose links are loaded here)
    constexpr int GT = (3 * E * Nfp + D::THREADS - 1) / D::THREADS;
    int cn[GT];
    auto gather = [&](int t0, const int* cnv) {
        const int kt = t0 * E;
        const int nt = 3 * min(E, a.K - kt) * Nfp;
#pragma unroll
        for (int j = 0; j < GT; j++) {
            const int t = tid + j * D::THREADS;
            if (t >= nt) break;
            const int ef = t / Nfp, i = t - ef * Nfp;  // ef = 3 e + f
            const int c = (t0 == (int)blockIdx.x) ? __ldg(a.conn + (size_t)kt * 3 + ef) : cnv[j];
            const double* src;
            int vstride;
            if (c >= 0) {
                const int nb = c >> 3, fn = c & 3, rot = (c >> 2) & 1;
                const int jj = rot ? (N - i) : i;
                src = a.qin + (size_t)nb * 4 * Np + (fn * N + jj) % NB;
                vstride = Np;
            } else {
                src = a.btrace + (size_t)(-1 - c) * 4 * Nfp + i;
                vstride = Nfp;
            }
            double* dst = sNB + (size_t)t * 4;
#pragma unroll
            for (int v = 0; v < 4; v++) umma::cp_async8(dst + v, src + v * vstride);
        }
    };
    auto issue_q = [&](int t) {
        const int k0t = t * E;
        const uint32_t bytes = (uint32_t)min(E, a.K - k0t) * 4u * (uint32_t)Np * 8u;
        umma::mbar_arrive_expect_tx(bq, bytes);
        umma::bulk_g2s(sQ64, a.qin + (size_t)k0t * 4 * Np, bytes, bq);
        qpend = true;
    };

    // constant operands and zero padding, once per CTA
    {
        const int4* src1 = reinterpret_cast<const int4*>(sa.b1);
        int4* dst1 = reinterpret_cast<int4*>(sB1);
        for (int i = tid; i < D::SZ_B1 / 16; i += blockDim.x) dst1[i] = src1[i];
        const int4* src2 = reinterpret_cast<const int4*>(sa.b2);
        int4* dst2 = reinterpret_cast<int4*>(sB2);
        for (int i = tid; i < D::SZ_B2 / 16; i += blockDim.x) dst2[i] = src2[i];
        for (int i = tid; i < D::SZ_A1 / 4; i += blockDim.x) sA1[i] = 0.f;
        for (int i = tid; i < D::SZ_AF / 4; i += blockDim.x) sAF[i] = 0.f;
    }
    if (tid == 0) {
        *fail_flag = 0;
        umma::mbar_init(bar1, 1);
        for (int b = 0; b < D::NBUF; b++) umma::mbar_init(bar2 + b, 1);
        if constexpr (D::STREAM)
            for (int b = 0; b < D::NBUF; b++) umma::mbar_init(bfull + b, 1);
        else if (sa.qbulk)
            umma::mbar_init(bq, 1);
        umma::fence_mbar_init();
        if constexpr (D::STREAM) {
            if ((int)blockIdx.x < ntiles) {
                issue_chunk(0, 0);
                issue_chunk(1, 1);
            }
        } else {
            if (sa.qbulk && (int)blockIdx.x < ntiles) issue_q(blockIdx.x);
        }
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
    const uint32_t tD1 = tmem, tD2 = tmem + D::D2_COL;
    const uint32_t idesc1 = umma::idesc_tf32(128, NG);
    const uint32_t idesc2 = umma::idesc_tf32(128, NP2);
    const uint32_t aB1 = umma::smem_u32(sB1), aB2 = umma::smem_u32(sB2);
    const uint32_t aA1 = umma::smem_u32(sA1), aAF = umma::smem_u32(sAF);
    const uint32_t aAC = umma::smem_u32(smem + D::OFF_AC);
    constexpr uint32_t LO_B1 = NG * KP1 * 4, LO_B2 = D::SZ_B2 / 2, LO_A1 = 128 * KP1 * 4, LO_AC = 128 * KC * 4,
                       LO_AF = 128 * NF * 4, STRIDE_AC = D::AL_AC, LO_BC = D::SZ_BC / 2;
    const uint32_t aBC = umma::smem_u32(smem + D::OFF_BC);
    uint32_t ph1 = 0;
    uint32_t ph2 = 0;  // bit b: phase parity of chunk buffer b's MMA barrier
    bool failed = false;

    // this thread's rows in the element-major TMEM layout r = 4 e + v; the
    // four warps sharing a lane quarter split the columns (sub = 0..3)
    const int qd = warp & 3, sub = warp >> 2;
    const int my_e = 8 * qd + (lane >> 2), my_v = lane & 3;

    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const int k0 = tile * E;
        const int ne = min(E, a.K - k0);
        // ---- (A) stage the tile: per-(element, variable) reference state (the
        //      mean of the three vertex values, in FP32), FP32 metrics, FP32
        //      deltas, TF32 hi/lo of the deltas.
        const double* qtile = a.qin + (size_t)k0 * 4 * Np;
        if constexpr (D::GATHER) {
            // this tile's neighbour traces were requested during the previous
            // tile (the first tile's here); read the next tile's face links now,
            // so that its requests go out without a dependent load
            if (tile == (int)blockIdx.x) gather(tile, cn);
            const int nt = tile + (int)gridDim.x;
#pragma unroll
            for (int j = 0; j < GT; j++) {
                const int t = tid + j * D::THREADS;
                cn[j] = (nt < ntiles && t < 3 * min(E, a.K - nt * E) * Nfp) ? __ldg(a.conn + (size_t)nt * E * 3 + t / Nfp)
                                                                          : 0;
            }
        }
        if constexpr (D::STREAM) {
            // N = 7: no FP64 tile copy (the values stay in registers across the
            // reference-state barrier; the vertex values come from L2), and the
            // deltas are formed with integer and FP32 operations (f64split.cuh):
            // at this order the FP64 pipe (2 operations per clock per SM) is the
            // scarcest resource.  Each warp instruction writes one 8-row x
            // 4-column core matrix of the K-major operand (lane = (row & 7) * 4 +
            // (k & 3), 128 contiguous bytes: no bank conflicts); padding rows and
            // columns are written as zeros.
            constexpr int NCM = (D::ROWS / 8) * (KP1 / 4);    // core matrices of the dQ operand
            constexpr int CMW = (NCM + 15) / 16;              // per warp (16 warps)
            auto cm_val = [&](int cm, int& r, int& k) -> bool {
                r = (cm / (KP1 / 4)) * 8 + (lane >> 2);
                k = (cm % (KP1 / 4)) * 4 + (lane & 3);
                return cm < NCM && (r >> 2) < ne && k < Np;
            };
            double qv[CMW];
#pragma unroll
            for (int j = 0; j < CMW; j++) {
                int r, k;
                qv[j] = cm_val(warp + 16 * j, r, k) ? __ldg(qtile + (size_t)r * Np + k) : 0.0;
            }
            if (tid < D::ROWS) {
                const int e = tid >> 2, v = tid & 3;
                float qb = 1.f;
                if (e < ne) {
                    const double* row = qtile + e * 4 * Np + v * Np;  // ring order: vertices at 0, N, 2N
                    qb = (f64s::trunc_f32(__ldg(row)) + f64s::trunc_f32(__ldg(row + N)) +
                          f64s::trunc_f32(__ldg(row + 2 * N))) * (1.f / 3.f);
                }
                sQB[tid] = qb;
            } else if (tid < D::ROWS + 4 * E) {
                const int e = (tid - D::ROWS) >> 2, c = (tid - D::ROWS) & 3;
                sGeo[tid - D::ROWS] = e < ne ? (float)a.geo[(size_t)(k0 + e) * 4 + c] : 0.f;
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < CMW; j++) {
                const int cm = warp + 16 * j;
                int r, k;
                const bool in = cm_val(cm, r, k);
                if (cm < NCM) {
                    float hi, lo;
                    umma::split_tf32(in ? f64s::minus_f32(qv[j], sQB[r]) : 0.f, hi, lo);
                    sA1[cm * 32 + lane] = hi;
                    sA1[cm * 32 + lane + LO_A1 / 4] = lo;
                }
            }
        } else {
            // N <= 6: FP64 tile copy, FP64 reference state copy; one FP64
            // subtraction and one conversion per value (at these orders the
            // kernel is issue-bound and the FP64 form takes fewer instructions)
            if (sa.qbulk) {
                const bool okq = umma::mbar_wait(bq, pq, kWaitLimit);
                pq ^= 1;
                if (okq) qpend = false;
                if (__syncthreads_or(!okq)) { failed = true; break; }
            } else {
                for (int i = tid; i < ne * 4 * Np; i += blockDim.x) sQ64[i] = qtile[i];
                __syncthreads();
            }
            if (tid < D::ROWS) {
                const int e = tid >> 2, v = tid & 3;
                float qb = 1.f;
                if (e < ne) {
                    const double* row = sQ64 + e * 4 * Np + v * Np;  // ring order: vertices at 0, N, 2N
                    qb = (float)((row[0] + row[N] + row[2 * N]) * (1.0 / 3.0));
                }
                sQB[tid] = qb;
                sQBd[tid] = (double)qb;
            } else if (tid < D::ROWS + 4 * E) {
                const int e = (tid - D::ROWS) >> 2, c = (tid - D::ROWS) & 3;
                sGeo[tid - D::ROWS] = e < ne ? (float)a.geo[(size_t)(k0 + e) * 4 + c] : 0.f;
            }
            __syncthreads();
            for (int i = tid; i < ne * 4 * Np; i += blockDim.x) {
                const int e = i / (4 * Np), rem = i - e * 4 * Np, v = rem / Np, p = rem - v * Np;
                const int r = 4 * e + v;
                const float d = (float)(sQ64[i] - sQBd[r]);
                sQF[i] = d;
                float hi, lo;
                umma::split_tf32(d, hi, lo);
                const uint32_t off = umma::kmajor_offset(r, p, KP1) >> 2;
                sA1[off] = hi;
                sA1[off + LO_A1 / 4] = lo;
            }
        }
        if constexpr (D::GATHER) umma::cp_async_wait_all();  // this thread's neighbour-trace copies
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        if constexpr (!D::STREAM) {
            // sQ64 has been read: the next tile's copy may overwrite it
            if (tid == 0 && sa.qbulk && tile + (int)gridDim.x < ntiles) issue_q(tile + gridDim.x);
        }
        if (tid == 0) {
            // GEMM1: D1 = dQ (hi,lo) x Vg (hi,lo)^T, 3 passes per K=8 step
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
        }
        // ---- (B) face fluxes while GEMM1 runs
        if constexpr (D::FP == 2) {
            // N = 4..7: one (element, face) per segment of FW = ceil(Nfq / 2) lanes,
            // lane li = face nodes li, li + FW (gather) and Gauss points li, li + FW
            // (flux): every face of the tile in one pass, two independent flux
            // evaluations per lane, and each shuffled node value serves both points
            constexpr int FW = D::FW, FPW = D::FPW;
            const int seg = lane / FW, li = lane - seg * FW;  // lanes with seg >= FPW idle
            const int sbase = (seg < FPW ? seg : 0) * FW;
            const int G = warp * FPW + seg;
            const bool gok = seg < FPW && G < 3 * E;
            const int Gc = gok ? G : warp * FPW;
            const int e = Gc / 3, f = Gc - 3 * e;
            const bool valid = gok && e < ne;
            const int k = k0 + (valid ? e : 0);
            float qbv[4];
            double qbd[4];
#pragma unroll
            for (int v = 0; v < 4; v++) {
                qbv[v] = sQB[4 * (valid ? e : 0) + v];
                if constexpr (!D::STREAM) qbd[v] = sQBd[4 * (valid ? e : 0) + v];
            }
            float own[2][4], nbr[2][4];
#pragma unroll
            for (int sl = 0; sl < 2; sl++) {
                const int i = li + sl * FW;
#pragma unroll
                for (int v = 0; v < 4; v++) own[sl][v] = nbr[sl][v] = 0.f;
                if (valid && i < Nfp) {
                    const int pos = (f * N + i) % NB;
                    if constexpr (D::STREAM) {
#pragma unroll
                        for (int v = 0; v < 4; v++) {
                            // the FP32 delta, read back from the TF32 operand: hi + lo is exact
                            const uint32_t off = umma::kmajor_offset(4 * e + v, pos, KP1) >> 2;
                            own[sl][v] = sA1[off] + sA1[off + LO_A1 / 4];
                        }
                    } else {
#pragma unroll
                        for (int v = 0; v < 4; v++) own[sl][v] = sQF[e * 4 * Np + v * Np + pos];
                    }
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
                        for (int v = 0; v < 4; v++)
                            nbr[sl][v] = D::STREAM ? f64s::minus_f32(__ldg(src + v * vs), qbv[v])
                                                   : (float)(__ldg(src + v * vs) - qbd[v]);
                    }
                }
            }
            // both traces at this lane's two Gauss points
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
            const RefState b = make_ref(gamma, qbv);
            DeltaPrim pm[2], pp[2];
#pragma unroll
            for (int sl = 0; sl < 2; sl++) {
                pm[sl] = delta_prim(gamma, b, dm[sl]);
                pp[sl] = delta_prim(gamma, b, dp[sl]);
            }
            float F[2][4];
            if (a.flux == 1) {
#pragma unroll
                for (int sl = 0; sl < 2; sl++) roe_flux_delta(gamma, nx, ny, b, dm[sl], pm[sl], dp[sl], pp[sl], F[sl]);
            } else {
                float lam = 0.f;
#pragma unroll
                for (int sl = 0; sl < 2; sl++)
                    if (li + sl * FW < Nfq)
                        lam = fmaxf(lam, fmaxf(wave_speed_delta(gamma, nx, ny, b, pm[sl]),
                                               wave_speed_delta(gamma, nx, ny, b, pp[sl])));
                float m = lam;
#pragma unroll
                for (int j = 0; j < FW; j++) m = fmaxf(m, __shfl_sync(0xffffffffu, lam, sbase + j));
#pragma unroll
                for (int sl = 0; sl < 2; sl++) lf_flux_delta(nx, ny, m, b, dm[sl], pm[sl], dp[sl], pp[sl], F[sl]);
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
            constexpr int SW = D::SW, SPW = D::SPW;
            const int seg = lane / SW, i = lane - seg * SW;  // lanes with seg >= SPW idle
            const int sbase = (seg < SPW ? seg : 0) * SW;     // first lane of this segment
            // the loop bound is warp-uniform, so the shuffles below see full warps
#pragma unroll 1
            for (int gbase = warp * SPW; gbase < 3 * E; gbase += (D::THREADS / 32) * SPW) {
                const int G = gbase + seg;
                const bool gok = seg < SPW && G < 3 * E;
                const int Gc = gok ? G : gbase;
                const int e = Gc / 3, f = Gc - 3 * e;
                const bool valid = gok && e < ne;
                const int k = k0 + (valid ? e : 0);
                float own[4] = {0.f, 0.f, 0.f, 0.f}, nbr[4] = {0.f, 0.f, 0.f, 0.f};
                float qbv[4];
                double qbd[4];
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    qbv[v] = sQB[4 * (valid ? e : 0) + v];
                    if constexpr (!D::STREAM) qbd[v] = sQBd[4 * (valid ? e : 0) + v];
                }
                if (valid && i < Nfp) {
                    const int pos = (f * N + i) % NB;
                    if constexpr (D::STREAM) {
#pragma unroll
                        for (int v = 0; v < 4; v++) {
                            // the FP32 delta, read back from the TF32 operand: hi + lo is exact
                            const uint32_t off = umma::kmajor_offset(4 * e + v, pos, KP1) >> 2;
                            own[v] = sA1[off] + sA1[off + LO_A1 / 4];
                        }
                    } else {
#pragma unroll
                        for (int v = 0; v < 4; v++) own[v] = sQF[e * 4 * Np + v * Np + pos];
                    }
                    if constexpr (D::GATHER) {
                        const double* nv = sNB + (size_t)((3 * e + f) * Nfp + i) * 4;
#pragma unroll
                        for (int v = 0; v < 4; v++) nbr[v] = f64s::minus_f32(nv[v], qbv[v]);
                    } else {
                        const int c = __ldg(a.conn + (size_t)k * 3 + f);
                        if (c >= 0) {
                            const int nb = c >> 3, fn = c & 3, rot = (c >> 2) & 1;
                            const int jj = rot ? (N - i) : i;
                            const int npos = (fn * N + jj) % NB;
                            const double* qn = a.qin + (size_t)nb * 4 * Np + npos;
#pragma unroll
                            for (int v = 0; v < 4; v++)
                                nbr[v] = D::STREAM ? f64s::minus_f32(__ldg(qn + v * Np), qbv[v])
                                                   : (float)(__ldg(qn + v * Np) - qbd[v]);
                        } else {
                            const double* bt = a.btrace + (size_t)(-1 - c) * 4 * Nfp + i;
#pragma unroll
                            for (int v = 0; v < 4; v++)
                                nbr[v] = D::STREAM ? f64s::minus_f32(__ldg(bt + v * Nfp), qbv[v])
                                                   : (float)(__ldg(bt + v * Nfp) - qbd[v]);
                        }
                    }
                }
                // interpolate both traces to Gauss point i (shuffles within the group)
                float dm[4] = {0.f, 0.f, 0.f, 0.f}, dp[4] = {0.f, 0.f, 0.f, 0.f};
                const int gi = i < Nfq ? i : 0;
#pragma unroll
                for (int jn = 0; jn < Nfp; jn++) {
                    const float w = __ldg(sa.If32 + gi * Nfp + jn);
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        if constexpr (D::PACKED) {
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
                const RefState b = make_ref(gamma, qbv);
                const DeltaPrim pm = delta_prim(gamma, b, dm), pp = delta_prim(gamma, b, dp);
                float F[4];
                if (a.flux == 1) {
                    roe_flux_delta(gamma, nx, ny, b, dm, pm, dp, pp, F);
                } else {
                    float lam = (i < Nfq) ? fmaxf(wave_speed_delta(gamma, nx, ny, b, pm),
                                                  wave_speed_delta(gamma, nx, ny, b, pp))
                                          : 0.f;
                    if constexpr (D::PACKED) {
                        float m = lam;
#pragma unroll
                        for (int j = 0; j < Nfq; j++) m = fmaxf(m, __shfl_sync(0xffffffffu, lam, sbase + j));
                        lam = m;
                    } else {
#pragma unroll
                        for (int o = 1; o < SW; o <<= 1) lam = fmaxf(lam, __shfl_xor_sync(0xffffffffu, lam, o, SW));
                    }
                    lf_flux_delta(nx, ny, lam, b, dm, pm, dp, pp, F);
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
        // per-thread element data for the volume flux: reference state and metrics
        float qbe[4];
#pragma unroll
        for (int v = 0; v < 4; v++) qbe[v] = sQB[4 * my_e + v];
        const RefState bref = make_ref(gamma, qbe);
        const float rx = sGeo[4 * my_e], sx = sGeo[4 * my_e + 1], ry = sGeo[4 * my_e + 2], sy = sGeo[4 * my_e + 3];
        // ---- (C) wait for GEMM1, then the volume flux per chunk of cubature points
        bool ok = umma::mbar_wait(bar1, ph1, kWaitLimit);
        ph1 ^= 1;
        if (__syncthreads_or(!ok)) { failed = true; break; }
        umma::fence_after_sync();
        if constexpr (D::GATHER) {
            // every warp has read sNB: request the next tile's traces, which land
            // during the volume phase
            if (tile + (int)gridDim.x < ntiles) gather(tile + gridDim.x, cn);
        }
        // volume flux of this thread's row (e, v) at 4 cubature points of chunk
        // ch; x = the row's values there (tensor memory)
        auto vol_flux = [&](const float* x, int ch, float* fr, float* fs) {
            // the 4 variables at point (sub*4 + my_v): a 4 x 4 transpose across the
            // element's 4 lanes in two butterfly stages (lane bit 1, then bit 0);
            // in a stage a lane sends the two slots whose index bit differs from
            // its own lane bit and receives the partner's into them
            float dq[4] = {x[0], x[1], x[2], x[3]};
            {
                const bool b = (my_v & 2) != 0;
                const float r0 = __shfl_xor_sync(0xffffffffu, b ? dq[0] : dq[2], 2);
                const float r1 = __shfl_xor_sync(0xffffffffu, b ? dq[1] : dq[3], 2);
                dq[0] = b ? r0 : dq[0];
                dq[1] = b ? r1 : dq[1];
                dq[2] = b ? dq[2] : r0;
                dq[3] = b ? dq[3] : r1;
            }
            {
                const bool b = (my_v & 1) != 0;
                const float r0 = __shfl_xor_sync(0xffffffffu, b ? dq[0] : dq[1], 1);
                const float r1 = __shfl_xor_sync(0xffffffffu, b ? dq[2] : dq[3], 1);
                dq[0] = b ? r0 : dq[0];
                dq[2] = b ? r1 : dq[2];
                dq[1] = b ? dq[1] : r0;
                dq[3] = b ? dq[3] : r1;
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
        // TF32 hi/lo of the chunk's flux rows into chunk buffer buf
        // (4-way bank conflicts: a rotation of the variable order per element
        // pair removes them but costs more issue slots than it saves)
        auto store_chunk = [&](int buf, const float* fr, const float* fs) {
            float* sAC = reinterpret_cast<float*>(smem + D::OFF_AC + buf * STRIDE_AC);
            const int gl = sub * 4 + my_v;
#pragma unroll
            for (int v = 0; v < 4; v++) {
                const int r = g2row(my_e, v);
                float hi, lo;
                umma::split_tf32(fr[v], hi, lo);
                uint32_t off = umma::kmajor_offset(r, gl, KC) >> 2;
                sAC[off] = hi;
                sAC[off + LO_AC / 4] = lo;
                umma::split_tf32(fs[v], hi, lo);
                off = umma::kmajor_offset(r, CH + gl, KC) >> 2;
                sAC[off] = hi;
                sAC[off + LO_AC / 4] = lo;
            }
        };
        // thread 0: GEMM2's MMAs for chunk ch in buffer buf (with the lift part
        // after the last chunk), completion on bar2[buf]
        auto issue_mma = [&](int ch, int buf) {
            constexpr uint32_t sboA = (KC / 4) * 128, sboB = (KP2 / 4) * 128;
            const uint32_t aC = aAC + buf * STRIDE_AC;
#pragma unroll
            for (int s = 0; s < KC / 8; s++) {
                const uint64_t ah = umma::smem_desc(aC + s * 256, 128, sboA);
                const uint64_t al = umma::smem_desc(aC + LO_AC + s * 256, 128, sboA);
                uint64_t bh, bl;
                if constexpr (D::STREAM) {
                    // the streamed slice has the chunk's own K layout [Sr 16 | Ss 16]
                    const uint32_t bC = aBC + buf * D::AL_BC;
                    bh = umma::smem_desc(bC + s * 256, 128, sboA);
                    bl = umma::smem_desc(bC + LO_BC + s * 256, 128, sboA);
                } else {
                    // chunk K step s: Fr part (s < 2) at B2 k = ch*CH + 8s, Fs part at NG + ch*CH + 8(s-2)
                    const int kb = (s < CH / 8) ? (ch * CH + 8 * s) : (NG + ch * CH + 8 * (s - CH / 8));
                    bh = umma::smem_desc(aB2 + kb * 32, 128, sboB);
                    bl = umma::smem_desc(aB2 + LO_B2 + kb * 32, 128, sboB);
                }
                const uint32_t acc = (ch > 0 || s > 0) ? 1u : 0u;
                umma::mma_tf32(tD2, ah, bh, idesc2, acc);
                umma::mma_tf32(tD2, al, bh, idesc2, 1);
                umma::mma_tf32(tD2, ah, bl, idesc2, 1);
            }
            if (ch == D::NCH - 1) {
                constexpr uint32_t sboF = (NF / 4) * 128;
#pragma unroll
                for (int s = 0; s < NF / 8; s++) {
                    // lift part: B2 k = 2 NG + 8s (resident image), or k = 8s of the lift-only image
                    const int kb = D::STREAM ? 8 * s : 2 * NG + 8 * s;
                    constexpr uint32_t sbo = D::STREAM ? sboF : sboB;
                    const uint64_t ah = umma::smem_desc(aAF + s * 256, 128, sboF);
                    const uint64_t al = umma::smem_desc(aAF + LO_AF + s * 256, 128, sboF);
                    const uint64_t bh = umma::smem_desc(aB2 + kb * 32, 128, sbo);
                    const uint64_t bl = umma::smem_desc(aB2 + LO_B2 + kb * 32, 128, sbo);
                    umma::mma_tf32(tD2, ah, bh, idesc2, 1);
                    umma::mma_tf32(tD2, al, bh, idesc2, 1);
                    umma::mma_tf32(tD2, ah, bl, idesc2, 1);
                }
            }
            umma::commit(bar2 + buf);
        };
        if constexpr (D::PAIR) {
            // two chunks per pass, one per buffer: each thread carries two
            // independent flux evaluations and a pass has one barrier; before
            // rewriting the buffers every thread waits for the previous pass's
            // MMAs (issued one pass earlier, normally complete by then)
            int prev_n = 0;
            for (int ch0 = 0; ch0 < D::NCH; ch0 += 2) {
                const int n = (D::NCH - ch0 >= 2) ? 2 : 1;
                float x0[4], x1[4];
                umma::tmem_ld4(tD1 + ((uint32_t)(32 * qd) << 16) + ch0 * CH + sub * 4, x0);
                if (n == 2) umma::tmem_ld4(tD1 + ((uint32_t)(32 * qd) << 16) + (ch0 + 1) * CH + sub * 4, x1);
                umma::tmem_ld_wait();
                float fr0[4], fs0[4], fr1[4], fs1[4];
                vol_flux(x0, ch0, fr0, fs0);
                if (n == 2) vol_flux(x1, ch0 + 1, fr1, fs1);
                bool okw = true;
                for (int b = 0; b < prev_n; b++) {
                    okw = umma::mbar_wait(bar2 + b, (ph2 >> b) & 1u, kWaitLimit) && okw;
                    ph2 ^= 1u << b;
                }
                store_chunk(0, fr0, fs0);
                if (n == 2) store_chunk(1, fr1, fs1);
                umma::fence_async_smem();
                umma::fence_before_sync();
                if (__syncthreads_or(!okw)) { failed = true; break; }
                umma::fence_after_sync();
                if (tid == 0) {
                    issue_mma(ch0, 0);
                    if (n == 2) issue_mma(ch0 + 1, 1);
                }
                prev_n = n;
            }
        } else {
            for (int ch = 0; ch < D::NCH; ch++) {
                const int buf = (D::NBUF == 2) ? (ch & 1) : 0;
                // this thread's row (e, v) at 4 cubature points of the chunk
                float x[4];
                umma::tmem_ld4(tD1 + ((uint32_t)(32 * qd) << 16) + ch * CH + sub * 4, x);
                umma::tmem_ld_wait();
                float fr[4], fs[4];
                vol_flux(x, ch, fr, fs);
                if constexpr (D::NBUF >= 2) {
                    // buffer reuse: thread 0 confirmed, before the previous chunk's
                    // barrier, that the MMAs which last read this buffer are complete
                    if (ch >= D::NBUF) ph2 ^= 1u << buf;
                } else {
                    // one buffer: the previous chunk's MMAs are issued after its barrier,
                    // so every thread waits for them here
                    if (ch >= D::NBUF) {
                        ok = umma::mbar_wait(bar2 + buf, (ph2 >> buf) & 1u, kWaitLimit);
                        ph2 ^= 1u << buf;
                        if (__syncthreads_or(!ok)) { failed = true; break; }
                    }
                }
                store_chunk(buf, fr, fs);
                umma::fence_async_smem();
                umma::fence_before_sync();
                if constexpr (D::NBUF >= 2) {
                    // chunk ch + 1 reuses the buffer of chunk ch + 1 - NBUF <= ch - 1, whose
                    // MMAs were issued before this point
                    if (tid == 0 && ch + 1 < D::NCH && ch + 1 >= D::NBUF) {
                        const int nb = (ch + 1) % D::NBUF;
                        if (!umma::mbar_wait(bar2 + nb, (ph2 >> nb) & 1u, kWaitLimit)) *fail_flag = 1;
                        else if constexpr (D::STREAM) issue_chunk(ch + 1, nb);  // its buffer is free now
                    }
                }
                if constexpr (D::STREAM) {
                    // this chunk's [Sr|Ss] slice has landed (issued one chunk earlier)
                    if (tid == 0) {
                        if (!umma::mbar_wait(bfull + buf, (pb >> buf) & 1u, kWaitLimit)) {
                            *fail_flag = 1;
                        } else {
                            pend &= ~(1u << buf);
                            pb ^= 1u << buf;
                        }
                    }
                }
                __syncthreads();
                umma::fence_after_sync();
                if (*fail_flag) { failed = true; break; }
                if (tid == 0) issue_mma(ch, buf);
            }
        }
        if (failed) break;
        // the epilogue's RK register values, loaded while the last MMAs run
        constexpr int EPI = D::EPI;
        const bool first = sa.first != 0;
        float resp[EPI];
        double q0v[EPI];  // N = 7, and N <= 6 with bulk tile copies: the stage input again (L2)
        {
            const size_t base = (size_t)k0 * 4 * Np;
            const bool need = a.mode == MODE_LSERK && !first;
            const bool needq = a.mode != MODE_RHS && (D::STREAM || sa.qbulk);
#pragma unroll
            for (int j = 0; j < EPI; j++) {
                const int i = tid + j * D::THREADS;
                resp[j] = (need && i < ne * 4 * Np) ? __ldg(sa.res32 + base + i) : 0.f;
                q0v[j] = (needq && i < ne * 4 * Np) ? __ldg(qtile + i) : 0.0;
            }
        }
        // outstanding commits
        if constexpr (D::PAIR) {
            // the last pass's buffers
            constexpr int last_n = (D::NCH % 2 == 0) ? 2 : 1;
            bool okw = true;
#pragma unroll
            for (int b = 0; b < last_n; b++) {
                okw = umma::mbar_wait(bar2 + b, (ph2 >> b) & 1u, kWaitLimit) && okw;
                ph2 ^= 1u << b;
            }
            if (__syncthreads_or(!okw)) { failed = true; break; }
        } else {
            // the last NBUF chunks (one per buffer)
#pragma unroll
            for (int b = 0; b < D::NBUF; b++) {
                const int chb = D::NCH - D::NBUF + b;
                if (chb < 0) continue;
                const int buf = (D::NBUF == 2) ? (chb & 1) : 0;
                ok = umma::mbar_wait(bar2 + buf, (ph2 >> buf) & 1u, kWaitLimit);
                ph2 ^= 1u << buf;
                if (__syncthreads_or(!ok)) { failed = true; break; }
            }
        }
        if (failed) break;
        umma::fence_after_sync();
        if constexpr (D::STREAM) {
            // every MMA of this tile is complete: prefetch the next tile's first two slices
            if (tid == 0 && tile + (int)gridDim.x < ntiles) {
                issue_chunk(0, 0);
                issue_chunk(1, 1);
            }
        }
        // ---- (D) epilogue: R (tensor memory) -> staging -> coalesced stage update
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
                    // tensor-memory lane (within the quarter) 8 v + e % 8
                    if (p < Np && e2 < ne) sRS[(4 * e2 + v2) * Np + p] = val[j];
                }
            }
        }
        umma::fence_before_sync();
        __syncthreads();
        if (a.mode == MODE_LSERK && !sa.dtk32) {
            // the LSERK stage with one time step for all elements: straight-line
            // loads and stores (no early exit, no per-value mode dispatch)
            const size_t base = (size_t)k0 * 4 * Np;
            const float rka = sa.rkaf, dtf0 = sa.dtf, rkb = sa.rkbf;
            const int nv = ne * 4 * Np;
#pragma unroll
            for (int j = 0; j < EPI; j++) {
                const int i = tid + j * D::THREADS;
                if (i < nv) {
                    const float R = sRS[i];
                    double q0;
                    if constexpr (D::STREAM) q0 = q0v[j];
                    else q0 = sa.qbulk ? q0v[j] : sQ64[i];
                    const float r = first ? dtf0 * R : fmaf(rka, resp[j], dtf0 * R);
                    sa.res32_out[base + i] = r;
                    a.qout[base + i] = q0 + (double)(rkb * r);
                }
            }
        } else {
            const size_t base = (size_t)k0 * 4 * Np;
            const float rka = sa.rkaf, dtf0 = sa.dtf, rkb = sa.rkbf;
#pragma unroll
            for (int j = 0; j < EPI; j++) {
                const int i = tid + j * D::THREADS;
                if (i >= ne * 4 * Np) break;
                const float R = sRS[i];
                double q0;
                if constexpr (D::STREAM) q0 = q0v[j];
                else q0 = sa.qbulk ? q0v[j] : sQ64[i];
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
        __syncthreads();  // staging buffers are rewritten by the next tile
    }
    if (failed && tid == 0) atomicExch(sa.status, 1);
    if constexpr (D::STREAM) {
        // after a timeout: let this CTA's bulk copies in flight land before it exits
        if (tid == 0)
            for (int b = 0; b < D::NBUF; b++)
                if ((pend >> b) & 1u) umma::mbar_wait(bfull + b, (pb >> b) & 1u, kWaitLimit);
    } else {
        if (tid == 0 && qpend) umma::mbar_wait(bq, pq, kWaitLimit);
        if constexpr (D::GATHER) umma::cp_async_wait_all();  // after a timeout: copies still in flight
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, D::TMEM_COLS);
}

// ---------------------------------------------------------------------------
// host side: operator images and launch

static inline float tf32_rna(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;
    float r;
    memcpy(&r, &u, 4);
    return r;
}

// canonical K-major image of an (rows x KP) operand given by f(row, k) (double),
// hi part then lo part
template <typename F>
static std::vector<float> operand_image(int rows, int KP, F f) {
    std::vector<float> img((size_t)2 * rows * KP, 0.f);
    const size_t lo = (size_t)rows * KP;
    for (int r = 0; r < rows; r++)
        for (int k = 0; k < KP; k++) {
            const double x = f(r, k);
            const float hi = tf32_rna((float)x);
            const float l = (float)(x - (double)hi);
            const size_t off = umma::kmajor_offset(r, k, KP) >> 2;
            img[off] = hi;
            img[lo + off] = l;
        }
    return img;
}

template <int N>
static int setup_n(dg_ctx* c) {
    using D = SplitDims<N>;
    const dgb::RefOps& o = c->ops;
    const int Np = D::Np, Ng = D::Ng, Nfq = D::Nfq, NG = D::NG;
    std::vector<float> b1 = operand_image(D::NG, D::KP1, [&](int g, int p) {
        return (g < Ng && p < Np) ? o.dVg[(size_t)g * Np + p] : 0.0;
    });
    std::vector<float> b2;
    if (D::STREAM) {
        // lift image (resident), then one [Sr 16 | Ss 16] image per chunk (streamed)
        b2 = operand_image(D::NP2, D::NF, [&](int p, int cc) {
            return (p < Np && cc < 3 * Nfq) ? o.dLift[(size_t)p * 3 * Nfq + cc] : 0.0;
        });
        for (int ch = 0; ch < D::NCH; ch++) {
            std::vector<float> bc = operand_image(D::NP2, D::KC, [&](int p, int k) {
                const int g = ch * D::CH + (k < D::CH ? k : k - D::CH);
                if (p >= Np || g >= Ng) return 0.0;
                return k < D::CH ? o.dSr[(size_t)p * Ng + g] : o.dSs[(size_t)p * Ng + g];
            });
            b2.insert(b2.end(), bc.begin(), bc.end());
        }
    } else {
        b2 = operand_image(D::NP2, D::KP2, [&](int p, int k) {
            if (p >= Np) return 0.0;
            if (k < NG) return k < Ng ? o.dSr[(size_t)p * Ng + k] : 0.0;
            if (k < 2 * NG) return (k - NG) < Ng ? o.dSs[(size_t)p * Ng + (k - NG)] : 0.0;
            const int cc = k - 2 * NG;
            return cc < 3 * Nfq ? o.dLift[(size_t)p * 3 * Nfq + cc] : 0.0;
        });
    }
    std::vector<float> if32(o.If.begin(), o.If.end());  // Nfq x Nfp
    size_t bytes = (b1.size() + b2.size() + if32.size()) * sizeof(float);
    float* d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) return DG_ERR_NOMEM;
    cudaMemcpy(d, b1.data(), b1.size() * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d + b1.size(), b2.data(), b2.size() * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d + b1.size() + b2.size(), if32.data(), if32.size() * 4, cudaMemcpyHostToDevice);
    c->split.d_ops = d;
    c->split.ops_bytes = bytes;
    c->split.b2_offset = b1.size();
    c->split.if32_offset = b1.size() + b2.size();
    if (cudaMalloc(&c->split.d_status, sizeof(int)) != cudaSuccess) return DG_ERR_NOMEM;
    cudaMemset(c->split.d_status, 0, sizeof(int));
    if (cudaMalloc(&c->split.d_res32, (size_t)c->K * 4 * Np * sizeof(float)) != cudaSuccess) return DG_ERR_NOMEM;
    cudaMemset(c->split.d_res32, 0, (size_t)c->K * 4 * Np * sizeof(float));
    if (cudaFuncSetAttribute(euler_stage_split_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, D::SMEM) !=
        cudaSuccess)
        return DG_ERR_CUDA;
    if constexpr (!D::STREAM) {
        if (setup_split_pipe<N>() != cudaSuccess) return DG_ERR_CUDA;
        if (setup_split_batch() != cudaSuccess) return DG_ERR_CUDA;
        c->split.variant = SplitPlan::PIPE;
        // DGCU_SPLIT_VARIANT=classic selects the tile-serial kernel (A/B measurements)
        const char* v = getenv("DGCU_SPLIT_VARIANT");
        if (v && strcmp(v, "classic") == 0) c->split.variant = SplitPlan::CLASSIC;
    } else {
        c->split.variant = SplitPlan::CLASSIC;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    c->split.sms = sms;
    c->split.N = N;
    c->split.ready = true;
    return DG_OK;
}

int split_fill_args(const EulerArgs& a, const SplitPlan& plan, SplitArgs* sa) {
    sa->e = a;
    sa->res32 = plan.d_res32;
    sa->res32_out = plan.d_res32;
    sa->b1 = static_cast<const float*>(plan.d_ops);
    sa->b2 = static_cast<const float*>(plan.d_ops) + plan.b2_offset;
    sa->status = plan.d_status;
    sa->qbulk = (reinterpret_cast<uintptr_t>(a.qin) & 15u) == 0;
    sa->If32 = static_cast<const float*>(plan.d_ops) + plan.if32_offset;
    sa->dtk32 = a.dtk ? a.dtk32 : nullptr;
    sa->rkaf = (float)a.rka;
    sa->rkbf = (float)a.rkb;
    sa->dtf = (float)a.dt;
    sa->first = a.rka == 0.0;
    return DG_OK;
}

template <int N>
static cudaError_t launch_split_n(const EulerArgs& a, const SplitPlan& plan, cudaStream_t s) {
    using D = SplitDims<N>;
    SplitArgs sa;
    split_fill_args(a, plan, &sa);
    const int ntiles = (a.K + D::E - 1) / D::E;
    const int sms = (plan.sm_budget > 0 && plan.sm_budget < plan.sms) ? plan.sm_budget : plan.sms;
    const int want = sms * (plan.ctas_per_sm > 0 ? plan.ctas_per_sm : 1);
    const int grid = ntiles < want ? ntiles : want;
    if constexpr (!D::STREAM) {
        if (plan.variant == SplitPlan::PIPE && sa.qbulk) return launch_split_pipe<N>(sa, grid, s);
    }
    euler_stage_split_kernel<N><<<grid, D::THREADS, D::SMEM, s>>>(sa);
    return cudaGetLastError();
}

cudaError_t launch_euler_split(int N, const EulerArgs& a, const SplitPlan& plan, cudaStream_t s) {
    if (!plan.ready || plan.N != N) return cudaErrorNotSupported;
    switch (N) {
        case 1: return launch_split_n<1>(a, plan, s);
        case 2: return launch_split_n<2>(a, plan, s);
        case 3: return launch_split_n<3>(a, plan, s);
        case 4: return launch_split_n<4>(a, plan, s);
        case 5: return launch_split_n<5>(a, plan, s);
        case 6: return launch_split_n<6>(a, plan, s);
        case 7: return launch_split_n<7>(a, plan, s);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace dgk

int split_setup(dg_ctx* c) {
    c->split.ready = false;
    switch (c->N) {
        case 1: return dgk::setup_n<1>(c);
        case 2: return dgk::setup_n<2>(c);
        case 3: return dgk::setup_n<3>(c);
        case 4: return dgk::setup_n<4>(c);
        case 5: return dgk::setup_n<5>(c);
        case 6: return dgk::setup_n<6>(c);
        case 7: return dgk::setup_n<7>(c);
        default: return DG_ERR_UNSUPPORTED;
    }
}

void split_teardown(dg_ctx* c) {
    if (c->split.d_ops) cudaFree(c->split.d_ops);
    if (c->split.d_status) cudaFree(c->split.d_status);
    if (c->split.d_res32) cudaFree(c->split.d_res32);
    c->split.d_ops = nullptr;
    c->split.d_status = nullptr;
    c->split.d_res32 = nullptr;
    c->split.ready = false;
}
