// euler_split.cuh -- shared definitions of the split-precision Euler stage
// kernels (euler_split.cu, euler_split_pipe.cu): tile sizes and the
// shared-memory layout per order, the kernel arguments, the GEMM2 row order.
#pragma once

#include <cstdint>

#include "dg_ctx.hpp"
#include "umma.cuh"

namespace dgk {

template <int N>
struct SplitDims {
    static constexpr int Np = Dims<N>::Np, Ng = Dims<N>::Ng, Nfp = Dims<N>::Nfp, Nfq = Dims<N>::Nfq;
    static constexpr int E = 32, ROWS = 128, THREADS = 512;
    static constexpr int KP1 = (Np + 7) / 8 * 8;      // GEMM1 K (padded nodes)
    static constexpr int NG = (Ng + 15) / 16 * 16;    // GEMM1 N (padded cubature points)
    static constexpr int NF = (3 * Nfq + 7) / 8 * 8;  // face-flux K
    static constexpr int KP2 = 2 * NG + NF;           // GEMM2 K
    static constexpr int NP2 = (Np + 15) / 16 * 16;   // GEMM2 N
    static constexpr int CH = 16;                     // cubature points per chunk
    static constexpr int NCH = NG / CH;
    static constexpr int KC = 2 * CH;                 // chunk buffer K: [Fr 16 | Fs 16]
    // N = 7: the volume operator [Sr|Ss] (110 KB as hi/lo) does not fit next to
    // the other operands.  It is streamed per chunk by bulk copies into
    // buffers that pair with the flux chunk buffers (only the lift part stays
    // resident), the FP64 tile copy is dropped (q is re-read from L2 in the
    // epilogue) and the face phase reads the FP32 deltas back from the TF32
    // hi + lo operand, which holds them exactly.
    static constexpr bool STREAM = (N == 7);
    static constexpr int NBUF = (N <= 5 || STREAM) ? 2 : 1;  // chunk buffers
    // N <= 5: the two buffers are filled in one pass (two chunks per thread)
    static constexpr bool PAIR = NBUF == 2 && !STREAM;
    // face phase: one (element, face) per segment of SW lanes, SPW segments per
    // warp.  Power-of-two groups (SW = 8) where packing would not save a pass
    // over the tile's 96 faces, packed segments (SW = Nfq) otherwise: at N = 7
    // two passes instead of three, at N <= 3 one instead of two.
    static constexpr bool PACKED = (N == 7) || (N <= 3);
    static constexpr int SW = PACKED ? Nfq : 8;
    static constexpr int SPW = 32 / SW;
    // N = 4..7: two Gauss points per lane, FW = ceil(Nfq / 2) lanes per face,
    // all 3 E faces of a tile in one pass
    static constexpr int FP = (STREAM || !PACKED) ? 2 : 1;
    static constexpr int FW = (Nfq + 1) / 2;
    static constexpr int FPW = 32 / FW;
    static_assert(FP == 1 || (16 * FPW >= 3 * E && 2 * FW >= Nfp), "one-pass face groups");
    // shared-memory layout (bytes, operand buffers 1024-aligned)
    static constexpr int SZ_B1 = 2 * NG * KP1 * 4;    // Vg hi/lo
    static constexpr int SZ_BC = 2 * NP2 * KC * 4;    // one streamed [Sr|Ss] chunk hi/lo
    static constexpr int SZ_B2 = STREAM ? 2 * NP2 * NF * 4    // Lift hi/lo
                                        : 2 * NP2 * KP2 * 4;  // [Sr|Ss|Lift] hi/lo
    static constexpr int SZ_A1 = 2 * ROWS * KP1 * 4;  // dQ hi/lo
    static constexpr int SZ_AC = 2 * ROWS * KC * 4;   // one flux chunk hi/lo
    static constexpr int SZ_AF = 2 * ROWS * NF * 4;   // face flux hi/lo
    static constexpr int SZ_QF = STREAM ? 0 : E * 4 * Np * 4;   // FP32 deltas of the tile state
    static constexpr int SZ_Q64 = STREAM ? 0 : E * 4 * Np * 8;  // FP64 tile state
    // reference state FP32 (+ FP64 copy on the resident path), FP32 metrics
    static constexpr int OFF_GEO_IN_QB = ROWS * 4 + (STREAM ? 0 : ROWS * 8);
    static constexpr int SZ_QB = OFF_GEO_IN_QB + E * 4 * 4;
    // the neighbour traces of the tile's faces, FP64 [3 E][Nfp][4], gathered
    // by asynchronous copies while the tile is staged, where shared memory
    // has room for them (N <= 5); otherwise the face phase loads them itself
    static constexpr int SZ_NB_FULL = 3 * E * Nfp * 4 * 8;
    static constexpr int al(int x) { return (x + 1023) / 1024 * 1024; }
    static constexpr int OFF_B1 = 0;
    static constexpr int OFF_B2 = OFF_B1 + al(SZ_B1);
    static constexpr int AL_BC = al(SZ_BC);           // stride between streamed operand buffers
    static constexpr int OFF_BC = OFF_B2 + al(SZ_B2);
    static constexpr int OFF_A1 = OFF_BC + (STREAM ? NBUF * AL_BC : 0);
    static constexpr int OFF_AC = OFF_A1 + al(SZ_A1);
    static constexpr int AL_AC = al(SZ_AC);           // stride between chunk buffers
    static constexpr int OFF_AF = OFF_AC + NBUF * AL_AC;
    static constexpr int OFF_QF = OFF_AF + al(SZ_AF);
    static constexpr int OFF_Q64 = OFF_QF + al(SZ_QF);
    static constexpr int OFF_QB = OFF_Q64 + al(SZ_Q64);
    static constexpr int OFF_NB = OFF_QB + al(SZ_QB);
    static constexpr bool GATHER = !STREAM && OFF_NB + al(SZ_NB_FULL) + 64 <= 232448;
    static constexpr int SZ_NB = GATHER ? SZ_NB_FULL : 0;
    static constexpr int OFF_BAR = OFF_NB + al(SZ_NB);
    static constexpr int SMEM = OFF_BAR + 64;
    static constexpr int RS_FLOATS = E * 4 * Np;      // epilogue staging (aliases chunk buffer 0)
    static constexpr int TILE_VALS = E * 4 * Np;
    static constexpr int EPI = (TILE_VALS + THREADS - 1) / THREADS;  // tile values per thread
    static_assert(RS_FLOATS * 4 <= SZ_AC, "epilogue staging does not fit");
    static_assert(SMEM <= 232448, "shared memory budget");
    static_assert(Nfq <= SW && Nfp <= SW, "face segment width");
    static_assert(!STREAM || NBUF == 2, "streamed operand buffers pair with two chunk buffers");
    static constexpr int TMEM_COLS = 256;
    static constexpr int D2_COL = 128;
    static_assert(NG <= 128 && NP2 <= 128, "tensor memory layout");
};

struct SplitArgs {
    EulerArgs e;
    const float* res32;  // FP32 low-storage RK register (read)
    float* res32_out;    // (write, may alias res32: element-local)
    const float* b1;     // device image of B1 (canonical layout, hi then lo)
    const float* b2;     // device image of B2
    int* status;         // nonzero on a bounded-wait timeout
    int qbulk;           // N <= 6: the state is 16-byte aligned, tiles arrive by bulk copy
    // FP32 forms of the stage's scalars and tables, prepared on the host so
    // that no thread converts them (FP64 <-> FP32 conversions occupy the FP64
    // pipe, two thread-operations per clock per SM on GB300)
    const float* If32;   // face interpolation Nfq x Nfp
    const float* dtk32;  // per-element time-step factors (null: none)
    float rkaf, rkbf, dtf;
    int first;           // LSERK stage with a = 0 (the register is not read)
};

constexpr uint32_t kWaitLimit = 1u << 22;

// GEMM2's A rows (and so its result rows in tensor memory) in the order
// r = 32 (e / 8) + 8 v + e % 8: the 8 elements a warp stores for one variable
// then sit in 8 different 16-byte slots of a core matrix, so the operand
// stores are free of bank conflicts.  GEMM1 keeps r = 4 e + v.
__device__ __forceinline__ int g2row(int e, int v) { return ((e >> 3) << 5) | (v << 3) | (e & 7); }

// one stage of several contexts (orders 1..6, pipelined body) in one launch:
// group g runs on blocks [cta_end[g-1], cta_end[g])
struct SplitBatchArgs {
    static constexpr int MAXG = 8;
    SplitArgs sa[MAXG];
    int order[MAXG];
    int cta_end[MAXG];
    int ngroups;
};
cudaError_t setup_split_batch();
cudaError_t launch_split_batch(const SplitBatchArgs& P, cudaStream_t s);

// the stage's kernel arguments from the context-level ones (FP32 scalars, tables)
int split_fill_args(const EulerArgs& a, const SplitPlan& plan, SplitArgs* sa);

// the pipelined variant of the stage (euler_split_pipe.cu) for N <= 6: the
// next tile's staging runs under this tile's volume phase and its face phase
// under this tile's epilogue
template <int N>
cudaError_t launch_split_pipe(const SplitArgs& sa, int grid, cudaStream_t s);
template <int N>
cudaError_t setup_split_pipe();

}  // namespace dgk
