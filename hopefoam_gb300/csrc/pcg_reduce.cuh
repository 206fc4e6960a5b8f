// pcg_reduce.cuh -- deterministic grid-wide sums and the device-side CG
// scalar updates shared by the SIPG PCG kernels and the learned
// preconditioner kernel.
//
// grid_sum: every CTA reduces its values (fixed warp order), stores them in
// part[q * nblk + blockIdx.x], and the last CTA to arrive (atomic counter,
// threadfence before the arrival) sums the partials in index order.  The
// result does not depend on the arrival order, so solves are bit-reproducible.
// One reduction at a time: the kernels that use it are stream-ordered, so a
// single counter (reset by the last CTA) serves them all.
#pragma once

#include <cuda_runtime.h>

#include "ipdg.hpp"

namespace dgk {

// fixed-order sum over the CTA of NV values per thread (blockDim.x a power
// of two <= 256): a shared-memory halving tree, blockDim.x - 1 additions per
// value.  (A warp butterfly would cost 5 FP64 additions per thread and value,
// and FP64 issue is scarce on this GPU.)  Result in red[q][0].
template <int NV>
__device__ __forceinline__ void block_tree(double (&val)[NV], double (&red)[NV][256]) {
    const int t = threadIdx.x;
#pragma unroll
    for (int q = 0; q < NV; q++) red[q][t] = val[q];
    __syncthreads();
    for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
        if (t < s) {
#pragma unroll
            for (int q = 0; q < NV; q++) red[q][t] += red[q][t + s];
        }
        __syncthreads();
    }
}

template <int NV>
__device__ __forceinline__ bool grid_sum(double (&val)[NV], double* part, int nblk, unsigned int* counter,
                                         double (&out)[NV]) {
    __shared__ double red[NV][256];
    __shared__ int s_last;
    block_tree<NV>(val, red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) part[(size_t)q * nblk + blockIdx.x] = red[q][0];
        __threadfence();
        const unsigned int t = atomicAdd(counter, 1u);
        s_last = (t == (unsigned int)nblk - 1u);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    // last CTA: fixed-order sum of all partials (L2 reads: other CTAs wrote them)
    double acc[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) {
        double s = 0;
        for (int i = threadIdx.x; i < nblk; i += blockDim.x) s += __ldcg(part + (size_t)q * nblk + i);
        acc[q] = s;
    }
    block_tree<NV>(acc, red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) out[q] = red[q][0];
        *counter = 0u;
    }
    return true;  // out[] valid in thread 0
}

// CG scalars after a new residual r (recurrence) and preconditioned z:
// beta = (r.z - rzo) / r_old.z_old with rzo = r.z_old for the flexible
// (Polak-Ribiere) form of a nonlinear preconditioner, 0 for the standard form;
// stop test on r.r.  Thread 0 of the last CTA only.
__device__ __forceinline__ void pcg_finish(PcgScalars* S, double rz_new, double rzo, double rr) {
    const double rz_old = S->rz;
    int stop = 0;
    if (!(rr == rr) || !(rz_new == rz_new) || !(rzo == rzo) || rz_old == 0.0) stop = 2;
    else if (rr <= S->tol2) stop = 1;
    S->beta = (rz_new - rzo) / rz_old;
    S->rz = rz_new;
    S->rr = rr;
    S->it += 1;
    if (stop) S->done = stop;
}

}  // namespace dgk
