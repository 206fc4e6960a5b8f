// euler_noalloc.cu -- allocation-free variant of the FP64 Euler right-hand side.
//
// dg_euler_rhs stages its data through buffers the context allocated with
// cudaMalloc.  This entry point does the same work without touching the
// allocator: the two scratch buffers it needs (the state in the kernel's
// internal layout and the right-hand side before it is put back into the
// reference layout) live in one fixed-size array of device global memory
// declared at file scope.  It exists for callers that must not allocate while
// they run: code inside a stream capture, where cudaMalloc breaks the
// capture; applications whose device memory is owned by a pool allocator or
// another framework and may not be grown behind its back; and loops with a
// real-time budget, where an allocation's latency or failure is not allowed.
//
// Boundary slots: fixed-value slots use the traces set on the context; wall
// and zero-gradient slots (dg_set_boundary_kinds) are recomputed from q_dev
// into the context's trace buffer, as dg_euler_rhs does from the context's
// state.
//
// Limits: 4 * K * Np <= DG_NOALLOC_MAX_VALUES (524288 values, 4 MiB per
// buffer, 8 MiB in total).  Every GPU that loads this library keeps the array
// until the process exits.  All calls share the array and it keeps the last
// call's contents (each call overwrites every value it reads, so nothing has
// to start at zero); calls whose GPU work overlaps in time race on it.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/dgcu.h"
#include "dg_ctx.hpp"

namespace {

constexpr size_t kMaxValues = (size_t)1 << 19;  // DG_NOALLOC_MAX_VALUES

// [0, kMaxValues): state, internal layout; [kMaxValues, 2 kMaxValues): right-hand side
static __device__ __align__(256) double g_noalloc_scratch[2 * kMaxValues];

constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;

// Device address of the scratch array on the current device, looked up once
// per device (host code must not use the symbol itself as a pointer).
cudaError_t scratch_address(int dev, double** out) {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

int nfail(dg_ctx* c, int code, const std::string& m) {
    c->err = m;
    return code;
}

}  // namespace

extern "C" int dg_euler_rhs_noalloc(dg_ctx* c, const double* q_dev, double* rhs_dev, int flux) {
    if (!c) return DG_ERR_ARG;
    if (!q_dev || !rhs_dev) return nfail(c, DG_ERR_ARG, "dg_euler_rhs_noalloc: null device pointer");
    if (flux != DG_FLUX_LF && flux != DG_FLUX_ROE) return nfail(c, DG_ERR_ARG, "dg_euler_rhs_noalloc: unknown flux");
    const size_t n = (size_t)c->K * 4 * c->Np;
    if (n > kMaxValues)
        return nfail(c, DG_ERR_ARG,
                     "dg_euler_rhs_noalloc: 4*K*Np = " + std::to_string(n) +
                         " exceeds the fixed scratch of 524288 values; use dg_euler_rhs");
    if (c->nb > 0 && !c->btrace_set) return nfail(c, DG_ERR_ARG, "boundary traces not set");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nfail(c, DG_ERR_CUDA, "cudaGetDevice failed");
    // the scratch address is per device: another device's would be a foreign
    // address for the kernels queued on this context's stream
    if (dev != c->device)
        return nfail(c, DG_ERR_ARG, "dg_euler_rhs_noalloc: the context's device (" + std::to_string(c->device) +
                                        ") is not the current device (" + std::to_string(dev) + ")");
    double* scratch = nullptr;
    e = scratch_address(dev, &scratch);
    if (e != cudaSuccess) return nfail(c, DG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    double* q_int = scratch;
    double* rhs_int = scratch + kMaxValues;
    e = dgk::launch_to_internal(q_dev, q_int, c->d_ring, c->K, c->Np, c->stream);
    if (e != cudaSuccess) return nfail(c, DG_ERR_CUDA, std::string("to_internal: ") + cudaGetErrorString(e));
    // wall and zero-gradient slots take their traces from this state (a kernel
    // writing the context's own trace buffer: no allocation)
    const int rc = refresh_boundary_traces(c, q_int);
    if (rc) return rc;
    dgk::EulerArgs a;
    memset(&a, 0, sizeof(a));
    a.qin = q_int;
    a.rhs = rhs_int;
    a.geo = c->d_geo;
    a.conn = c->d_conn;
    a.btrace = c->d_btrace;
    a.ops = dgk::EulerOps{c->d_Vg, c->d_Sr, c->d_Ss, c->d_Lift, c->d_If};
    a.K = c->K;
    a.flux = flux;
    a.mode = dgk::MODE_RHS;
    a.gamma = c->gamma;
    e = dgk::launch_euler_fp64(c->N, a, c->stream);
    if (e != cudaSuccess) return nfail(c, DG_ERR_CUDA, std::string("euler rhs: ") + cudaGetErrorString(e));
    e = dgk::launch_to_reference(rhs_int, rhs_dev, c->d_ring, c->K, c->Np, c->stream);
    if (e != cudaSuccess) return nfail(c, DG_ERR_CUDA, std::string("to_reference: ") + cudaGetErrorString(e));
    return DG_OK;
}
