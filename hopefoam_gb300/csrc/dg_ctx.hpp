// dg_ctx.hpp -- the context behind the opaque dg_ctx handle.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "dg_basis.hpp"
#include "dg_internal.hpp"

namespace dgk {

// device operators and launch shape of the split-precision path
struct SplitPlan {
    bool ready = false;
    int N = 0;
    int sms = 0;
    void* d_ops = nullptr;    // operator images B1 | B2 (see euler_split.cu)
    size_t ops_bytes = 0;
    size_t b2_offset = 0;     // in floats
    size_t if32_offset = 0;   // FP32 face interpolation table, in floats
    int* d_status = nullptr;  // bounded-wait timeout flag
    float* d_res32 = nullptr; // FP32 low-storage RK register
    int ctas_per_sm = 1;      // launch shape (persistent grid = SMs used x CTAs per SM)
    int sm_budget = 0;        // SMs the grid is sized for (0: all)
    // kernel variant: tile-serial (every order) or software-pipelined across
    // tiles (N <= 6, euler_split_pipe.cu)
    enum { CLASSIC = 0, PIPE = 1 };
    int variant = CLASSIC;
};

cudaError_t launch_euler_split(int N, const EulerArgs& a, const SplitPlan& plan, cudaStream_t s);

}  // namespace dgk

struct dg_ctx {
    int K = 0, N = 0, Np = 0, Ng = 0, Nfp = 0, Nfq = 0, nb = 0;
    int device = 0;  // the CUDA device current at dg_ctx_create (every buffer lives there)
    double gamma = 1.4;
    double min_h = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    dgb::RefOps ops;
    std::vector<double> geo_host;
    std::vector<int> conn_host;
    std::vector<int> etov_host;  // [K][3] vertex ids (empty when the mesh descriptor has none)
    std::vector<double> vxy_host;  // [K][3][2] vertex coordinates
    // [2][K][Np] node locations from dg_set_node_locations (curved patches);
    // empty: the straight element's x(r, s)
    std::vector<double> node_xy_host;
    struct LimState* lim = nullptr;  // slope limiter / limited SSP-RK2 state (limiter.cu)
    // device buffers
    double* d_q[2] = {nullptr, nullptr};
    double* d_res = nullptr;
    double* d_stage = nullptr;
    double* d_geo = nullptr;
    double* d_btrace = nullptr;
    int* d_conn = nullptr;
    int* d_ring = nullptr;
    double *d_Vg = nullptr, *d_Sr = nullptr, *d_Ss = nullptr, *d_Lift = nullptr, *d_If = nullptr;
    double* d_dtk = nullptr;  // per-element time-step factors (dg_set_element_dt), null: none
    double* dtk_buf = nullptr;
    float* d_dtk32 = nullptr;  // their FP32 copy (split-precision path)
    float* dtk32_buf = nullptr;
    int cur = 0;
    bool btrace_set = false;
    dgk::SplitPlan split;
    struct IpdgState* ipdg = nullptr;
    std::vector<void*> allocs;
    size_t bytes = 0;
    std::string err;
};

int split_setup(dg_ctx* c);
void split_teardown(dg_ctx* c);

// one LSERK4 stage (0..4) of a context on c->stream, no host synchronisation
// (usable inside a stream capture); flips c->cur
int lserk_stage(dg_ctx* c, double dt, int stage, int flux, int precision);
// the arguments of that stage (from the context's current buffer parity),
// without launching or flipping anything
int lserk_stage_args(dg_ctx* c, double dt, int stage, int flux, dgk::EulerArgs* out);
// true when wall / zero-gradient slots need their traces refreshed per stage
bool has_dynamic_traces(const dg_ctx* c);
// validates flux / precision / boundary state for stepping
int check_run_args(dg_ctx* c, int flux, int precision);
// reads and clears the split kernel's timeout flag (synchronises c->stream)
int check_split_status(dg_ctx* c, int precision);
// one Euler stage kernel (mode: StageMode) from qin into qout with the given
// boundary traces (null: the context's)
int euler_stage_mode(dg_ctx* c, const double* qin, double* qout, const double* qold, int mode, double dt, int flux,
                     int precision, const double* btrace);
// limiter state teardown (limiter.cu)
void limiter_teardown(dg_ctx* c);
// traces of wall and zero-gradient slots from state q (no-op without such slots)
int refresh_boundary_traces(dg_ctx* c, const double* q);

// SIPG / PCG state (ipdg_api.cu)
namespace dgk {
struct IpdgArgs;
}
struct IpdgState;
void ipdg_teardown(dg_ctx* c);
// FP64 block-Jacobi PCG with the context's SIPG operator on ring-order device
// vectors (x: initial guess in, solution out)
int ipdg_solve_device(dg_ctx* c, const double* b_dev, double* x_dev, double rtol, int maxit, int* iters,
                      double* rel_out, int pc, int precision);
// the operator's device tables (null before dg_ipdg_setup), the boundary
// types per slot and the host copy of the face coefficients as built
const dgk::IpdgArgs* ipdg_args(dg_ctx* c);
const std::vector<int>* ipdg_btypes(dg_ctx* c);
const std::vector<double>* ipdg_face_coefs(dg_ctx* c);
