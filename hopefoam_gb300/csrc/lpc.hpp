// lpc.hpp -- learned element-block preconditioner for the SIPG PCG.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "ipdg.hpp"

namespace dgk {

struct SchwarzArgs;

// z_k = (P r)_k + s_k * W2 relu(W1 x_k / s_k)   with the feature vector
// x_k = [(P r)_k, rotated (P r) of the 3 neighbours, 4 scaled metrics]
struct LpcNet {
    int F = 0;       // features = 4 Np + 4
    int H = 128;     // hidden width
    int linear = 0;  // 1: identity activation and no metric features, so M(r) is linear in r
    int Np = 0;      // outputs
    const __nv_bfloat16* W1 = nullptr;  // H x F (BF16 copy used by the kernels)
    const __nv_bfloat16* W2 = nullptr;  // Np x H
    const int* perm = nullptr;          // 3 x Np ring-order node permutation per neighbour face
    const SchwarzArgs* sw = nullptr;  // learned additive-Schwarz form (then W1/W2 unused)
    float* U = nullptr;                      // its per-element local outputs (K x 4 Np)
};

struct LpcFeatArgs {
    int K, Np;
    int linear;           // metric features zero (linear preconditioner)
    const double* zb;     // block-Jacobi output, ring order, K x Np
    const int* conn;      // packed neighbours
    const double* geo;    // metrics
    const int* perm;      // 3 x Np
};

// features X (K x F, BF16) and per-element scale s (K) from zb
cudaError_t launch_lpc_features(const LpcFeatArgs& a, __nv_bfloat16* X, float* s, cudaStream_t st);
// targets T (K x Np) = (e - zb) / s
cudaError_t launch_lpc_targets(const double* e, const double* zb, const float* s, int K, int Np, float* T,
                               cudaStream_t st);
// training step pieces on a batch of B samples (rows of X, T)
cudaError_t launch_lpc_forward(const LpcNet& n, const __nv_bfloat16* X, const float* T, int B, float* Hs, float* dY,
                               double* loss_part, int G, cudaStream_t st);
cudaError_t launch_lpc_backward(const LpcNet& n, const __nv_bfloat16* X, const float* Hs, const float* dY, int B,
                                float* gW1, float* gW2, cudaStream_t st);
cudaError_t launch_lpc_adam(float* W, float* m, float* v, const float* g, __nv_bfloat16* Wb, int n, float lr,
                            float b1, float b2, float eps, int step, float gscale, cudaStream_t st);
// z = zb + s y
cudaError_t launch_lpc_combine(const double* zb, const float* s, const float* y, int K, int Np, double* z,
                               cudaStream_t st);
// dY = s ((a/b) w - r) with a, b the sums of G partials each (energy-loss output gradient)
cudaError_t launch_lpc_energy_dy(const double* r, const double* w, const float* s, const double* part_a,
                                 const double* part_b, int G, int K, int Np, float* dY, cudaStream_t st);
// inference: z = zb + s * MLP(x); the CG scalars completed depend on mode
enum { LPC_APPLY = 0, LPC_PCG_INIT = 1, LPC_PCG_REFRESH = 2, LPC_PCG_ITERATION = 3 };
// dz (may be null): FP32 offset mirror of z (z minus the element's first-node value)
cudaError_t launch_lpc_precond(const LpcNet& n, const LpcFeatArgs& fa, const double* r, double* z, int mode,
                               PcgScalars* S, double* part, float* dz, cudaStream_t st);

// learned additive-Schwarz form: M r = P r + sum_m G_m^T W^T W G_m r, or with
// mlp = 1 the two-layer network with tied weights M r = P r + sum_m G_m^T W^T relu(W G_m r)
constexpr int kSchwarzMaxH = 128;
constexpr int kSchwarzMlpH = 128;
struct SchwarzArgs {
    int K, Np, H, sms;
    const __nv_bfloat16* W;  // H x 4 Np
    const int* conn;         // packed neighbours
    const int* perm;         // 3 x Np: node permutation that rotates a neighbour's face fn onto face 0
    const int* iperm;        // 3 x Np: inverse of perm
    int* tc_status;          // non-null: run the local stage on the tensor cores (H = 32, or mlp); timeout flag
    int mlp;                 // 1: (leaky) relu between the two layers (H = 128, BF16 tensor-core kernels)
    int flex;                // 1: the collect step also forms r.z_old (flexible beta: M is not linear)
    float slope;             // mlp: activation max(h, slope h), slope in [0, 1] (0: relu)
};
// tensor-core local stage (schwarz_tc.cu); cudaErrorNotSupported when H != 32 or N > 6
cudaError_t launch_schwarz_local_tc(const SchwarzArgs& a, const double* r, const float* r32, float* U,
                                    const int* done, int* status, cudaStream_t st);
// r32 (may be null): FP32 copy of r, read instead of r
cudaError_t launch_schwarz_local(const SchwarzArgs& a, const double* r, const float* r32, float* U, const int* done,
                                 cudaStream_t st);
// z = zb + G^T U; dz (may be null): on entry the FP32 offset mirror of zb, on
// exit that of z; mode as for launch_lpc_precond
cudaError_t launch_schwarz_collect(const SchwarzArgs& a, const double* zb, const float* U, const double* r,
                                   double* z, float* dz, int mode, PcgScalars* S, double* part, cudaStream_t st);
cudaError_t launch_schwarz_gather_rows(const SchwarzArgs& a, const double* v, float* X, cudaStream_t st);
cudaError_t launch_schwarz_cross(const float* X, const float* A, int K, int F, float* C, cudaStream_t st);
cudaError_t launch_schwarz_wgrad(const float* W, const float* C, int H, int F, const double* part_a,
                                 const double* part_b, int G, float* gW, cudaStream_t st);
// two-layer (mlp) form on the tensor cores (schwarz_mlp.cu): the local stage
// U_m = W^T relu(W G_m r) (BF16 hi + lo operands, FP32 accumulation), and the
// energy-loss weight gradient: per CTA a partial sum over its patches of
// h a^T + (D W a) x^T (x = G_m r, a = G_m g, h = relu(W x), D its 0/1 mask),
// then gW = (2 a / b) times the sum over the CTAs
cudaError_t launch_schwarz_mlp_local(const SchwarzArgs& a, const double* r, const float* r32, float* U,
                                     const int* done, int* status, cudaStream_t st);
int schwarz_mlp_wgrad_ctas(const SchwarzArgs& a);
cudaError_t launch_schwarz_mlp_wgrad(const SchwarzArgs& a, const double* r, const double* g, float* part,
                                     int* status, cudaStream_t st);
cudaError_t launch_schwarz_mlp_wreduce(const float* part, int nparts, int H, int F, const double* part_a,
                                       const double* part_b, int G, float* gW, cudaStream_t st);
cudaError_t launch_schwarz_outgrad(const double* r, const double* w, const double* part_a, const double* part_b,
                                   int G, size_t n, double* g, cudaStream_t st);

}  // namespace dgk
