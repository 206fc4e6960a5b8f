// lpc.cu -- learned element-block preconditioner: features, BF16 training
// kernels (BF16 operands, FP32 accumulation, FP32 master weights with Adam)
// and the inference kernel used inside the flexible PCG.
//
// Network (no biases, so it is positively homogeneous: M(a r) = a M(r), a > 0):
//   x_k   = [z_k, Rot(z_n0), Rot(z_n1), Rot(z_n2)] / s_k  ++  h_k (rx, sx, ry, sy)
//   z_k  <- z_k + s_k W2 relu(W1 x_k)
// with z = P r the block-Jacobi output, Rot the node permutation that turns a
// neighbour's shared face into its face 0 (3-fold symmetry of the node set),
// s_k the RMS of the element's 4 z blocks and h_k = sqrt(J_k).  Trained on
// (r, e) pairs from the method's own PCG solves: target (e_k - z_k) / s_k.
#include <cuda_bf16.h>

#include "lpc.hpp"
#include "pcg_reduce.cuh"

namespace dgk {

__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16(x)); }

// features of element k into x[0..F) (FP32) and its scale; returns s
__device__ __forceinline__ float lpc_element_features(const LpcFeatArgs& a, int k, float* x) {
    const int Np = a.Np;
    const double* zk = a.zb + (size_t)k * Np;
    double ss = 0;
    for (int i = 0; i < Np; i++) {
        x[i] = (float)zk[i];
        ss += zk[i] * zk[i];
    }
    for (int f = 0; f < 3; f++) {
        const int c = a.conn[(size_t)k * 3 + f];
        float* xf = x + (f + 1) * Np;
        if (c >= 0) {
            const int nb = c >> 3, fn = c & 3;
            const double* zn = a.zb + (size_t)nb * Np;
            const int* pm = a.perm + fn * Np;
            for (int i = 0; i < Np; i++) {
                const double v = zn[pm[i]];
                xf[i] = (float)v;
                ss += v * v;
            }
        } else {
            for (int i = 0; i < Np; i++) xf[i] = 0.f;
        }
    }
    const float s = (float)sqrt(ss / (4.0 * Np)) + 1e-30f;
    const float inv = 1.f / s;
    for (int i = 0; i < 4 * Np; i++) x[i] *= inv;
    const double* g = a.geo + (size_t)k * 4;
    const double J = 1.0 / (g[0] * g[3] - g[1] * g[2]);
    const double h = sqrt(J);
    const float gm = a.linear ? 0.f : 1.f;  // the linear form takes no (scale-free) metric input
    x[4 * Np + 0] = gm * (float)(g[0] * h);
    x[4 * Np + 1] = gm * (float)(g[1] * h);
    x[4 * Np + 2] = gm * (float)(g[2] * h);
    x[4 * Np + 3] = gm * (float)(g[3] * h);
    return s;
}

constexpr int kMaxF = 4 * 36 + 4;

__global__ void lpc_features_kernel(LpcFeatArgs a, __nv_bfloat16* __restrict__ X, float* __restrict__ s) {
    const int F = 4 * a.Np + 4;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < a.K; k += gridDim.x * blockDim.x) {
        float x[kMaxF];
        s[k] = lpc_element_features(a, k, x);
        for (int i = 0; i < F; i++) X[(size_t)k * F + i] = __float2bfloat16(x[i]);
    }
}

__global__ void lpc_targets_kernel(const double* __restrict__ e, const double* __restrict__ zb,
                                   const float* __restrict__ s, int K, int Np, float* __restrict__ T) {
    const size_t n = (size_t)K * Np;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / Np);
        T[t] = (float)((e[t] - zb[t]) / (double)s[k]);
    }
}

// forward on a batch: Hs[b][h] = bf16(relu(W1 x_b)), dY[b][j] = W2 Hs_b - T_b (T null: the
// network output itself); loss partials.
// CTA = 128 threads, 32 samples per tile, grid-stride over tiles.
__global__ void lpc_forward_kernel(LpcNet n, const __nv_bfloat16* __restrict__ X, const float* __restrict__ T, int B,
                                   float* __restrict__ Hs, float* __restrict__ dY, double* __restrict__ part) {
    extern __shared__ float fsm[];
    const int F = n.F, H = n.H, Np = n.Np;
    float* xs = fsm;             // [32][F]
    float* hs = xs + 32 * F;     // [32][H]
    __shared__ double red[4];
    double loss = 0;
    const int ntiles = (B + 31) / 32;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int b0 = tile * 32, nb = min(32, B - b0);
        for (int i = threadIdx.x; i < nb * F; i += blockDim.x) xs[i] = __bfloat162float(X[(size_t)b0 * F + i]);
        __syncthreads();
        for (int it = threadIdx.x; it < nb * H; it += blockDim.x) {
            const int sidx = it / H, h = it - sidx * H;
            const __nv_bfloat16* w = n.W1 + (size_t)h * F;
            float acc = 0.f;
            for (int k = 0; k < F; k++) acc = fmaf(__bfloat162float(w[k]), xs[sidx * F + k], acc);
            const float hv = bf(n.linear ? acc : fmaxf(acc, 0.f));
            hs[sidx * H + h] = hv;
            Hs[(size_t)(b0 + sidx) * H + h] = hv;
        }
        __syncthreads();
        for (int it = threadIdx.x; it < nb * Np; it += blockDim.x) {
            const int sidx = it / Np, j = it - sidx * Np;
            const __nv_bfloat16* w = n.W2 + (size_t)j * H;
            float acc = 0.f;
            for (int h = 0; h < H; h++) acc = fmaf(__bfloat162float(w[h]), hs[sidx * H + h], acc);
            const float d = T ? acc - T[(size_t)(b0 + sidx) * Np + j] : acc;
            dY[(size_t)(b0 + sidx) * Np + j] = d;
            loss += (double)d * d;
        }
        __syncthreads();
    }
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = loss;
    __syncthreads();
    if (threadIdx.x == 0) part[blockIdx.x] = red[0] + red[1] + red[2] + red[3];
}

// dH[b][h] = (W2^T dY_b)_h * (Hs[b][h] > 0), written over Hs' companion buffer
__global__ void lpc_dh_kernel(LpcNet n, const float* __restrict__ Hs, const float* __restrict__ dY, int B,
                              float* __restrict__ dH) {
    const int H = n.H, Np = n.Np;
    const size_t tot = (size_t)B * H;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tot; t += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(t / H), h = (int)(t - (size_t)b * H);
        float acc = 0.f;
        if (n.linear || Hs[t] > 0.f)
            for (int j = 0; j < Np; j++) acc = fmaf(__bfloat162float(n.W2[(size_t)j * H + h]), dY[(size_t)b * Np + j], acc);
        dH[t] = bf(acc);
    }
}

// gW2[j][h] = sum_b dY[b][j] Hs[b][h] / B ; gW1[h][k] = sum_b dH[b][h] X[b][k] / B
__global__ void lpc_gw_kernel(LpcNet n, const __nv_bfloat16* __restrict__ X, const float* __restrict__ Hs,
                              const float* __restrict__ dY, const float* __restrict__ dH, int B,
                              float* __restrict__ gW1, float* __restrict__ gW2) {
    const int F = n.F, H = n.H, Np = n.Np;
    const int n1 = H * F, n2 = Np * H;
    const float invB = 1.f / (float)B;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n1 + n2; t += gridDim.x * blockDim.x) {
        float acc = 0.f;
        if (t < n1) {
            const int h = t / F, k = t - h * F;
            for (int b = 0; b < B; b++) acc = fmaf(dH[(size_t)b * H + h], __bfloat162float(X[(size_t)b * F + k]), acc);
            gW1[t] = acc * invB;
        } else {
            const int u = t - n1, j = u / H, h = u - j * H;
            for (int b = 0; b < B; b++) acc = fmaf(dY[(size_t)b * Np + j], Hs[(size_t)b * H + h], acc);
            gW2[u] = acc * invB;
        }
    }
}

__global__ void lpc_adam_kernel(float* W, float* m, float* v, const float* g, __nv_bfloat16* Wb, int n, float lr,
                                float b1, float b2, float eps, int step, float gscale) {
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i] * gscale;
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float w = W[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        W[i] = w;
        Wb[i] = __float2bfloat16(w);
    }
}

// PCG preconditioner: z_k = zb_k + s_k W2 relu(W1 x_k), with the CG scalars
// it completes (mode): LPC_APPLY none; LPC_PCG_INIT / LPC_PCG_REFRESH S->rz;
// LPC_PCG_ITERATION beta and the stop test (r.z, r.z_old, S->rr).
// Weights staged in shared memory (BF16); one thread per element; grid-stride.
__global__ void lpc_precond_kernel(LpcNet n, LpcFeatArgs a, const double* __restrict__ r, double* __restrict__ z,
                                   int mode, PcgScalars* S, double* part, float* __restrict__ dz) {
    extern __shared__ __nv_bfloat16 wsm[];
    if (mode == LPC_PCG_ITERATION && S->done) return;
    const int F = n.F, H = n.H, Np = n.Np;
    __nv_bfloat16* w1 = wsm;
    __nv_bfloat16* w2 = wsm + H * F;
    for (int i = threadIdx.x; i < H * F; i += blockDim.x) w1[i] = n.W1[i];
    for (int i = threadIdx.x; i < Np * H; i += blockDim.x) w2[i] = n.W2[i];
    __syncthreads();
    double rz = 0, rzo = 0;
    const int nthr = gridDim.x * blockDim.x;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < a.K; k += nthr) {
        float x[kMaxF];
        const float s = lpc_element_features(a, k, x);
        for (int i = 0; i < F; i++) x[i] = bf(x[i]);
        float y[36];
        for (int j = 0; j < Np; j++) y[j] = 0.f;
        for (int h = 0; h < H; h++) {
            const __nv_bfloat16* wr = w1 + h * F;
            float acc = 0.f;
            for (int i = 0; i < F; i++) acc = fmaf(__bfloat162float(wr[i]), x[i], acc);
            const float hv = bf(n.linear ? acc : fmaxf(acc, 0.f));
            for (int j = 0; j < Np; j++) y[j] = fmaf(__bfloat162float(w2[j * H + h]), hv, y[j]);
        }
        const double* zbk = a.zb + (size_t)k * Np;
        const double* rk = r + (size_t)k * Np;
        double* zk = z + (size_t)k * Np;
        const double z0 = zbk[0] + (double)s * (double)y[0];
        for (int j = 0; j < Np; j++) {
            const double zn = zbk[j] + (double)s * (double)y[j];
            if (mode == LPC_PCG_ITERATION) rzo += rk[j] * zk[j];
            rz += rk[j] * zn;
            zk[j] = zn;
            if (dz) dz[(size_t)k * Np + j] = (float)(zn - z0);
        }
    }
    if (mode == LPC_APPLY) return;
    double val[2] = {rz, rzo}, tot[2];
    if (grid_sum<2>(val, part, gridDim.x, &S->counter, tot) && threadIdx.x == 0) {
        if (mode == LPC_PCG_ITERATION) pcg_finish(S, tot[0], tot[1], S->rr);
        else S->rz = tot[0];
    }
}

// z = zb + s y (the preconditioner output the PCG uses), ring order
__global__ void lpc_combine_kernel(const double* __restrict__ zb, const float* __restrict__ s,
                                   const float* __restrict__ y, int K, int Np, double* __restrict__ z) {
    const size_t n = (size_t)K * Np;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / Np);
        z[t] = zb[t] + (double)s[k] * (double)y[t];
    }
}

// output gradient of the energy loss L = -(r.z)|r.z| / (z.Sz): dL/dz is a
// positive multiple (2|a|/b) of (a/b) Sz - r (a = r.z, b = z.Sz, each reduced
// from G partials); chained through z = zb + s y: dY = s ((a/b) w - r)
__global__ void lpc_energy_dy_kernel(const double* __restrict__ r, const double* __restrict__ w,
                                     const float* __restrict__ s, const double* __restrict__ part_a,
                                     const double* __restrict__ part_b, int G, int K, int Np,
                                     float* __restrict__ dY) {
    __shared__ double s_ab;
    if (threadIdx.x < 32) {
        double a = 0, b = 0;
        for (int i = threadIdx.x; i < G; i += 32) { a += part_a[i]; b += part_b[i]; }
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        if (threadIdx.x == 0) s_ab = (b > 0) ? a / b : 0.0;
    }
    __syncthreads();
    const double ab = s_ab;
    const size_t n = (size_t)K * Np;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / Np);
        dY[t] = (float)((double)s[k] * (ab * w[t] - r[t]));
    }
}

cudaError_t launch_lpc_combine(const double* zb, const float* s, const float* y, int K, int Np, double* z,
                               cudaStream_t st) {
    lpc_combine_kernel<<<608, 256, 0, st>>>(zb, s, y, K, Np, z);
    return cudaGetLastError();
}

cudaError_t launch_lpc_energy_dy(const double* r, const double* w, const float* s, const double* part_a,
                                 const double* part_b, int G, int K, int Np, float* dY, cudaStream_t st) {
    lpc_energy_dy_kernel<<<608, 256, 0, st>>>(r, w, s, part_a, part_b, G, K, Np, dY);
    return cudaGetLastError();
}

cudaError_t launch_lpc_features(const LpcFeatArgs& a, __nv_bfloat16* X, float* s, cudaStream_t st) {
    lpc_features_kernel<<<(a.K + 127) / 128, 128, 0, st>>>(a, X, s);
    return cudaGetLastError();
}

cudaError_t launch_lpc_targets(const double* e, const double* zb, const float* s, int K, int Np, float* T,
                               cudaStream_t st) {
    lpc_targets_kernel<<<608, 256, 0, st>>>(e, zb, s, K, Np, T);
    return cudaGetLastError();
}

cudaError_t launch_lpc_forward(const LpcNet& n, const __nv_bfloat16* X, const float* T, int B, float* Hs, float* dY,
                               double* loss_part, int G, cudaStream_t st) {
    const size_t smem = sizeof(float) * 32 * (n.F + n.H);
    lpc_forward_kernel<<<G, 128, smem, st>>>(n, X, T, B, Hs, dY, loss_part);
    return cudaGetLastError();
}

cudaError_t launch_lpc_backward(const LpcNet& n, const __nv_bfloat16* X, const float* Hs, const float* dY, int B,
                                float* gW1, float* gW2, cudaStream_t st) {
    // dH is stored in the second half of the Hs buffer (caller allocates 2 x B x H)
    float* dH = const_cast<float*>(Hs) + (size_t)B * n.H;
    lpc_dh_kernel<<<608, 256, 0, st>>>(n, Hs, dY, B, dH);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    lpc_gw_kernel<<<(n.H * n.F + n.Np * n.H + 127) / 128, 128, 0, st>>>(n, X, Hs, dY, dH, B, gW1, gW2);
    return cudaGetLastError();
}

cudaError_t launch_lpc_adam(float* W, float* m, float* v, const float* g, __nv_bfloat16* Wb, int n, float lr, float b1,
                            float b2, float eps, int step, float gscale, cudaStream_t st) {
    lpc_adam_kernel<<<(n + 255) / 256, 256, 0, st>>>(W, m, v, g, Wb, n, lr, b1, b2, eps, step, gscale);
    return cudaGetLastError();
}

cudaError_t launch_lpc_precond(const LpcNet& n, const LpcFeatArgs& fa, const double* r, double* z, int mode,
                               PcgScalars* S, double* part, float* dz, cudaStream_t st) {
    const size_t smem = sizeof(__nv_bfloat16) * (size_t)(n.H * n.F + n.Np * n.H);
    lpc_precond_kernel<<<608, 128, smem, st>>>(n, fa, r, z, mode, S, part, dz);
    return cudaGetLastError();
}

}  // namespace dgk

// ---------------------------------------------------------------------------
// Learned additive-Schwarz form (SPD by construction):
//   M r = P r + sum_m G_m^T W^T W G_m r
// G_m gathers the residual on element m and its three face neighbours (each
// neighbour rotated so that the shared face is its face 0; zero across a
// boundary), F = 4 Np values; W (H x F) is stored in BF16, activations are
// FP32, so M is exactly linear and symmetric positive definite and plain CG
// applies.  The transpose is computed by the owner: element k collects its
// own slot of U_k = W^T W G_k r and, through each face f with neighbour m
// (m's face fn), the entries of m's slot fn + 1 at the node permutation of
// face f.

namespace dgk {

namespace {

// x = G_m v (FP32) for element m
__device__ __forceinline__ void schwarz_gather(const SchwarzArgs& a, const double* __restrict__ v, int m, float* x) {
    const int Np = a.Np;
    const double* vm = v + (size_t)m * Np;
    for (int i = 0; i < Np; i++) x[i] = (float)vm[i];
    for (int f = 0; f < 3; f++) {
        const int c = a.conn[(size_t)m * 3 + f];
        float* xf = x + (f + 1) * Np;
        if (c >= 0) {
            const double* vn = v + (size_t)(c >> 3) * Np;
            const int* pm = a.perm + (c & 3) * Np;
            for (int i = 0; i < Np; i++) xf[i] = (float)vn[pm[i]];
        } else {
            for (int i = 0; i < Np; i++) xf[i] = 0.f;
        }
    }
}

}  // namespace

// U[m] = W^T (W G_m r); W staged in shared memory (FP32 from the BF16 copy);
// one thread per element, Np and H compile-time so x and h stay in registers
template <int NP, int H>
struct SchwarzLocalDims {
    static constexpr int THREADS = H > 32 ? 64 : 128;  // static shared memory stays under 48 KB
    static constexpr int MIN_BLOCKS = NP <= 15 ? (H > 32 ? 10 : 6) : (H > 32 ? 6 : 4);
};

template <int NP, int H>
__global__ void __launch_bounds__(SchwarzLocalDims<NP, H>::THREADS, SchwarzLocalDims<NP, H>::MIN_BLOCKS)
    schwarz_local_kernel(SchwarzArgs a, const double* __restrict__ r, const float* __restrict__ r32,
                         float* __restrict__ U, const int* __restrict__ done) {
    constexpr int F = 4 * NP;  // a multiple of 4: W rows are read as float4
    constexpr int HP = H + 1;  // padded per-thread row of the hidden vector (no bank conflicts)
    constexpr int T = SchwarzLocalDims<NP, H>::THREADS;
    __shared__ __align__(16) float wsh[H * F];
    __shared__ float hsh[T * HP];
    if (done && *done) return;
    for (int i = threadIdx.x; i < H * F; i += blockDim.x) wsh[i] = __bfloat162float(a.W[i]);
    __syncthreads();
    const float4* w4 = reinterpret_cast<const float4*>(wsh);
    float* hrow = hsh + threadIdx.x * HP;
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < a.K; m += gridDim.x * blockDim.x) {
        {
            float x[F];
            if (r32) {  // FP32 copy of the residual: no FP64 conversions here
                const float* vm = r32 + (size_t)m * NP;
#pragma unroll
                for (int i = 0; i < NP; i++) x[i] = vm[i];
#pragma unroll
                for (int f = 0; f < 3; f++) {
                    const int c = a.conn[(size_t)m * 3 + f];
                    const float* vn = r32 + (size_t)(c >= 0 ? (c >> 3) : 0) * NP;
                    const int* pm = a.perm + (c & 3) * NP;
#pragma unroll
                    for (int i = 0; i < NP; i++) x[(f + 1) * NP + i] = c >= 0 ? vn[pm[i]] : 0.f;
                }
            } else {
                const double* vm = r + (size_t)m * NP;
#pragma unroll
                for (int i = 0; i < NP; i++) x[i] = (float)vm[i];
#pragma unroll
                for (int f = 0; f < 3; f++) {
                    const int c = a.conn[(size_t)m * 3 + f];
                    const double* vn = r + (size_t)(c >= 0 ? (c >> 3) : 0) * NP;
                    const int* pm = a.perm + (c & 3) * NP;
#pragma unroll
                    for (int i = 0; i < NP; i++) x[(f + 1) * NP + i] = c >= 0 ? (float)vn[pm[i]] : 0.f;
                }
            }
            // h = W x: four W entries per shared-memory load (broadcast)
#pragma unroll 2
            for (int j = 0; j < H; j++) {
                float acc = 0.f;
#pragma unroll
                for (int i4 = 0; i4 < F / 4; i4++) {
                    const float4 w = w4[j * (F / 4) + i4];
                    acc = fmaf(w.x, x[4 * i4], acc);
                    acc = fmaf(w.y, x[4 * i4 + 1], acc);
                    acc = fmaf(w.z, x[4 * i4 + 2], acc);
                    acc = fmaf(w.w, x[4 * i4 + 3], acc);
                }
                hrow[j] = acc;
            }
        }
        // u = W^T h, accumulated row by row of W in registers, in two halves of
        // the columns (fewer live registers: more resident warps)
        float4* um = reinterpret_cast<float4*>(U + (size_t)m * F);
        constexpr int Q = F / 4, Q0 = (Q + 1) / 2;
#pragma unroll
        for (int half = 0; half < 2; half++) {
            constexpr int QH = Q0;
            float u[4 * QH];
#pragma unroll
            for (int i = 0; i < 4 * QH; i++) u[i] = 0.f;
            const int q0 = half * Q0;
#pragma unroll 2
            for (int j = 0; j < H; j++) {
                const float hj = hrow[j];
#pragma unroll
                for (int i4 = 0; i4 < QH; i4++) {
                    if (q0 + i4 < Q) {
                        const float4 w = w4[j * Q + q0 + i4];
                        u[4 * i4] = fmaf(w.x, hj, u[4 * i4]);
                        u[4 * i4 + 1] = fmaf(w.y, hj, u[4 * i4 + 1]);
                        u[4 * i4 + 2] = fmaf(w.z, hj, u[4 * i4 + 2]);
                        u[4 * i4 + 3] = fmaf(w.w, hj, u[4 * i4 + 3]);
                    }
                }
            }
#pragma unroll
            for (int i4 = 0; i4 < QH; i4++)
                if (q0 + i4 < Q) um[q0 + i4] = make_float4(u[4 * i4], u[4 * i4 + 1], u[4 * i4 + 2], u[4 * i4 + 3]);
        }
    }
}

// z_k = zb_k + (G^T U)_k, one thread per element row; the FP32 offset mirror
// of z is that of zb (written by the PCG update) plus c - c0 in FP32 (no FP64
// operation: forming it from z itself costs two FP64-pipe slots per row);
// partial sums of r.z for the CG scalars (the linear form is SPD: the
// standard beta applies; the two-layer form (FLEX) also sums r.z_old, read
// from z before it is overwritten, for the flexible beta).  Up to Np = 32
// each warp holds whole elements (32 / Np of them) and an element's c0
// reaches its rows by a shuffle; beyond that, element groups of 256 / Np
// rows exchange it through shared memory.
template <bool FLEX>
__global__ void schwarz_collect_kernel(SchwarzArgs a, const double* __restrict__ zb, const float* __restrict__ U,
                                       const double* __restrict__ r, double* __restrict__ z, float* __restrict__ dz,
                                       int mode, PcgScalars* S, double* part) {
    __shared__ float c0s[256];
    if (mode == LPC_PCG_ITERATION && S->done) return;
    const int Np = a.Np, F = 4 * Np;
    const bool wa = Np <= 32;
    const int lane = threadIdx.x & 31;
    const int EW = wa ? 32 / Np : 0;
    const int EB = wa ? 8 * EW : 256 / Np;
    int e, q;
    if (wa) {
        e = (threadIdx.x >> 5) * EW + lane / Np;
        q = lane % Np;
        if (lane >= EW * Np) e = EB;  // idle lane
    } else {
        e = threadIdx.x / Np;
        q = threadIdx.x - e * Np;
    }
    const int lb = lane - q;  // lane of the element's row 0 (warp-aligned layout)
    const int ngroups = (a.K + EB - 1) / EB;
    const bool flex = FLEX && mode == LPC_PCG_ITERATION;
    double rz = 0, rzo = 0;
    for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const int k = grp * EB + e;
        const bool act = e < EB && k < a.K;
        float c = 0.f;
        if (act) {
            const size_t t = (size_t)k * Np + q;
            c = U[(size_t)k * F + q];
#pragma unroll
            for (int f = 0; f < 3; f++) {
                const int cn = a.conn[(size_t)k * 3 + f];
                if (cn >= 0) c += U[(size_t)(cn >> 3) * F + ((cn & 3) + 1) * Np + a.iperm[f * Np + q]];
            }
            const double zv = zb[t] + (double)c;
            if (flex) rzo += r[t] * z[t];
            z[t] = zv;
            if (r) rz += r[t] * zv;
        }
        if (dz) {
            // dz enters as the offset mirror of zb: z - z0 = (zb - zb0) + (c - c0)
            float c0;
            if (wa) {
                c0 = __shfl_sync(0xffffffffu, c, lb);
            } else {
                if (act && q == 0) c0s[e] = c;
                __syncthreads();
                c0 = act ? c0s[e] : 0.f;
                __syncthreads();
            }
            if (act) {
                const size_t t = (size_t)k * Np + q;
                dz[t] = dz[t] + (c - c0);
            }
        }
    }
    if (mode == LPC_APPLY) return;
    if (FLEX) {
        double val[2] = {rz, rzo}, tot[2];
        if (grid_sum<2>(val, part, gridDim.x, &S->counter, tot) && threadIdx.x == 0) {
            if (mode == LPC_PCG_ITERATION) pcg_finish(S, tot[0], tot[1], S->rr);
            else S->rz = tot[0];
        }
    } else {
        double val[1] = {rz}, tot[1];
        if (grid_sum<1>(val, part, gridDim.x, &S->counter, tot) && threadIdx.x == 0) {
            if (mode == LPC_PCG_ITERATION) pcg_finish(S, tot[0], 0.0, S->rr);
            else S->rz = tot[0];
        }
    }
}

// X[m] = G_m v as FP32 rows (training)
__global__ void schwarz_gather_rows_kernel(SchwarzArgs a, const double* __restrict__ v, float* __restrict__ X) {
    const int F = 4 * a.Np;
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < a.K; m += gridDim.x * blockDim.x) {
        float x[kMaxF];
        schwarz_gather(a, v, m, x);
        for (int i = 0; i < F; i++) X[(size_t)m * F + i] = x[i];
    }
}

// C = X^T A + A^T X (F x F), one thread per entry, fixed summation order
__global__ void schwarz_cross_kernel(const float* __restrict__ X, const float* __restrict__ A, int K, int F,
                                     float* __restrict__ C) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= F * F) return;
    const int i = t / F, j = t - i * F;
    float acc = 0.f;
    for (int m = 0; m < K; m++) {
        const float* xm = X + (size_t)m * F;
        const float* am = A + (size_t)m * F;
        acc = fmaf(xm[i], am[j], fmaf(am[i], xm[j], acc));
    }
    C[t] = acc;
}

// gW = scale W C (H x F)
__global__ void schwarz_wgrad_kernel(const float* __restrict__ W, const float* __restrict__ C, int H, int F,
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
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= H * F) return;
    const int h = t / F, j = t - h * F;
    float acc = 0.f;
    for (int i = 0; i < F; i++) acc = fmaf(W[h * F + i], C[i * F + j], acc);
    gW[t] = s_scale * acc;
}

// g = (a/b) w - r as FP64 (the energy-loss output gradient direction)
__global__ void schwarz_outgrad_kernel(const double* __restrict__ r, const double* __restrict__ w,
                                       const double* __restrict__ part_a, const double* __restrict__ part_b, int G,
                                       size_t n, double* __restrict__ g) {
    __shared__ double s_ab;
    if (threadIdx.x < 32) {
        double aa = 0, bb = 0;
        for (int i = threadIdx.x; i < G; i += 32) { aa += part_a[i]; bb += part_b[i]; }
        for (int o = 16; o > 0; o >>= 1) {
            aa += __shfl_xor_sync(0xffffffffu, aa, o);
            bb += __shfl_xor_sync(0xffffffffu, bb, o);
        }
        if (threadIdx.x == 0) s_ab = bb > 0 ? aa / bb : 0.0;
    }
    __syncthreads();
    const double ab = s_ab;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        g[t] = ab * w[t] - r[t];
}

template <int NP, int H>
static cudaError_t schwarz_local_nh(const SchwarzArgs& a, const double* r, const float* r32, float* U,
                                    const int* done, cudaStream_t st) {
    constexpr int T = SchwarzLocalDims<NP, H>::THREADS;
    const int blocks = (a.K + T - 1) / T;
    const int cap = (T == 128 ? 8 : 16) * a.sms;
    schwarz_local_kernel<NP, H><<<blocks < cap ? blocks : cap, T, 0, st>>>(a, r, r32, U, done);
    return cudaGetLastError();
}

template <int NP>
static cudaError_t schwarz_local_np(const SchwarzArgs& a, const double* r, const float* r32, float* U,
                                    const int* done, cudaStream_t st) {
    switch (a.H) {
        case 32: return schwarz_local_nh<NP, 32>(a, r, r32, U, done, st);
        case 64: return schwarz_local_nh<NP, 64>(a, r, r32, U, done, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_schwarz_local(const SchwarzArgs& a, const double* r, const float* r32, float* U, const int* done,
                                 cudaStream_t st) {
    if (a.mlp) return launch_schwarz_mlp_local(a, r, r32, U, done, a.tc_status, st);
    if (a.tc_status && a.H == 32) return launch_schwarz_local_tc(a, r, r32, U, done, a.tc_status, st);
    switch (a.Np) {
        case 3: return schwarz_local_np<3>(a, r, r32, U, done, st);
        case 6: return schwarz_local_np<6>(a, r, r32, U, done, st);
        case 10: return schwarz_local_np<10>(a, r, r32, U, done, st);
        case 15: return schwarz_local_np<15>(a, r, r32, U, done, st);
        case 21: return schwarz_local_np<21>(a, r, r32, U, done, st);
        case 28: return schwarz_local_np<28>(a, r, r32, U, done, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_schwarz_collect(const SchwarzArgs& a, const double* zb, const float* U, const double* r,
                                   double* z, float* dz, int mode, PcgScalars* S, double* part, cudaStream_t st) {
    const bool wa = a.Np <= 32;
    const int EB = wa ? 8 * (32 / a.Np) : 256 / a.Np;
    const int threads = wa ? 256 : (EB * a.Np + 31) / 32 * 32;
    const int ngroups = (a.K + EB - 1) / EB;
    const int grid = ngroups < 8 * a.sms ? ngroups : 8 * a.sms;
    if (a.flex)
        schwarz_collect_kernel<true><<<grid, threads, 0, st>>>(a, zb, U, r, z, dz, mode, S, part);
    else
        schwarz_collect_kernel<false><<<grid, threads, 0, st>>>(a, zb, U, r, z, dz, mode, S, part);
    return cudaGetLastError();
}

cudaError_t launch_schwarz_gather_rows(const SchwarzArgs& a, const double* v, float* X, cudaStream_t st) {
    schwarz_gather_rows_kernel<<<(a.K + 127) / 128, 128, 0, st>>>(a, v, X);
    return cudaGetLastError();
}

cudaError_t launch_schwarz_cross(const float* X, const float* A, int K, int F, float* C, cudaStream_t st) {
    schwarz_cross_kernel<<<(F * F + 127) / 128, 128, 0, st>>>(X, A, K, F, C);
    return cudaGetLastError();
}

cudaError_t launch_schwarz_wgrad(const float* W, const float* C, int H, int F, const double* part_a,
                                 const double* part_b, int G, float* gW, cudaStream_t st) {
    schwarz_wgrad_kernel<<<(H * F + 127) / 128, 128, 0, st>>>(W, C, H, F, part_a, part_b, G, gW);
    return cudaGetLastError();
}

cudaError_t launch_schwarz_outgrad(const double* r, const double* w, const double* part_a, const double* part_b,
                                   int G, size_t n, double* g, cudaStream_t st) {
    schwarz_outgrad_kernel<<<608, 256, 0, st>>>(r, w, part_a, part_b, G, n, g);
    return cudaGetLastError();
}

}  // namespace dgk
