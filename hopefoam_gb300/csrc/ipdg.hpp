// ipdg.hpp -- SIPG operator / PCG shared declarations.
#pragma once

#include <cuda_runtime.h>

namespace dgk {

// reference operators in the arithmetic type of the apply (ring order)
template <typename T>
struct IpdgOps {
    const T* Srr;   // Np x Np reference stiffness parts (symmetric)
    const T* Srs2;
    const T* Sss;
    const T* Drf;   // [3 Nfq][Np]: d/dr of the nodal basis at face f's Gauss points
    const T* Dsf;
    const T* DrfT;  // [Np][3 Nfq] (transposed copies for the per-Gauss-point threads)
    const T* DsfT;
    const T* If;    // Nfq x Nfp
    const T* fw;    // Nfq face Gauss weights
    const T* fc;    // K x 3 x 6 per element face:
                    //   [n.grad r, n.grad s, n.grad r of the neighbour, n.grad s of the neighbour, tau/2, sJ]
    const T* vc;    // K x 3 volume coefficients J (rx^2+ry^2), J (rx sx+ry sy), J (sx^2+sy^2)
    const T* Mr;    // Np x Np reference mass matrix (J = 1, symmetric)
    const T* mrow;  // Np row sums of Mr (the mass term acts on offsets plus a constant)
};

struct IpdgArgs {
    int K, N, Np, Nfp, Nfq;
    int sms;             // SMs of the device (persistent grids)
    double tau_coef;
    const double* geo;   // K x 4 metrics
    const double* J;     // K Jacobians
    const int* conn;     // K x 3 packed neighbours
    double mass_coef;    // S + mass_coef M (Helmholtz form); 0: the Laplacian alone
    IpdgOps<double> o64;
    IpdgOps<float> o32;
    // two-pass FP32 apply of the PCG iterations (N <= 5; null: not built):
    // the host copy of the reference tables passed to its kernels by value
    // (IpLaneTab<N>); per element and face, the input's trace and outward
    // normal derivative at the face's Gauss points (lane_face_rec(N) floats,
    // element's own point order); per element the input's value at its first
    // node as an FP32 pair (hi = the value rounded, lo = the rest rounded)
    const void* lane_tab;
    float* lane_ftr;
    float2* lane_p0;
};

constexpr int kFaceCoef = 6;

// floats per face record of the two-pass apply: Nfq traces, Nfq normal
// derivatives, padded to 16 bytes
constexpr int lane_face_rec(int N) { return (2 * (N + 2) + 3) / 4 * 4; }

// reference tables of the element-per-lane apply, FP32, ring order; passed
// as a kernel parameter so that every table read is a constant-bank operand
template <int N>
struct IpLaneTab {
    static constexpr int Np = (N + 1) * (N + 2) / 2, Nfp = N + 1, Nfq = N + 2, NF = 3 * Nfq;
    float DrfT[Np][NF];  // d/dr of basis function p at face Gauss point fg
    float DsfT[Np][NF];
    float If[Nfq][Nfp];
    float fw[Nfq];
    float Srr[Np][Np], Srs2[Np][Np], Sss[Np][Np];
    float Mr[Np][Np];
    float mrow[Np];
};

// device-side CG state; the kernels read and update it, the host reads it
// every few iterations
struct PcgScalars {
    double bb;      // ||b||^2
    double tol2;    // stop when r.r <= tol2
    double rz;      // r.z of the current residual
    double pap;     // p.Ap of the current search direction
    double alpha;   // rz / pap
    double beta;    // next p = z + beta p (0: restart from z)
    double rr;      // recurrence residual r.r
    int done;       // 1 converged, 2 breakdown / non-finite
    int it;         // iterations taken
    unsigned int counter;  // arrival counter of the grid-wide sums
};

struct MgLevels;

struct PcgVecs {
    double *x, *r, *z, *Ap;      // ring-order FP64 vectors of length K*Np
    double* p[2];                // search directions, ping-pong (iteration j reads p[j&1], writes p[(j+1)&1])
    double* part;                // [3][nmax] per-CTA partial sums
    int nmax;                    // largest grid of any PCG kernel
    const float* P32;            // block-Jacobi inverse blocks (FP32), grouped layout
    const double* P64;           // FP64 blocks (grouped); used instead of P32 when set
    double* zb;                  // learned mode: block-Jacobi output (z holds the learned one)
    PcgScalars* S;
    // FP32 offset mirrors (value minus the element's first-node value) of z
    // and of the search directions (ping-pong like p); null: the apply stages
    // from the FP64 vectors
    float* dz;
    float* dp[2];
    float* r32;                  // learned Schwarz mode: FP32 copy of r for the learned kernel (else null)
    const MgLevels* mg;          // multilevel mode (with zb): the coarse-space correction forms z
    double* zl;                  // learned + multilevel: the learned output, before the coarse correction
};

// largest grid of the PCG kernels (sizes the partials)
int pcg_max_grid(int K, int N, int sms);
// grouped inverse-block layout of the element-aligned kernels: element count
// of the padded storage, and the conversion from row-major blocks
size_t grouped_blocks_size(int K, int Np);
cudaError_t launch_group_blocks(const IpdgArgs& a, const double* blocks, double* P64, float* P32, cudaStream_t s);

// y = S u (standalone)
cudaError_t launch_ipdg_apply(const IpdgArgs& a, bool fp32, const double* u, double* y, cudaStream_t s);
cudaError_t launch_ipdg_diag(const IpdgArgs& a, double* blocks, cudaStream_t s);
cudaError_t launch_invert_blocks(double* blocks, float* blocks32, int K, int Np, int* status, cudaStream_t s);
struct LpcNet;
struct LpcFeatArgs;
// lpc / fa may be null (block-Jacobi only).  init: z = M r, S->rz, S->rr, beta = 0
cudaError_t launch_pcg_init(const IpdgArgs& a, const PcgVecs& v, const LpcNet* lpc, const LpcFeatArgs* fa,
                            cudaStream_t s);
// one iteration: p_new = z + beta p_old fused into Ap = S p_new (alpha on the
// device), then x, r, z updates with beta and the stop test on the device
cudaError_t launch_pcg_iteration(const IpdgArgs& a, const PcgVecs& v, bool fp32, int parity, const LpcNet* lpc,
                                 const LpcFeatArgs* fa, cudaStream_t s);
// residual replacement: z = M r, S->rz (and S->rr) from the current r; beta kept
cudaError_t launch_pcg_refresh(const IpdgArgs& a, const PcgVecs& v, const LpcNet* lpc, const LpcFeatArgs* fa,
                               cudaStream_t s);
cudaError_t launch_bj(const IpdgArgs& a, const float* P32, const double* r, double* z, cudaStream_t s);
cudaError_t launch_dot(const double* x, const double* y, size_t n, double* part, int G, cudaStream_t s);
cudaError_t launch_reduce_to(const double* part, int G, double* out, cudaStream_t s);
cudaError_t launch_axpy(double* y, const double* x, double alpha, size_t n, cudaStream_t s);      // y += alpha x
cudaError_t launch_xmy(double* out, const double* b, const double* y, size_t n, cudaStream_t s);  // out = b - y
cudaError_t launch_permute(const double* in, double* out, const int* perm, int K, int Np, bool to_ring,
                           cudaStream_t s);

}  // namespace dgk
