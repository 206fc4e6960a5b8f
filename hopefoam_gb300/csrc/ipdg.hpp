// ipdg.hpp -- SIPG operator / PCG shared declarations.
#pragma once

#include <cuda_runtime.h>

namespace dgk {

struct IpdgArgs {
    int K, N, Np, Nfp, Nfq;
    double tau_coef;
    const double* geo;   // K x 4 metrics
    const double* J;     // K Jacobians
    const int* conn;     // K x 3 packed neighbours
    const double* Srr;   // Np x Np reference stiffness parts (ring order)
    const double* Srs2;
    const double* Sss;
    const double* Drf;   // 3 x Nfq x Np: d/dr of the nodal basis at face f's Gauss points
    const double* Dsf;
    const double* If;    // Nfq x Nfp
    const double* fw;    // Nfq face Gauss weights
};

struct PcgScalars {
    double bb;      // ||b||^2 of the current (inner) system
    double tol2;    // stop when r.r <= tol2
    int done;       // 1 converged, 2 breakdown / non-finite
    int it;         // iterations taken
};

struct PcgVecs {
    double *x, *r, *z, *p, *Ap;  // ring-order FP64 vectors of length K*Np
    double *part_pap;            // [G]
    double *part_rz;             // [2][G]
    double *part_rr;             // [G]
    double *part_rzo;            // [G] r_new . z_old (flexible beta)
    const float* P32;            // block-Jacobi inverse blocks (FP32), K x Np x Np
    const double* P64;           // FP64 blocks; used instead of P32 when set
    PcgScalars* S;
    int G;                       // grid of the reduction kernels
};

cudaError_t launch_ipdg_apply(const IpdgArgs& a, bool fp32, const double* u, double* y, double* part, int G,
                              cudaStream_t s);
cudaError_t launch_ipdg_diag(const IpdgArgs& a, double* blocks, cudaStream_t s);
cudaError_t launch_invert_blocks(double* blocks, float* blocks32, int K, int Np, int* status, cudaStream_t s);
cudaError_t launch_pcg_init(const IpdgArgs& a, const PcgVecs& v, cudaStream_t s);
cudaError_t launch_pcg_iteration(const IpdgArgs& a, const PcgVecs& v, bool fp32, int parity, cudaStream_t s);
cudaError_t launch_dot(const double* x, const double* y, size_t n, double* part, int G, cudaStream_t s);
cudaError_t launch_reduce_to(const double* part, int G, double* out, cudaStream_t s);
cudaError_t launch_axpy(double* y, const double* x, double alpha, size_t n, cudaStream_t s);      // y += alpha x
cudaError_t launch_xmy(double* out, const double* b, const double* y, size_t n, cudaStream_t s);  // out = b - y
cudaError_t launch_permute(const double* in, double* out, const int* perm, int K, int Np, bool to_ring,
                           cudaStream_t s);

}  // namespace dgk
