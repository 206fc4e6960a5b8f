// dg_internal.hpp -- shared declarations between the C-ABI layer and the kernels.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "dg_basis.hpp"

namespace dgk {

// compile-time sizes per order (cubature sizes from the strength-3(N+1) table)
template <int N>
struct Dims {
    static constexpr int Np = (N + 1) * (N + 2) / 2;
    static constexpr int Nfp = N + 1;
    static constexpr int Nfq = N + 2;
    static constexpr int Ng = (N == 1) ? 12 : (N == 2) ? 19 : (N == 3) ? 36 : (N == 4) ? 54 : (N == 5) ? 73 : (N == 6) ? 93 : 118;
};

enum StageMode {
    MODE_RHS = 0,     // rhs = R(qin)
    MODE_LSERK = 1,   // res = a res + dt R(qin); qout = qin + b res
    MODE_EULER = 2,   // qout = qin + dt R(qin)
    MODE_SSP2 = 3     // qout = 1/2 qold + 1/2 (qin + dt R(qin))
};

struct EulerOps {
    const double* Vg;    // Ng x Np
    const double* Sr;    // Np x Ng
    const double* Ss;    // Np x Ng
    const double* Lift;  // Np x 3Nfq
    const double* If;    // Nfq x Nfp
};

// Device state layout: q[k][v][p], v = rho, rhou, rhov, E, p in ring order.
// conn[k*3+f]: >= 0 -> (nbr << 3) | (rot << 2) | nbr_face;  < 0 -> -1 - boundary slot.
struct EulerArgs {
    const double* qin;
    double* qout;
    double* res;
    const double* qold;
    double* rhs;
    const double* geo;     // K x 4: rx, sx, ry, sy
    const int* conn;       // K x 3
    const double* btrace;  // nb x 4 x Nfp (face direction)
    EulerOps ops;
    int K;
    int flux;
    int mode;
    double gamma, dt, rka, rkb;
    const double* dtk;     // per-element time-step factors (null: 1); the step of element k is dt * dtk[k]
    const float* dtk32;    // FP32 copy of dtk (the split-precision path)
};

// launchers (return cudaError_t of the launch)
cudaError_t launch_euler_fp64(int N, const EulerArgs& a, cudaStream_t s);
cudaError_t launch_to_internal(const double* ref, double* q, const int* ring, int K, int Np, cudaStream_t s);
cudaError_t launch_to_reference(const double* q, double* ref, const int* ring, int K, int Np, cudaStream_t s);

}  // namespace dgk
