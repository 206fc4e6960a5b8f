// euler_fp64.cu -- plain FP64 fused DG Euler stage (sm_103a).
//
// One CTA advances E elements through one Runge-Kutta stage:
//   1. stage the elements' nodal state (E x 4 x Np doubles, contiguous) in shared memory;
//   2. in parallel (a) evaluate the state at the Ng cubature points and the
//      metric-scaled volume fluxes Fr = rx Fx + ry Fy, Fs = sx Fx + sy Fy
//      (dgGaussField::initField cell part, dgEulerFoam.C:81-82, the volume
//      loops of defaultConvectionScheme.C:79-90, defaultGrad.C:120-125,
//      defaultDivScheme.C:118-123) and (b) per element face, gather the own and
//      the neighbour face traces, interpolate to the Nfq face Gauss points
//      (dgGaussField.C:204-238) and evaluate the numerical flux (Roe:
//      RoeFlux.C:109-178; or Euler Lax-Friedrichs);
//   3. contract: R = Sr Fr + Ss Fs - sum_f (sJ/J)_f Lift_f F*_f  (the weak
//      form with the affine mass inverse folded in), then apply the stage
//      update in FP64 and write the element back.
// Each element evaluates the flux of its own three faces with its own outward
// normal; F*(q-,q+,n) = -F*(q+,q-,-n) makes this the reference's
// owner/neighbour lift (defaultConvectionScheme.C:93-128) up to round-off.
// On GB300 the FP64 pipe (~2 DFMA/clk/SM) bounds this kernel; it is the
// parity path, the split-precision kernel is the fast one.
#include "dg_internal.hpp"
#include "euler_flux.cuh"

namespace dgk {

template <int N>
struct Fp64Tile {
    static constexpr int E = (N == 1) ? 32 : (N <= 3) ? 16 : (N <= 5) ? 8 : 4;
    static constexpr int THREADS = 256;
    static constexpr int Np = Dims<N>::Np, Ng = Dims<N>::Ng, Nfp = Dims<N>::Nfp, Nfq = Dims<N>::Nfq;
    static constexpr size_t SMEM = sizeof(double) * (size_t)E * (4 * Np + 8 * Ng + 12 * Nfq);
};

template <int N>
__global__ void __launch_bounds__(256) euler_stage_fp64_kernel(EulerArgs a) {
    using T = Fp64Tile<N>;
    constexpr int E = T::E, Np = T::Np, Ng = T::Ng, Nfp = T::Nfp, Nfq = T::Nfq;
    constexpr int NB = 3 * N;  // boundary nodes in the ring
    extern __shared__ double sm[];
    double* qs = sm;                        // [E][4][Np]
    double* Fr = qs + E * 4 * Np;           // [E][4][Ng]
    double* Fs = Fr + E * 4 * Ng;           // [E][4][Ng]
    double* Ff = Fs + E * 4 * Ng;           // [E][4][3*Nfq]

    const int k0 = blockIdx.x * E;
    const int ne = min(E, a.K - k0);
    const double gamma = a.gamma;

    // 1. stage the tile
    const double* qin = a.qin + (size_t)k0 * 4 * Np;
    for (int i = threadIdx.x; i < ne * 4 * Np; i += blockDim.x) qs[i] = qin[i];
    __syncthreads();

    // 2a/2b. volume fluxes at cubature points and face fluxes
    const int nvol = ne * Ng;
    const int nitems = nvol + ne * 3;
    for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
        if (it < nvol) {
            const int e = it / Ng, g = it - e * Ng;
            const double* qe = qs + e * 4 * Np;
            const double* vg = a.ops.Vg + g * Np;
            double q[4] = {0, 0, 0, 0};
#pragma unroll 4
            for (int p = 0; p < Np; p++) {
                const double w = __ldg(vg + p);
                q[0] += w * qe[p];
                q[1] += w * qe[Np + p];
                q[2] += w * qe[2 * Np + p];
                q[3] += w * qe[3 * Np + p];
            }
            const double* gk = a.geo + (size_t)(k0 + e) * 4;
            const double rx = gk[0], sx = gk[1], ry = gk[2], sy = gk[3];
            double fx[4], fy[4];
            euler_phys_flux(gamma, q, fx, fy);
#pragma unroll
            for (int v = 0; v < 4; v++) {
                Fr[(e * 4 + v) * Ng + g] = rx * fx[v] + ry * fy[v];
                Fs[(e * 4 + v) * Ng + g] = sx * fx[v] + sy * fy[v];
            }
        } else {
            const int j2 = it - nvol;
            const int e = j2 / 3, f = j2 - e * 3;
            const int k = k0 + e;
            const double* gk = a.geo + (size_t)k * 4;
            double nx, ny, fsc;
            face_normal(f, gk[0], gk[1], gk[2], gk[3], nx, ny, fsc);
            double um[4][Nfp], up[4][Nfp];
            const double* qe = qs + e * 4 * Np;
#pragma unroll
            for (int j = 0; j < Nfp; j++) {
                const int pos = (f * N + j) % NB;
#pragma unroll
                for (int v = 0; v < 4; v++) um[v][j] = qe[v * Np + pos];
            }
            const int c = __ldg(a.conn + (size_t)k * 3 + f);
            if (c >= 0) {
                const int nb = c >> 3, fn = c & 3, rot = (c >> 2) & 1;
                const double* qn = a.qin + (size_t)nb * 4 * Np;
#pragma unroll
                for (int j = 0; j < Nfp; j++) {
                    const int jj = rot ? (N - j) : j;
                    const int pos = (fn * N + jj) % NB;
#pragma unroll
                    for (int v = 0; v < 4; v++) up[v][j] = __ldg(qn + v * Np + pos);
                }
            } else {
                const double* bt = a.btrace + (size_t)(-1 - c) * 4 * Nfp;
#pragma unroll
                for (int j = 0; j < Nfp; j++)
#pragma unroll
                    for (int v = 0; v < 4; v++) up[v][j] = __ldg(bt + v * Nfp + j);
            }
            double qm[Nfq][4], qp[Nfq][4];
#pragma unroll
            for (int i = 0; i < Nfq; i++) {
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    double sm_ = 0, sp_ = 0;
#pragma unroll
                    for (int j = 0; j < Nfp; j++) {
                        const double w = __ldg(a.ops.If + i * Nfp + j);
                        sm_ += w * um[v][j];
                        sp_ += w * up[v][j];
                    }
                    qm[i][v] = sm_;
                    qp[i][v] = sp_;
                }
            }
            double* ff = Ff + e * 4 * 3 * Nfq + f * Nfq;
            if (a.flux == 1) {
#pragma unroll
                for (int i = 0; i < Nfq; i++) {
                    double F[4];
                    roe_flux(gamma, nx, ny, qm[i], qp[i], F);
#pragma unroll
                    for (int v = 0; v < 4; v++) ff[v * 3 * Nfq + i] = fsc * F[v];
                }
            } else {
                double lam = 0;
#pragma unroll
                for (int i = 0; i < Nfq; i++) {
                    lam = fmax(lam, wave_speed(gamma, nx, ny, qm[i]));
                    lam = fmax(lam, wave_speed(gamma, nx, ny, qp[i]));
                }
#pragma unroll
                for (int i = 0; i < Nfq; i++) {
                    double F[4];
                    lf_flux(gamma, nx, ny, lam, qm[i], qp[i], F);
#pragma unroll
                    for (int v = 0; v < 4; v++) ff[v * 3 * Nfq + i] = fsc * F[v];
                }
            }
        }
    }
    __syncthreads();

    // 3. contraction + stage update
    for (int it = threadIdx.x; it < ne * 4 * Np; it += blockDim.x) {
        const int e = it / (4 * Np);
        const int rem = it - e * 4 * Np;
        const int v = rem / Np, p = rem - v * Np;
        const double* fr = Fr + (e * 4 + v) * Ng;
        const double* fs = Fs + (e * 4 + v) * Ng;
        const double* sr = a.ops.Sr + p * Ng;
        const double* ss = a.ops.Ss + p * Ng;
        double acc = 0, acc2 = 0;
#pragma unroll 4
        for (int g = 0; g < Ng; g++) {
            acc += __ldg(sr + g) * fr[g];
            acc2 += __ldg(ss + g) * fs[g];
        }
        acc += acc2;
        const double* ff = Ff + (e * 4 + v) * 3 * Nfq;
        const double* lf = a.ops.Lift + p * 3 * Nfq;
        double accf = 0;
#pragma unroll
        for (int c = 0; c < 3 * Nfq; c++) accf += __ldg(lf + c) * ff[c];
        const double R = acc - accf;
        const size_t idx = (size_t)k0 * 4 * Np + it;
        const double q0 = qs[it];
        const double dt = a.dtk ? a.dt * a.dtk[k0 + e] : a.dt;
        switch (a.mode) {
            case MODE_RHS: a.rhs[idx] = R; break;
            case MODE_LSERK: {
                const double r = a.rka * a.res[idx] + dt * R;
                a.res[idx] = r;
                a.qout[idx] = q0 + a.rkb * r;
            } break;
            case MODE_EULER: a.qout[idx] = q0 + dt * R; break;
            default: a.qout[idx] = 0.5 * a.qold[idx] + 0.5 * (q0 + dt * R); break;
        }
    }
}

template <int N>
static cudaError_t launch_n(const EulerArgs& a, cudaStream_t s) {
    using T = Fp64Tile<N>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(euler_stage_fp64_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int grid = (a.K + T::E - 1) / T::E;
    euler_stage_fp64_kernel<N><<<grid, T::THREADS, T::SMEM, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_euler_fp64(int N, const EulerArgs& a, cudaStream_t s) {
    switch (N) {
        case 1: return launch_n<1>(a, s);
        case 2: return launch_n<2>(a, s);
        case 3: return launch_n<3>(a, s);
        case 4: return launch_n<4>(a, s);
        case 5: return launch_n<5>(a, s);
        case 6: return launch_n<6>(a, s);
        case 7: return launch_n<7>(a, s);
        default: return cudaErrorInvalidValue;
    }
}

// layout conversion: reference q[v][k][i] <-> device q[k][v][p], p ring order
__global__ void to_internal_kernel(const double* __restrict__ ref, double* __restrict__ q, const int* __restrict__ ring,
                                   int K, int Np) {
    const size_t n = (size_t)K * 4 * Np;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / (4 * Np));
        const int rem = (int)(t - (size_t)k * 4 * Np);
        const int v = rem / Np, p = rem - v * Np;
        q[t] = ref[(size_t)v * K * Np + (size_t)k * Np + ring[p]];
    }
}

__global__ void to_reference_kernel(const double* __restrict__ q, double* __restrict__ ref, const int* __restrict__ ring,
                                    int K, int Np) {
    const size_t n = (size_t)K * 4 * Np;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / (4 * Np));
        const int rem = (int)(t - (size_t)k * 4 * Np);
        const int v = rem / Np, p = rem - v * Np;
        ref[(size_t)v * K * Np + (size_t)k * Np + ring[p]] = q[t];
    }
}

static int grid_for(size_t n) {
    size_t g = (n + 255) / 256;
    return (int)(g > 152 * 32 ? 152 * 32 : (g == 0 ? 1 : g));
}

cudaError_t launch_to_internal(const double* ref, double* q, const int* ring, int K, int Np, cudaStream_t s) {
    to_internal_kernel<<<grid_for((size_t)K * 4 * Np), 256, 0, s>>>(ref, q, ring, K, Np);
    return cudaGetLastError();
}

cudaError_t launch_to_reference(const double* q, double* ref, const int* ring, int K, int Np, cudaStream_t s) {
    to_reference_kernel<<<grid_for((size_t)K * 4 * Np), 256, 0, s>>>(q, ref, ring, K, Np);
    return cudaGetLastError();
}

}  // namespace dgk
