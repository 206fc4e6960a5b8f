// ins.cu -- the incompressible Navier-Stokes (Chorin / velocity-correction)
// step of tutorials/DG/2D/pearsonVortex/dgChorinFoam/dgChorinFoam.C:63-109 on
// the GPU (FP64).
//
// One step (all on one stream, vectors ring order, component-major U[c][k][p]):
//   1. N = div(U (x) U): the reference's dgc::div(U, U) on dof fields with the
//      LF flux (defaultConvectionScheme.C:216-300, LFFlux.C:103-211): products
//      at the nodes interpolated to the cubature points, weak divergence,
//      node-based LF face flux interpolated to the face Gauss points, lifted,
//      solved against the mass matrix (dgm::Sp(convecU) == dgc::div(U, U)).
//   2. UT = (a0 U + a1 U_old - dt (b0 N + b1 N_old)) / g0.
//   3. Pressure Neumann data on the faces where U has a fixed value
//      (pEqnCorrect.H, pCorrectEquation.H:78-110): nbp = n.(N + nu curl curl U)
//      + extra (the caller's n.dU/dt), extrapolated b0 nbp + b1 nbp_old.
//   4. S_p p = -(q3 b_Lp + F^T W F nbp + (g0/dt) M div UT), S = -(reference
//      Laplacian) (SPD), block-Jacobi PCG (the reference: PETSc LU).
//   5. UT -= (dt/g0) grad p (strong nodal gradient, defaultGrad.C:44-78).
//   6. (g0/(dt nu) M + S_U) U = g0/(dt nu) M UT - q4 b_LU per component.
// b_L are the reference Laplacian's boundary-data terms
// (defaultLaplacianScheme.C:157-220): Dirichlet -tau F^T W F g + Dn^T W F g,
// Neumann -F^T W F h; q3, q4 are the caller's factors on them (the
// reference's bCorrectEquation paraT3 / paraT4).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/dgcu.h"
#include "dg_ctx.hpp"
#include "euler_flux.cuh"
#include "ipdg.hpp"

// ---------------------------------------------------------------------------
// kernels

namespace dgk {

struct InsTables {
    const double* Dr;    // Np x Np nodal derivatives, ring order
    const double* Ds;
    const double* Vg;    // Ng x Np cubature interpolation, ring order
    const double* Sr;    // Np x Ng  M_ref^-1 Drg^T W
    const double* Ss;
    const double* Lift;  // Np x 3Nfq M_ref^-1 F_f^T diag(fw)
    const double* If;    // Nfq x Nfp
    const double* Mr;    // Np x Np reference mass
};

template <int N>
struct InsDims {
    static constexpr int Np = Dims<N>::Np, Ng = Dims<N>::Ng, Nfp = Dims<N>::Nfp, Nfq = Dims<N>::Nfq;
    static constexpr int THREADS = 128;
    static constexpr int BYTES = 8 * (2 * Np + 4 * Np + 4 * Ng + 6 * Nfq);
    static constexpr int E0 = 40960 / BYTES;
    static constexpr int E = E0 < 1 ? 1 : (E0 > 16 ? 16 : E0);
};

// N = div(U (x) U); ubnd[slot][c][j] boundary values of fixed-value faces,
// ukind[slot] == 1: the boundary value is the interior trace (fixedGradient)
template <int N>
__global__ void __launch_bounds__(128) ins_convection_kernel(int K, const double* __restrict__ geo,
                                                            const int* __restrict__ conn, InsTables t,
                                                            const double* __restrict__ u,
                                                            const double* __restrict__ ubnd,
                                                            const int* __restrict__ ukind, double* __restrict__ out) {
    using D = InsDims<N>;
    constexpr int Np = D::Np, Ng = D::Ng, Nfp = D::Nfp, Nfq = D::Nfq, E = D::E, NB = 3 * N;
    __shared__ double us[E][2][Np];
    __shared__ double pr[E][4][Np];     // products u_d u_c at the nodes, (d, c) = xx, xy, yx, yy
    __shared__ double fr[E][2][Ng];     // rx Fx + ry Fy at the cubature points, per component c
    __shared__ double fs[E][2][Ng];
    __shared__ double fl[E][2][3 * Nfq];  // (sJ/J) face flux at the face Gauss points
    const size_t KN = (size_t)K * Np;
    const int ntiles = (K + E - 1) / E;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int k0 = tile * E, ne = min(E, K - k0);
        for (int i = threadIdx.x; i < ne * 2 * Np; i += blockDim.x) {
            const int e = i / (2 * Np), r = i - e * 2 * Np, c = r / Np, p = r - c * Np;
            us[e][c][p] = u[c * KN + (size_t)(k0 + e) * Np + p];
        }
        __syncthreads();
        for (int i = threadIdx.x; i < ne * Np; i += blockDim.x) {
            const int e = i / Np, p = i - e * Np;
            const double ux = us[e][0][p], uy = us[e][1][p];
            pr[e][0][p] = ux * ux;
            pr[e][1][p] = ux * uy;
            pr[e][2][p] = uy * ux;
            pr[e][3][p] = uy * uy;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < ne * Ng; i += blockDim.x) {
            const int e = i / Ng, g = i - e * Ng;
            const double* gk = geo + 4 * (size_t)(k0 + e);
            const double rx = gk[0], sx = gk[1], ry = gk[2], sy = gk[3];
            double F[4] = {0, 0, 0, 0};
            for (int j = 0; j < Np; j++) {
                const double v = t.Vg[g * Np + j];
#pragma unroll
                for (int m = 0; m < 4; m++) F[m] += v * pr[e][m][j];
            }
            // component c: Fx = (u_x u_c), Fy = (u_y u_c)
#pragma unroll
            for (int c = 0; c < 2; c++) {
                const double Fx = F[c], Fy = F[2 + c];
                fr[e][c][g] = rx * Fx + ry * Fy;
                fs[e][c][g] = sx * Fx + sy * Fy;
            }
        }
        for (int i = threadIdx.x; i < ne * 3; i += blockDim.x) {
            const int e = i / 3, f = i - e * 3, k = k0 + e;
            const double* gk = geo + 4 * (size_t)k;
            double nx, ny, fsc;
            face_normal(f, gk[0], gk[1], gk[2], gk[3], nx, ny, fsc);
            double UO[2][Nfp], UN[2][Nfp];
            const int cn = conn[(size_t)k * 3 + f];
            for (int j = 0; j < Nfp; j++) {
                const int pos = (f * N + j) % NB;
                UO[0][j] = us[e][0][pos];
                UO[1][j] = us[e][1][pos];
                if (cn >= 0) {
                    const int nb = cn >> 3, fn = cn & 3, rot = (cn >> 2) & 1;
                    const int jj = rot ? (N - j) : j;
                    const size_t q = (size_t)nb * Np + (fn * N + jj) % NB;
                    UN[0][j] = u[q];
                    UN[1][j] = u[KN + q];
                } else {
                    const int slot = -1 - cn;
                    if (ukind[slot] == 1) {
                        UN[0][j] = UO[0][j];
                        UN[1][j] = UO[1][j];
                    } else {
                        UN[0][j] = ubnd[((size_t)slot * 2 + 0) * Nfp + j];
                        UN[1][j] = ubnd[((size_t)slot * 2 + 1) * Nfp + j];
                    }
                }
            }
            double vO[Nfp], vN[Nfp], lam = 0.0;
            for (int j = 0; j < Nfp; j++) {
                vO[j] = nx * UO[0][j] + ny * UO[1][j];
                vN[j] = nx * UN[0][j] + ny * UN[1][j];
                lam = fmax(lam, fmax(fabs(vO[j]), fabs(vN[j])));
            }
#pragma unroll
            for (int c = 0; c < 2; c++) {
                double tn[Nfp];
                for (int j = 0; j < Nfp; j++)
                    tn[j] = (vO[j] * UO[c][j] + vN[j] * UN[c][j]) * 0.5 + lam * (UO[c][j] - UN[c][j]) * 0.5;
                for (int g = 0; g < Nfq; g++) {
                    double s = 0;
                    for (int j = 0; j < Nfp; j++) s += t.If[g * Nfp + j] * tn[j];
                    fl[e][c][f * Nfq + g] = fsc * s;
                }
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < ne * 2 * Np; i += blockDim.x) {
            const int e = i / (2 * Np), r = i - e * 2 * Np, c = r / Np, p = r - c * Np;
            double v = 0;
            for (int g = 0; g < Ng; g++) v -= t.Sr[p * Ng + g] * fr[e][c][g] + t.Ss[p * Ng + g] * fs[e][c][g];
            for (int q = 0; q < 3 * Nfq; q++) v += t.Lift[p * 3 * Nfq + q] * fl[e][c][q];
            out[c * KN + (size_t)(k0 + e) * Np + p] = v;
        }
        __syncthreads();
    }
}

// nodal operators on affine elements: mode 0 div (2 -> 1), 1 grad (1 -> 2), 2 curl curl (2 -> 2)
template <int N>
__global__ void __launch_bounds__(128) ins_nodal_kernel(int mode, int K, const double* __restrict__ geo, InsTables t,
                                                       const double* __restrict__ in, double* __restrict__ out) {
    constexpr int Np = Dims<N>::Np, E = 128 / Np > 0 ? 128 / Np : 1;
    __shared__ double w[E][Np];
    const size_t KN = (size_t)K * Np;
    const int ntiles = (K + E - 1) / E;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int e = threadIdx.x / Np, i = threadIdx.x - e * Np, k = tile * E + e;
        const bool ok = e < E && k < K;
        double rx = 0, sx = 0, ry = 0, sy = 0;
        if (ok) {
            const double* gk = geo + 4 * (size_t)k;
            rx = gk[0]; sx = gk[1]; ry = gk[2]; sy = gk[3];
        }
        double dxu = 0, dyu = 0, dxv = 0, dyv = 0;
        if (ok) {
            const double* a = in + (size_t)k * Np;
            const double* b = in + KN + (size_t)k * Np;
            for (int j = 0; j < Np; j++) {
                const double dr = t.Dr[i * Np + j], ds = t.Ds[i * Np + j];
                const double dx = dr * rx + ds * sx, dy = dr * ry + ds * sy;
                dxu += dx * a[j];
                dyu += dy * a[j];
                if (mode != 1) {
                    dxv += dx * b[j];
                    dyv += dy * b[j];
                }
            }
        }
        if (mode == 0) {
            if (ok) out[(size_t)k * Np + i] = dxu + dyv;
        } else if (mode == 1) {
            if (ok) {
                out[(size_t)k * Np + i] = dxu;
                out[KN + (size_t)k * Np + i] = dyu;
            }
        } else {
            // w = dv/dx - du/dy, then curl w = (dw/dy, -dw/dx)
            if (ok) w[e][i] = dxv - dyu;
            __syncthreads();
            if (ok) {
                double cx = 0, cy = 0;
                for (int j = 0; j < Np; j++) {
                    const double dr = t.Dr[i * Np + j], ds = t.Ds[i * Np + j];
                    cx += (dr * ry + ds * sy) * w[e][j];
                    cy -= (dr * rx + ds * sx) * w[e][j];
                }
                out[(size_t)k * Np + i] = cx;
                out[KN + (size_t)k * Np + i] = cy;
            }
            __syncthreads();
        }
    }
}

// y = coef J_k M_ref x (per element)
template <int N>
__global__ void ins_mass_kernel(int K, const double* __restrict__ J, InsTables t, double coef,
                                const double* __restrict__ x, double* __restrict__ y) {
    constexpr int Np = Dims<N>::Np;
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)K * Np) return;
    const size_t k = idx / Np;
    const int i = (int)(idx - k * Np);
    double s = 0;
    for (int j = 0; j < Np; j++) s += t.Mr[i * Np + j] * x[k * Np + j];
    y[idx] = coef * J[k] * s;
}

// per boundary slot data of the boundary-term kernel
struct InsSlots {
    int nb;
    const int* k;       // element
    const int* f;       // its face
    const double* sJ;   // face Jacobian (edge length / 2)
    const double* tau;  // penalty of the face
    const double* dnr;  // n . grad r, n . grad s of the element
    const double* dns;
    const double* nx;   // outward unit normal
    const double* ny;
};

// target[k][.] += scale * (reference Laplacian boundary terms) on the slots with
// sel[slot] == want:  kind 0 Dirichlet (-tau F^T W F g + Dn^T W F g), kind 1
// face mass only (-F^T W F g); g = data[slot * dstride + doff + j]
template <int N>
__global__ void ins_bdata_kernel(InsSlots s, const dgk::IpdgOps<double> o, const int* __restrict__ sel, int want,
                                 int kind, const double* __restrict__ data, int dstride, int doff, double scale,
                                 double* __restrict__ target) {
    constexpr int Np = Dims<N>::Np, Nfp = Dims<N>::Nfp, Nfq = Dims<N>::Nfq, NB = 3 * N;
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= s.nb || sel[slot] != want) return;
    const int k = s.k[slot], f = s.f[slot];
    const double* g = data + (size_t)slot * dstride + doff;
    double gq[Nfq];
    for (int q = 0; q < Nfq; q++) {
        double a = 0;
        for (int j = 0; j < Nfp; j++) a += o.If[q * Nfp + j] * g[j];
        gq[q] = a * s.sJ[slot] * o.fw[q];  // W F g
    }
    const double pen = kind == 0 ? s.tau[slot] : 1.0;
    for (int i = 0; i < Nfp; i++) {
        double a = 0;
        for (int q = 0; q < Nfq; q++) a += o.If[q * Nfp + i] * gq[q];
        atomicAdd(target + (size_t)k * Np + (f * N + i) % NB, -scale * pen * a);
    }
    if (kind == 0) {
        const double ar = s.dnr[slot], as = s.dns[slot];
        for (int p = 0; p < Np; p++) {
            double a = 0;
            for (int q = 0; q < Nfq; q++) {
                const int fq = f * Nfq + q;
                a += (ar * o.Drf[fq * Np + p] + as * o.Dsf[fq * Np + p]) * gq[q];
            }
            atomicAdd(target + (size_t)k * Np + p, scale * a);
        }
    }
}

// pressure Neumann data of the fixed-velocity faces (pEqnCorrect.H:28-60,
// pCorrectEquation.H:78-93): nbp = n.(N + nu cc) at the face nodes + extra;
// nbp_old = b0 nbp + b1 nbp_prev; nbp_prev = nbp
template <int N>
__global__ void ins_nbp_kernel(InsSlots s, const int* __restrict__ ukind, int K, const double* __restrict__ Nc,
                               const double* __restrict__ cc, double nu, const double* __restrict__ extra, double b0,
                               double b1, double* __restrict__ nbp_prev, double* __restrict__ nbp_old) {
    constexpr int Np = Dims<N>::Np, Nfp = Dims<N>::Nfp, NB = 3 * N;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= s.nb * Nfp) return;
    const int slot = idx / Nfp, j = idx - slot * Nfp;
    if (ukind[slot] != 0) {
        nbp_old[idx] = 0.0;
        return;
    }
    const size_t KN = (size_t)K * Np;
    const size_t q = (size_t)s.k[slot] * Np + (s.f[slot] * N + j) % NB;
    const double cx = Nc[q] + nu * cc[q], cy = Nc[KN + q] + nu * cc[KN + q];
    const double v = s.nx[slot] * cx + s.ny[slot] * cy + extra[idx];
    nbp_old[idx] = b0 * v + b1 * nbp_prev[idx];
    nbp_prev[idx] = v;
}

// UT = (a0 U + a1 Uo - dt (b0 Nn + b1 No)) / g0
__global__ void ins_ut_kernel(size_t n, double a0, double a1, double b0, double b1, double dt, double g0,
                              const double* __restrict__ U, const double* __restrict__ Uo,
                              const double* __restrict__ Nn, const double* __restrict__ No, double* __restrict__ UT) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) UT[i] = (a0 * U[i] + a1 * Uo[i] - dt * (b0 * Nn[i] + b1 * No[i])) / g0;
}

// initial guess of a solve from the previous solutions, polynomial
// extrapolation in time: x = c0 x0 + c1 x1 + c2 x2
__global__ void ins_extrap_kernel(size_t n, double c0, double c1, double c2, const double* __restrict__ x0,
                                  const double* __restrict__ x1, const double* __restrict__ x2,
                                  double* __restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = c0 * x0[i] + (c1 != 0.0 ? c1 * x1[i] : 0.0) + (c2 != 0.0 ? c2 * x2[i] : 0.0);
}

__global__ void ins_axpy_kernel(size_t n, double a, const double* __restrict__ x, double* __restrict__ y) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] += a * x[i];
}

}  // namespace dgk

// ---------------------------------------------------------------------------
// host side

using namespace dgk;

struct dg_ins {
    dg_ctx* cp = nullptr;  // pressure operator
    dg_ctx* cu = nullptr;  // velocity (Helmholtz) operator
    int K = 0, N = 0, Np = 0, Nfp = 0, nb = 0;
    double nu = 0, dt = 0, mass_coef = -1;
    int nstep = 0;
    int pc = DG_PC_MULTILEVEL;  // block Jacobi when the multilevel preconditioner cannot be built
    int precision = DG_PREC_FP64;  // of the linear solves (dg_ins_set_precision)
    InsTables t{};
    InsSlots sl{};
    std::vector<void*> allocs;
    double *U = nullptr, *Uo = nullptr, *Nn = nullptr, *No = nullptr, *UT = nullptr, *P = nullptr, *w1 = nullptr,
           *w2 = nullptr, *rhs = nullptr, *sol = nullptr;
    double *Ph1 = nullptr, *Ph2 = nullptr;  // the two pressure solutions before P
    double* Pg = nullptr;                   // scratch: the extrapolated initial guess
    int nhist = 0;                          // valid solutions among P, Ph1, Ph2
    double *nbp_prev = nullptr, *nbp_old = nullptr, *ubnd = nullptr, *ugrad = nullptr, *pval = nullptr,
           *pext = nullptr;
    int *ukind = nullptr, *pkind = nullptr;
    std::vector<int> ukind_h, pkind_h;
    std::string err;
};

namespace {

int insfail(dg_ins* s, int code, const std::string& m) {
    s->err = m;
    return code;
}

#define INS_CUDA(ins, call)                                                                  \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) return insfail(ins, DG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
int ins_alloc(dg_ins* s, T** p, size_t n) {
    if (cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
        *p = nullptr;
        return insfail(s, DG_ERR_NOMEM, "cudaMalloc failed in dg_ins_create");
    }
    s->allocs.push_back((void*)*p);
    return DG_OK;
}

template <typename T>
int ins_upload(dg_ins* s, T** p, const std::vector<T>& h) {
    int rc = ins_alloc(s, p, h.size());
    if (rc) return rc;
    if (cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        return insfail(s, DG_ERR_CUDA, "upload failed in dg_ins_create");
    return DG_OK;
}

unsigned blocks_for(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

template <int N>
cudaError_t launch_convection(dg_ins* s, const double* u, double* out, cudaStream_t st) {
    using D = InsDims<N>;
    const int ntiles = (s->K + D::E - 1) / D::E;
    ins_convection_kernel<N><<<std::min(ntiles, 8192), D::THREADS, 0, st>>>(s->K, s->cu->d_geo, s->cu->d_conn, s->t, u,
                                                                           s->ubnd, s->ukind, out);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_nodal(dg_ins* s, int mode, const double* in, double* out, cudaStream_t st) {
    constexpr int Np = Dims<N>::Np, E = 128 / Np > 0 ? 128 / Np : 1;
    const int ntiles = (s->K + E - 1) / E;
    ins_nodal_kernel<N><<<std::min(ntiles, 8192), 128, 0, st>>>(mode, s->K, s->cu->d_geo, s->t, in, out);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_mass(dg_ins* s, double coef, const double* x, double* y, cudaStream_t st) {
    const size_t n = (size_t)s->K * Dims<N>::Np;
    ins_mass_kernel<N><<<blocks_for(n, 256), 256, 0, st>>>(s->K, ipdg_args(s->cu)->J, s->t, coef, x, y);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_bdata(dg_ins* s, const int* sel, int want, int kind, const double* data, int dstride, int doff,
                         double scale, double* target, cudaStream_t st) {
    if (s->nb == 0) return cudaSuccess;
    ins_bdata_kernel<N><<<blocks_for(s->nb, 128), 128, 0, st>>>(s->sl, ipdg_args(s->cu)->o64, sel, want, kind, data,
                                                               dstride, doff, scale, target);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_nbp(dg_ins* s, double b0, double b1, const double* cc, cudaStream_t st) {
    if (s->nb == 0) return cudaSuccess;
    const int n = s->nb * s->Nfp;
    ins_nbp_kernel<N><<<blocks_for(n, 128), 128, 0, st>>>(s->sl, s->ukind, s->K, s->Nn, cc, s->nu, s->pext, b0, b1,
                                                          s->nbp_prev, s->nbp_old);
    return cudaGetLastError();
}

template <int N>
int ins_step_n(dg_ins* s, const dg_ins_bdata* bd, double rtol, int maxit, dg_ins_stats* stats) {
    cudaStream_t st = s->cu->stream;
    const size_t KN = (size_t)s->K * s->Np, n2 = 2 * KN;
    const int nb = s->nb, Nfp = s->Nfp;
    double g0, a0, a1, b0, b1;
    if (s->nstep == 0) { g0 = 1.0; a0 = 1.0; a1 = 0.0; b0 = 1.0; b1 = 0.0; }
    else { g0 = 1.5; a0 = 2.0; a1 = -0.5; b0 = 2.0; b1 = -1.0; }
    // this step's boundary data (per slot, face-node order)
    if (nb > 0) {
        INS_CUDA(s, cudaMemcpyAsync(s->ubnd, bd->u_value, (size_t)nb * 2 * Nfp * sizeof(double), cudaMemcpyHostToDevice, st));
        INS_CUDA(s, cudaMemcpyAsync(s->ugrad, bd->u_gradient, (size_t)nb * 2 * Nfp * sizeof(double), cudaMemcpyHostToDevice, st));
        INS_CUDA(s, cudaMemcpyAsync(s->pval, bd->p_value, (size_t)nb * Nfp * sizeof(double), cudaMemcpyHostToDevice, st));
        INS_CUDA(s, cudaMemcpyAsync(s->pext, bd->p_neumann_extra, (size_t)nb * Nfp * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    // 1-2: convection and the extrapolated intermediate velocity
    INS_CUDA(s, launch_convection<N>(s, s->U, s->Nn, st));
    dgk::ins_ut_kernel<<<blocks_for(n2, 256), 256, 0, st>>>(n2, a0, a1, b0, b1, s->dt, g0, s->U, s->Uo, s->Nn, s->No, s->UT);
    INS_CUDA(s, cudaGetLastError());
    // 3: pressure Neumann data
    INS_CUDA(s, launch_nodal<N>(s, 2, s->U, s->w2, st));
    INS_CUDA(s, launch_nbp<N>(s, b0, b1, s->w2, st));
    // 4: pressure: S_p p = -(q3 b_Lp + F^T W F nbp_old + (g0/dt) M div UT)
    INS_CUDA(s, launch_nodal<N>(s, 0, s->UT, s->w1, st));
    INS_CUDA(s, launch_mass<N>(s, -g0 / s->dt, s->w1, s->rhs, st));
    INS_CUDA(s, launch_bdata<N>(s, s->pkind, 0, 0, s->pval, Nfp, 0, -bd->p_data_scale, s->rhs, st));
    // + F^T W F nbp_old: the face-mass kernel adds -scale F^T W F g
    INS_CUDA(s, launch_bdata<N>(s, s->ukind, 0, 1, s->nbp_old, Nfp, 0, 1.0, s->rhs, st));
    int itp = 0, itu[2] = {0, 0};
    double relp = 0, relu[2] = {0, 0};
    // initial guess: the pressure extrapolated in time from the last solutions
    // (quadratic from three, linear from two); the solution changes only by the
    // solver tolerance, the iteration count drops
    {
        double c0 = 1, c1 = 0, c2 = 0;
        if (s->nhist >= 3) { c0 = 3; c1 = -3; c2 = 1; }
        else if (s->nhist == 2) { c0 = 2; c1 = -1; }
        dgk::ins_extrap_kernel<<<blocks_for(KN, 256), 256, 0, st>>>(KN, c0, c1, c2, s->P, s->Ph1, s->Ph2, s->Pg);
        INS_CUDA(s, cudaGetLastError());
        // history rotation: Ph2 <- Ph1 <- P, the guess becomes the solve's vector
        double* freed = s->Ph2;
        s->Ph2 = s->Ph1;
        s->Ph1 = s->P;
        s->P = s->Pg;
        s->Pg = freed;
        s->nhist = std::min(s->nhist + 1, 3);
    }
    int rc = ipdg_solve_device(s->cp, s->rhs, s->P, rtol, maxit, &itp, &relp, s->pc, s->precision);
    if (rc == DG_ERR_UNSUPPORTED && s->pc == DG_PC_MULTILEVEL) {
        s->pc = DG_PC_BLOCK_JACOBI;  // no multilevel preconditioner on this mesh: block Jacobi
        rc = ipdg_solve_device(s->cp, s->rhs, s->P, rtol, maxit, &itp, &relp, s->pc, s->precision);
    }
    if (rc) return insfail(s, rc, std::string("pressure solve: ") + s->cp->err);
    // 5: velocity correction
    INS_CUDA(s, launch_nodal<N>(s, 1, s->P, s->w2, st));
    dgk::ins_axpy_kernel<<<blocks_for(n2, 256), 256, 0, st>>>(n2, -s->dt / g0, s->w2, s->UT);
    INS_CUDA(s, cudaGetLastError());
    // 6: viscous step, per component
    const double tmp = g0 / (s->dt * s->nu);
    if (tmp != s->mass_coef) {
        rc = dg_ipdg_set_mass(s->cu, tmp);
        if (rc) return insfail(s, rc, std::string("Helmholtz operator: ") + s->cu->err);
        s->mass_coef = tmp;
    }
    for (int c = 0; c < 2; c++) {
        INS_CUDA(s, launch_mass<N>(s, tmp, s->UT + c * KN, s->rhs, st));
        // - q4 b_LU: Dirichlet terms on fixed-value slots, -F^T W F h on fixed-gradient slots
        INS_CUDA(s, launch_bdata<N>(s, s->ukind, 0, 0, s->ubnd, 2 * Nfp, c * Nfp, -bd->u_data_scale, s->rhs, st));
        INS_CUDA(s, launch_bdata<N>(s, s->ukind, 1, 1, s->ugrad, 2 * Nfp, c * Nfp, -bd->u_data_scale, s->rhs, st));
        // initial guess: U extrapolated linearly in time (U itself on the first step)
        dgk::ins_extrap_kernel<<<blocks_for(KN, 256), 256, 0, st>>>(KN, s->nstep > 0 ? 2.0 : 1.0,
                                                                    s->nstep > 0 ? -1.0 : 0.0, 0.0, s->U + c * KN,
                                                                    s->Uo + c * KN, nullptr, s->sol + c * KN);
        INS_CUDA(s, cudaGetLastError());
        rc = ipdg_solve_device(s->cu, s->rhs, s->sol + c * KN, rtol, maxit, &itu[c], &relu[c], s->pc, s->precision);
        if (rc) return insfail(s, rc, std::string("velocity solve: ") + s->cu->err);
    }
    cudaEventRecord(e1, st);
    // shift the time levels: U_old <- U, U <- solution, N_old <- N
    std::swap(s->Uo, s->U);
    std::swap(s->U, s->sol);
    std::swap(s->No, s->Nn);
    INS_CUDA(s, cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s->nstep++;
    if (stats) {
        stats->iterations_p = itp;
        stats->iterations_u[0] = itu[0];
        stats->iterations_u[1] = itu[1];
        stats->rel_residual_p = relp;
        stats->rel_residual_u = std::max(relu[0], relu[1]);
        stats->ms = ms;
    }
    return DG_OK;
}

}  // namespace

extern "C" {

int dg_ins_create(const dg_mesh_desc* mesh, const dg_opts* opts, const int* u_kind, const int* p_kind, double nu,
                  double dt, double tau_coef, dg_ins** out) {
    if (!mesh || !opts || !out || !(nu > 0) || !(dt > 0) || !(tau_coef > 0)) return DG_ERR_ARG;
    *out = nullptr;
    dg_ins* s = new dg_ins();
    // both operators on one stream (the step's kernels and solves are ordered on it)
    int rc = dg_ctx_create(mesh, opts, &s->cp);
    if (!rc) {
        dg_opts o2 = *opts;
        o2.stream = (void*)s->cp->stream;
        rc = dg_ctx_create(mesh, &o2, &s->cu);
    }
    if (rc) { dg_ins_destroy(s); return rc; }
    dg_ctx* c = s->cu;
    s->K = c->K;
    s->N = c->N;
    s->Np = c->Np;
    s->Nfp = c->Nfp;
    s->nb = c->nb;
    s->nu = nu;
    s->dt = dt;
    if (c->N < 1 || c->N > 7) { dg_ins_destroy(s); return DG_ERR_UNSUPPORTED; }
    if (s->nb > 0 && (!u_kind || !p_kind)) { dg_ins_destroy(s); return DG_ERR_ARG; }
    s->ukind_h.assign(u_kind, u_kind + s->nb);
    s->pkind_h.assign(p_kind, p_kind + s->nb);
    std::vector<int> bt_u(s->nb), bt_p(s->nb);
    for (int i = 0; i < s->nb; i++) {
        if ((u_kind[i] != 0 && u_kind[i] != 1) || (p_kind[i] != 0 && p_kind[i] != 2)) {
            dg_ins_destroy(s);
            return DG_ERR_ARG;
        }
        bt_u[i] = u_kind[i];
        bt_p[i] = p_kind[i];
    }
    if ((rc = dg_ipdg_setup(s->cp, tau_coef)) || (rc = dg_ipdg_setup(s->cu, tau_coef)) ||
        (rc = dg_ipdg_set_boundary_types(s->cp, bt_p.data())) || (rc = dg_ipdg_set_boundary_types(s->cu, bt_u.data()))) {
        dg_ins_destroy(s);
        return rc;
    }
    // ring-order tables
    const dgb::RefOps& o = c->ops;
    const int Np = s->Np;
    std::vector<double> Dr((size_t)Np * Np), Ds((size_t)Np * Np), Mr((size_t)Np * Np);
    for (int i = 0; i < Np; i++)
        for (int j = 0; j < Np; j++) {
            Dr[(size_t)i * Np + j] = o.Dr[(size_t)o.ring[i] * Np + o.ring[j]];
            Ds[(size_t)i * Np + j] = o.Ds[(size_t)o.ring[i] * Np + o.ring[j]];
            Mr[(size_t)i * Np + j] = o.Mref[(size_t)o.ring[i] * Np + o.ring[j]];
        }
    rc = 0;
    rc |= ins_upload(s, (double**)&s->t.Dr, Dr);
    rc |= ins_upload(s, (double**)&s->t.Ds, Ds);
    rc |= ins_upload(s, (double**)&s->t.Mr, Mr);
    s->t.Vg = c->d_Vg;
    s->t.Sr = c->d_Sr;
    s->t.Ss = c->d_Ss;
    s->t.Lift = c->d_Lift;
    s->t.If = c->d_If;
    // boundary slots (the context's numbering: boundary faces in element, face order)
    const std::vector<double>& fc = *ipdg_face_coefs(c);
    std::vector<int> bk, bf;
    std::vector<double> bsj, btau, bdr, bds, bnx, bny;
    for (int k = 0; k < s->K; k++)
        for (int f = 0; f < 3; f++) {
            const int cn = c->conn_host[(size_t)k * 3 + f];
            if (cn >= 0) continue;
            const double* g = &c->geo_host[4 * (size_t)k];
            double nx, ny, fsc;
            face_normal(f, g[0], g[1], g[2], g[3], nx, ny, fsc);
            const double* fk = &fc[((size_t)k * 3 + f) * kFaceCoef];
            bk.push_back(k);
            bf.push_back(f);
            bsj.push_back(fk[5]);
            btau.push_back(2.0 * fk[4]);
            bdr.push_back(fk[0]);
            bds.push_back(fk[1]);
            bnx.push_back(nx);
            bny.push_back(ny);
        }
    s->sl.nb = s->nb;
    rc |= ins_upload(s, (int**)&s->sl.k, bk);
    rc |= ins_upload(s, (int**)&s->sl.f, bf);
    rc |= ins_upload(s, (double**)&s->sl.sJ, bsj);
    rc |= ins_upload(s, (double**)&s->sl.tau, btau);
    rc |= ins_upload(s, (double**)&s->sl.dnr, bdr);
    rc |= ins_upload(s, (double**)&s->sl.dns, bds);
    rc |= ins_upload(s, (double**)&s->sl.nx, bnx);
    rc |= ins_upload(s, (double**)&s->sl.ny, bny);
    rc |= ins_upload(s, &s->ukind, s->ukind_h);
    rc |= ins_upload(s, &s->pkind, s->pkind_h);
    const size_t KN = (size_t)s->K * Np;
    for (double** p : {&s->U, &s->Uo, &s->Nn, &s->No, &s->UT, &s->w2, &s->sol}) rc |= ins_alloc(s, p, 2 * KN);
    for (double** p : {&s->P, &s->w1, &s->rhs, &s->Ph1, &s->Ph2, &s->Pg}) rc |= ins_alloc(s, p, KN);
    const size_t nbf = (size_t)std::max(s->nb, 1) * s->Nfp;
    for (double** p : {&s->nbp_prev, &s->nbp_old, &s->pval, &s->pext}) rc |= ins_alloc(s, p, nbf);
    for (double** p : {&s->ubnd, &s->ugrad}) rc |= ins_alloc(s, p, 2 * nbf);
    if (rc) { dg_ins_destroy(s); return DG_ERR_NOMEM; }
    for (double* p : {s->U, s->Uo, s->Nn, s->No, s->UT, s->w2, s->sol}) cudaMemset(p, 0, 2 * KN * sizeof(double));
    for (double* p : {s->P, s->w1, s->rhs, s->Ph1, s->Ph2, s->Pg}) cudaMemset(p, 0, KN * sizeof(double));
    for (double* p : {s->nbp_prev, s->nbp_old, s->pval, s->pext}) cudaMemset(p, 0, nbf * sizeof(double));
    for (double* p : {s->ubnd, s->ugrad}) cudaMemset(p, 0, 2 * nbf * sizeof(double));
    if (cudaDeviceSynchronize() != cudaSuccess) { dg_ins_destroy(s); return DG_ERR_CUDA; }
    *out = s;
    return DG_OK;
}

int dg_ins_set_precision(dg_ins* s, int precision) {
    if (!s || (precision != DG_PREC_FP64 && precision != DG_PREC_SPLIT)) return DG_ERR_ARG;
    s->precision = precision;
    return DG_OK;
}

int dg_ins_destroy(dg_ins* s) {
    if (!s) return DG_OK;
    if (s->cu && s->cu->stream) cudaStreamSynchronize(s->cu->stream);
    for (void* p : s->allocs) cudaFree(p);
    if (s->cu) dg_ctx_destroy(s->cu);  // borrows the stream of cp: destroyed first
    if (s->cp) dg_ctx_destroy(s->cp);
    delete s;
    return DG_OK;
}

const char* dg_ins_last_error(const dg_ins* s) { return s ? s->err.c_str() : ""; }

int dg_ins_set_state(dg_ins* s, const double* U_host, const double* p_host) {
    if (!s || !U_host || !p_host) return DG_ERR_ARG;
    cudaStream_t st = s->cu->stream;
    const size_t KN = (size_t)s->K * s->Np;
    for (int c = 0; c < 2; c++) {
        INS_CUDA(s, cudaMemcpyAsync(s->w1, U_host + c * KN, KN * sizeof(double), cudaMemcpyHostToDevice, st));
        INS_CUDA(s, launch_permute(s->w1, s->U + c * KN, s->cu->d_ring, s->K, s->Np, true, st));
    }
    INS_CUDA(s, cudaMemcpyAsync(s->Uo, s->U, 2 * KN * sizeof(double), cudaMemcpyDeviceToDevice, st));
    INS_CUDA(s, cudaMemsetAsync(s->Nn, 0, 2 * KN * sizeof(double), st));
    INS_CUDA(s, cudaMemsetAsync(s->No, 0, 2 * KN * sizeof(double), st));
    INS_CUDA(s, cudaMemsetAsync(s->nbp_prev, 0, (size_t)std::max(s->nb, 1) * s->Nfp * sizeof(double), st));
    INS_CUDA(s, cudaMemcpyAsync(s->w1, p_host, KN * sizeof(double), cudaMemcpyHostToDevice, st));
    INS_CUDA(s, launch_permute(s->w1, s->P, s->cu->d_ring, s->K, s->Np, true, st));
    INS_CUDA(s, cudaStreamSynchronize(st));
    s->nstep = 0;
    s->nhist = 1;
    return DG_OK;
}

int dg_ins_get_state(dg_ins* s, double* U_host, double* p_host) {
    if (!s || !U_host || !p_host) return DG_ERR_ARG;
    cudaStream_t st = s->cu->stream;
    const size_t KN = (size_t)s->K * s->Np;
    for (int c = 0; c < 2; c++) {
        INS_CUDA(s, launch_permute(s->U + c * KN, s->w1, s->cu->d_ring, s->K, s->Np, false, st));
        INS_CUDA(s, cudaMemcpyAsync(U_host + c * KN, s->w1, KN * sizeof(double), cudaMemcpyDeviceToHost, st));
        INS_CUDA(s, cudaStreamSynchronize(st));
    }
    INS_CUDA(s, launch_permute(s->P, s->w1, s->cu->d_ring, s->K, s->Np, false, st));
    INS_CUDA(s, cudaMemcpyAsync(p_host, s->w1, KN * sizeof(double), cudaMemcpyDeviceToHost, st));
    INS_CUDA(s, cudaStreamSynchronize(st));
    return DG_OK;
}

int dg_ins_step(dg_ins* s, const dg_ins_bdata* bd, double rtol, int maxit, dg_ins_stats* stats) {
    if (!s || !bd || !(rtol > 0) || maxit < 1) return DG_ERR_ARG;
    if (s->nb > 0 && (!bd->u_value || !bd->u_gradient || !bd->p_value || !bd->p_neumann_extra)) return DG_ERR_ARG;
    switch (s->N) {
        case 1: return ins_step_n<1>(s, bd, rtol, maxit, stats);
        case 2: return ins_step_n<2>(s, bd, rtol, maxit, stats);
        case 3: return ins_step_n<3>(s, bd, rtol, maxit, stats);
        case 4: return ins_step_n<4>(s, bd, rtol, maxit, stats);
        case 5: return ins_step_n<5>(s, bd, rtol, maxit, stats);
        case 6: return ins_step_n<6>(s, bd, rtol, maxit, stats);
        case 7: return ins_step_n<7>(s, bd, rtol, maxit, stats);
        default: return DG_ERR_UNSUPPORTED;
    }
}

// the step's operators alone, for parity tests: op 0 convection (U -> N, with
// the boundary values of bd), 1 div, 2 grad, 3 curl curl; host arrays in the
// reference node order, component-major
int dg_ins_operator(dg_ins* s, int op, const dg_ins_bdata* bd, const double* in_host, double* out_host) {
    if (!s || !in_host || !out_host || op < 0 || op > 3) return DG_ERR_ARG;
    cudaStream_t st = s->cu->stream;
    const size_t KN = (size_t)s->K * s->Np;
    const int nin = (op == 2) ? 1 : 2, nout = (op == 1) ? 1 : 2;
    if (op == 0 && s->nb > 0) {
        if (!bd || !bd->u_value) return DG_ERR_ARG;
        INS_CUDA(s, cudaMemcpyAsync(s->ubnd, bd->u_value, (size_t)s->nb * 2 * s->Nfp * sizeof(double),
                                    cudaMemcpyHostToDevice, st));
    }
    for (int c = 0; c < nin; c++) {
        INS_CUDA(s, cudaMemcpyAsync(s->w1, in_host + c * KN, KN * sizeof(double), cudaMemcpyHostToDevice, st));
        INS_CUDA(s, launch_permute(s->w1, s->UT + c * KN, s->cu->d_ring, s->K, s->Np, true, st));
    }
    cudaError_t e = cudaSuccess;
    auto run = [&](auto tag) {
        constexpr int N = decltype(tag)::value;
        if (op == 0) e = launch_convection<N>(s, s->UT, s->w2, st);
        else e = launch_nodal<N>(s, op == 1 ? 0 : (op == 2 ? 1 : 2), s->UT, s->w2, st);
    };
    switch (s->N) {
        case 1: run(std::integral_constant<int, 1>()); break;
        case 2: run(std::integral_constant<int, 2>()); break;
        case 3: run(std::integral_constant<int, 3>()); break;
        case 4: run(std::integral_constant<int, 4>()); break;
        case 5: run(std::integral_constant<int, 5>()); break;
        case 6: run(std::integral_constant<int, 6>()); break;
        case 7: run(std::integral_constant<int, 7>()); break;
    }
    INS_CUDA(s, e);
    for (int c = 0; c < nout; c++) {
        INS_CUDA(s, launch_permute(s->w2 + c * KN, s->w1, s->cu->d_ring, s->K, s->Np, false, st));
        INS_CUDA(s, cudaMemcpyAsync(out_host + c * KN, s->w1, KN * sizeof(double), cudaMemcpyDeviceToHost, st));
        INS_CUDA(s, cudaStreamSynchronize(st));
    }
    return DG_OK;
}

}  // extern "C"
