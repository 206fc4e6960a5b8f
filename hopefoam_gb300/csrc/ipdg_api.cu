// ipdg_api.cu -- C ABI of the SIPG pressure operator and its PCG solve.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dgcu.h"
#include "dg_ctx.hpp"
#include "ipdg.hpp"

using namespace dgk;

struct IpdgState {
    bool ready = false;
    double tau_coef = 20.0;
    IpdgArgs args;
    std::vector<void*> allocs;
    double *d_J = nullptr, *d_Srr = nullptr, *d_Srs2 = nullptr, *d_Sss = nullptr, *d_Drf = nullptr, *d_Dsf = nullptr,
           *d_fw = nullptr;
    double* d_blocks = nullptr;  // FP64 inverse diagonal blocks
    float* d_blocks32 = nullptr;
    // solver vectors (ring order)
    double *d_b = nullptr, *d_x = nullptr, *d_e = nullptr, *d_r = nullptr, *d_z = nullptr, *d_p = nullptr,
           *d_Ap = nullptr, *d_part = nullptr;
    PcgScalars* d_S = nullptr;
    double* d_scal = nullptr;  // small FP64 results (dot products)
    int* d_status = nullptr;
    int G = 608;
};

namespace {

int ifail(dg_ctx* c, int code, const std::string& m) {
    c->err = m;
    return code;
}

#define IP_CUDA(ctx, call)                                                                   \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) return ifail(ctx, DG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
int ialloc(dg_ctx* c, IpdgState* s, T** p, size_t n) {
    if (cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
        *p = nullptr;
        return ifail(c, DG_ERR_NOMEM, "cudaMalloc failed in dg_ipdg_setup");
    }
    s->allocs.push_back((void*)*p);
    return DG_OK;
}

template <typename T>
int iupload(dg_ctx* c, IpdgState* s, T** p, const std::vector<T>& h) {
    int rc = ialloc(c, s, p, h.size());
    if (rc) return rc;
    IP_CUDA(c, cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return DG_OK;
}

// y = S x (FP64) on ring-order device vectors
int apply64(dg_ctx* c, const double* x, double* y) {
    IpdgState* s = c->ipdg;
    cudaError_t e = launch_ipdg_apply(s->args, false, x, y, nullptr, s->G, c->stream);
    if (e != cudaSuccess) return ifail(c, DG_ERR_CUDA, std::string("ipdg apply: ") + cudaGetErrorString(e));
    return DG_OK;
}

int dot_host(dg_ctx* c, const double* x, const double* y, double* out) {
    IpdgState* s = c->ipdg;
    const size_t n = (size_t)c->K * c->Np;
    IP_CUDA(c, launch_dot(x, y, n, s->d_part, s->G, c->stream));
    IP_CUDA(c, launch_reduce_to(s->d_part, s->G, s->d_scal, c->stream));
    IP_CUDA(c, cudaMemcpyAsync(out, s->d_scal, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    IP_CUDA(c, cudaStreamSynchronize(c->stream));
    return DG_OK;
}

// runs PCG iterations on S e = r (vectors in v) until S->done or `limit`
// iterations; returns the iterations taken and the stop code
int run_cg(dg_ctx* c, const PcgVecs& v, bool fp32, double tol2, int limit, int* iters, int* stop) {
    IpdgState* s = c->ipdg;
    PcgScalars h;
    memset(&h, 0, sizeof(h));
    h.tol2 = tol2;
    IP_CUDA(c, cudaMemcpyAsync(s->d_S, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
    IP_CUDA(c, launch_pcg_init(s->args, v, c->stream));
    const int CHECK = 16;
    int issued = 0;
    *stop = 0;
    *iters = 0;
    while (issued < limit) {
        const int batch = std::min(CHECK, limit - issued);
        for (int j = 0; j < batch; j++) {
            IP_CUDA(c, launch_pcg_iteration(s->args, v, fp32, (issued + j) & 1, c->stream));
        }
        issued += batch;
        IP_CUDA(c, cudaMemcpyAsync(&h, s->d_S, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
        IP_CUDA(c, cudaStreamSynchronize(c->stream));
        if (h.done) break;
    }
    *iters = h.it;
    *stop = h.done;
    return DG_OK;
}

}  // namespace

void ipdg_teardown(dg_ctx* c) {
    if (!c->ipdg) return;
    for (void* p : c->ipdg->allocs) cudaFree(p);
    delete c->ipdg;
    c->ipdg = nullptr;
}

extern "C" {

int dg_ipdg_setup(dg_ctx* c, double tau_coef) {
    if (!c || !(tau_coef > 0)) return DG_ERR_ARG;
    ipdg_teardown(c);
    IpdgState* s = new IpdgState();
    c->ipdg = s;
    s->tau_coef = tau_coef;
    const dgb::RefOps& o = c->ops;
    const int Np = c->Np, Ng = c->Ng, Nfp = c->Nfp, Nfq = c->Nfq, K = c->K;
    // reference stiffness parts (ring order)
    std::vector<double> Srr((size_t)Np * Np, 0.0), Srs2((size_t)Np * Np, 0.0), Sss((size_t)Np * Np, 0.0);
    for (int i = 0; i < Np; i++)
        for (int j = 0; j < Np; j++) {
            const int ri = o.ring[i], rj = o.ring[j];
            double a = 0, b = 0, d = 0;
            for (int g = 0; g < Ng; g++) {
                const double dri = o.Drg[(size_t)g * Np + ri], dsi = o.Dsg[(size_t)g * Np + ri];
                const double drj = o.Drg[(size_t)g * Np + rj], dsj = o.Dsg[(size_t)g * Np + rj];
                a += o.gw[g] * dri * drj;
                b += o.gw[g] * (dri * dsj + dsi * drj);
                d += o.gw[g] * dsi * dsj;
            }
            Srr[(size_t)i * Np + j] = a;
            Srs2[(size_t)i * Np + j] = b;
            Sss[(size_t)i * Np + j] = d;
        }
    // derivatives of the nodal basis at each face's Gauss points (face-node Dr rows interpolated)
    std::vector<double> Drf((size_t)3 * Nfq * Np, 0.0), Dsf((size_t)3 * Nfq * Np, 0.0);
    for (int f = 0; f < 3; f++)
        for (int g = 0; g < Nfq; g++)
            for (int p = 0; p < Np; p++) {
                const int rp = o.ring[p];
                double a = 0, b = 0;
                for (int j = 0; j < Nfp; j++) {
                    const int node = o.fnode[f * Nfp + j];
                    a += o.If[(size_t)g * Nfp + j] * o.Dr[(size_t)node * Np + rp];
                    b += o.If[(size_t)g * Nfp + j] * o.Ds[(size_t)node * Np + rp];
                }
                Drf[((size_t)f * Nfq + g) * Np + p] = a;
                Dsf[((size_t)f * Nfq + g) * Np + p] = b;
            }
    std::vector<double> J(K);
    for (int k = 0; k < K; k++) {
        const double* g = &c->geo_host[4 * (size_t)k];
        J[k] = 1.0 / (g[0] * g[3] - g[1] * g[2]);
    }
    int rc = 0;
    rc |= iupload(c, s, &s->d_J, J);
    rc |= iupload(c, s, &s->d_Srr, Srr);
    rc |= iupload(c, s, &s->d_Srs2, Srs2);
    rc |= iupload(c, s, &s->d_Sss, Sss);
    rc |= iupload(c, s, &s->d_Drf, Drf);
    rc |= iupload(c, s, &s->d_Dsf, Dsf);
    rc |= iupload(c, s, &s->d_fw, o.fw);
    const size_t n = (size_t)K * Np;
    rc |= ialloc(c, s, &s->d_blocks, n * Np);
    rc |= ialloc(c, s, &s->d_blocks32, n * Np);
    rc |= ialloc(c, s, &s->d_b, n);
    rc |= ialloc(c, s, &s->d_x, n);
    rc |= ialloc(c, s, &s->d_e, n);
    rc |= ialloc(c, s, &s->d_r, n);
    rc |= ialloc(c, s, &s->d_z, n);
    rc |= ialloc(c, s, &s->d_p, n);
    rc |= ialloc(c, s, &s->d_Ap, n);
    rc |= ialloc(c, s, &s->d_part, (size_t)5 * s->G);
    rc |= ialloc(c, s, &s->d_S, 1);
    rc |= ialloc(c, s, &s->d_scal, 4);
    rc |= ialloc(c, s, &s->d_status, 1);
    if (rc) return DG_ERR_NOMEM;
    IpdgArgs& a = s->args;
    a.K = K;
    a.N = c->N;
    a.Np = Np;
    a.Nfp = Nfp;
    a.Nfq = Nfq;
    a.tau_coef = tau_coef;
    a.geo = c->d_geo;
    a.J = s->d_J;
    a.conn = c->d_conn;
    a.Srr = s->d_Srr;
    a.Srs2 = s->d_Srs2;
    a.Sss = s->d_Sss;
    a.Drf = s->d_Drf;
    a.Dsf = s->d_Dsf;
    a.If = c->d_If;
    a.fw = s->d_fw;
    IP_CUDA(c, cudaMemsetAsync(s->d_status, 0, sizeof(int), c->stream));
    IP_CUDA(c, launch_ipdg_diag(a, s->d_blocks, c->stream));
    IP_CUDA(c, launch_invert_blocks(s->d_blocks, s->d_blocks32, K, Np, s->d_status, c->stream));
    int st = 0;
    IP_CUDA(c, cudaMemcpyAsync(&st, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    IP_CUDA(c, cudaStreamSynchronize(c->stream));
    if (st) return ifail(c, DG_ERR_NONFINITE, "singular diagonal block in the SIPG operator");
    s->ready = true;
    return DG_OK;
}

int dg_ipdg_apply(dg_ctx* c, const double* x_host, double* y_host) {
    if (!c || !x_host || !y_host) return DG_ERR_ARG;
    if (!c->ipdg || !c->ipdg->ready) return ifail(c, DG_ERR_ARG, "dg_ipdg_setup not called");
    IpdgState* s = c->ipdg;
    const size_t n = (size_t)c->K * c->Np;
    IP_CUDA(c, cudaMemcpyAsync(s->d_z, x_host, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    IP_CUDA(c, launch_permute(s->d_z, s->d_p, c->d_ring, c->K, c->Np, true, c->stream));
    int rc = apply64(c, s->d_p, s->d_Ap);
    if (rc) return rc;
    IP_CUDA(c, launch_permute(s->d_Ap, s->d_z, c->d_ring, c->K, c->Np, false, c->stream));
    IP_CUDA(c, cudaMemcpyAsync(y_host, s->d_z, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    IP_CUDA(c, cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_pcg_solve(dg_ctx* c, const double* b_host, double* x_host, double rtol, int maxit, int pc, int precision,
                 dg_solve_stats* stats) {
    if (!c || !b_host || !x_host || !(rtol > 0) || maxit < 1) return DG_ERR_ARG;
    if (!c->ipdg || !c->ipdg->ready) return ifail(c, DG_ERR_ARG, "dg_ipdg_setup not called");
    if (pc != DG_PC_BLOCK_JACOBI) return ifail(c, DG_ERR_UNSUPPORTED, "preconditioner not available");
    if (precision != DG_PREC_FP64 && precision != DG_PREC_SPLIT) return ifail(c, DG_ERR_ARG, "unknown precision");
    IpdgState* s = c->ipdg;
    const size_t n = (size_t)c->K * c->Np;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    IP_CUDA(c, cudaMemcpyAsync(s->d_z, b_host, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    IP_CUDA(c, launch_permute(s->d_z, s->d_b, c->d_ring, c->K, c->Np, true, c->stream));
    IP_CUDA(c, cudaMemcpyAsync(s->d_z, x_host, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    IP_CUDA(c, launch_permute(s->d_z, s->d_x, c->d_ring, c->K, c->Np, true, c->stream));
    cudaEventRecord(e0, c->stream);
    double bb = 0;
    int rc = dot_host(c, s->d_b, s->d_b, &bb);
    if (rc) return rc;
    PcgVecs v;
    v.r = s->d_r;
    v.z = s->d_z;
    v.p = s->d_p;
    v.Ap = s->d_Ap;
    v.part_pap = s->d_part;
    v.part_rz = s->d_part + s->G;  // [2][G]
    v.part_rr = s->d_part + 3 * s->G;
    v.part_rzo = s->d_part + 4 * s->G;
    v.P32 = s->d_blocks32;
    v.P64 = nullptr;
    v.S = s->d_S;
    v.G = s->G;
    int total_it = 0, stop = 0;
    double rel = 0;
    if (bb == 0.0) {
        IP_CUDA(c, cudaMemsetAsync(s->d_x, 0, n * sizeof(double), c->stream));
    } else if (precision == DG_PREC_FP64) {
        // plain PCG, FP64 operator every iteration
        rc = apply64(c, s->d_x, s->d_Ap);
        if (rc) return rc;
        IP_CUDA(c, launch_xmy(s->d_r, s->d_b, s->d_Ap, n, c->stream));
        v.x = s->d_x;
        v.P64 = s->d_blocks;  // FP64 preconditioner: an inexact one stalls CG at high condition numbers
        rc = run_cg(c, v, false, rtol * rtol * bb, maxit, &total_it, &stop);
        if (rc) return rc;
    } else {
        // mixed-precision refinement: FP32-arithmetic operator inside CG, FP64 outer residual
        for (int outer = 0; outer < 20 && total_it < maxit; outer++) {
            rc = apply64(c, s->d_x, s->d_Ap);
            if (rc) return rc;
            IP_CUDA(c, launch_xmy(s->d_r, s->d_b, s->d_Ap, n, c->stream));
            double rr = 0;
            rc = dot_host(c, s->d_r, s->d_r, &rr);
            if (rc) return rc;
            if (!(rr == rr)) { stop = 2; break; }
            if (rr <= rtol * rtol * bb) { stop = 1; break; }
            IP_CUDA(c, cudaMemsetAsync(s->d_e, 0, n * sizeof(double), c->stream));
            v.x = s->d_e;
            const double tol2 = std::max(0.25 * rtol * rtol * bb, 1e-12 * rr);
            int it = 0, st = 0;
            rc = run_cg(c, v, true, tol2, maxit - total_it, &it, &st);
            if (rc) return rc;
            total_it += it;
            if (st == 2) { stop = 2; break; }
            IP_CUDA(c, launch_axpy(s->d_x, s->d_e, 1.0, n, c->stream));
        }
    }
    // true FP64 residual
    rc = apply64(c, s->d_x, s->d_Ap);
    if (rc) return rc;
    IP_CUDA(c, launch_xmy(s->d_r, s->d_b, s->d_Ap, n, c->stream));
    double rr = 0;
    rc = dot_host(c, s->d_r, s->d_r, &rr);
    if (rc) return rc;
    cudaEventRecord(e1, c->stream);
    IP_CUDA(c, launch_permute(s->d_x, s->d_z, c->d_ring, c->K, c->Np, false, c->stream));
    IP_CUDA(c, cudaMemcpyAsync(x_host, s->d_z, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    IP_CUDA(c, cudaStreamSynchronize(c->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    rel = bb > 0 ? std::sqrt(rr / bb) : 0.0;
    if (stats) {
        stats->iterations = total_it;
        stats->rel_residual = rel;
        stats->ms = ms;
    }
    if (!(rel == rel) || stop == 2) return ifail(c, DG_ERR_NONFINITE, "PCG breakdown or non-finite residual");
    if (rel > rtol) return ifail(c, DG_ERR_NOT_CONVERGED, "PCG reached the iteration limit");
    return DG_OK;
}

}  // extern "C"
