// ipdg_api.cu -- C ABI of the SIPG pressure operator and its PCG solve.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/dgcu.h"
#include "dg_ctx.hpp"
#include "euler_flux.cuh"
#include "ipdg.hpp"
#include "lpc.hpp"
#include "mg.hpp"

#include <random>

using namespace dgk;

struct IpdgState {
    bool ready = false;
    double tau_coef = 20.0;
    IpdgArgs args;
    std::vector<void*> allocs;
    double* d_J = nullptr;
    IpdgOps<double> o64h{};  // device pointers of the operator tables
    IpdgOps<float> o32h{};
    // multilevel preconditioner (DG_PC_MULTILEVEL); rebuilt when the operator changes
    MgLevels mg{};
    bool mg_ready = false;
    std::string mg_err;
    std::vector<void*> mg_allocs;
    std::vector<double> fc_host;  // face coefficients as built (boundary types reset sJ from it)
    std::vector<unsigned char> lane_tab;  // IpLaneTab<N> of the two-pass FP32 apply (N <= 5)
    std::vector<int> btype;       // per boundary slot: 0 fixesValue, 1 fixesGradient, 2 neither
    double* d_blocks = nullptr;  // FP64 inverse diagonal blocks (row-major per element)
    double* d_P64 = nullptr;     // the same, grouped layout of the element-aligned kernels
    float* d_P32 = nullptr;      // FP32 copy, grouped
    // solver vectors (ring order)
    double *d_b = nullptr, *d_x = nullptr, *d_r = nullptr, *d_z = nullptr, *d_p = nullptr, *d_p2 = nullptr,
           *d_Ap = nullptr, *d_part = nullptr;
    double* d_ppart = nullptr;  // [3][nmax] partials of the PCG grid-wide sums
    float *d_dz = nullptr, *d_dp = nullptr, *d_dp2 = nullptr;  // FP32 offset mirrors of z and p
    float* d_r32 = nullptr;      // FP32 copy of r (learned Schwarz mode)
    float* d_lane_ftr = nullptr;  // face records of the two-pass FP32 apply (N <= 5)
    float2* d_lane_p0 = nullptr;  // first-node values of its input (FP32 pairs)
    int nmax = 0;
    int sms = 1;
    PcgScalars* d_S = nullptr;
    double* d_scal = nullptr;  // small FP64 results (dot products)
    int* d_status = nullptr;
    int G = 608;
    // learned preconditioner
    bool lpc_ready = false;
    int F = 0, H = 128;
    int lpc_linear = 0;
    int lpc_form = DG_LPC_RELU;
    SchwarzArgs sw{};                 // learned additive-Schwarz form
    float* d_U = nullptr;             // its local outputs (K x F)
    int* d_iperm = nullptr;
    float *d_Xs = nullptr, *d_As = nullptr, *d_C = nullptr;  // training: gathered rows, F x F cross term
    double* d_gvec = nullptr;         // training: output-gradient vector
    int* d_tcstatus = nullptr;        // timeout flag of the tensor-core local stage
    float* d_wpart = nullptr;         // two-layer form: per-CTA weight-gradient partials
    bool lpc_coarse = false;          // training: z = learned local stage + the coarse-space correction
    float *d_W1 = nullptr, *d_W2 = nullptr, *d_m1 = nullptr, *d_v1 = nullptr, *d_m2 = nullptr, *d_v2 = nullptr;
    float *d_g1 = nullptr, *d_g2 = nullptr;
    __nv_bfloat16 *d_W1b = nullptr, *d_W2b = nullptr;
    int* d_perm = nullptr;
    double* d_zb = nullptr;
    double* d_zl = nullptr;  // learned + multilevel: the learned output before the coarse correction
    float* d_sc = nullptr;  // per-element feature scale
    __nv_bfloat16* d_X = nullptr;  // features of the current residual (K x F)
    float *d_Hs = nullptr, *d_y = nullptr, *d_dY = nullptr;  // hidden (+ its gradient), output, output gradient
    double *d_zt = nullptr, *d_w = nullptr;  // preconditioner output z and S z during training
    double* d_lpart = nullptr;               // [5][G] partial sums of the training losses
    double* d_R = nullptr;                   // stored training residuals (ring order, r.P r = 1)
    size_t cap = 0, count = 0;
    int adam_step = 0;
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
    cudaError_t e = launch_ipdg_apply(s->args, false, x, y, c->stream);
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

// the additive-Schwarz forms: one tied weight matrix W (H x 4 Np)
bool schwarz_form(int form) { return form == DG_LPC_SCHWARZ || form == DG_LPC_SCHWARZ_MLP; }

// runs PCG iterations on S e = r (vectors in v) until S->done or `limit`
// iterations; returns the iterations taken and the stop code
void lpc_descr(dg_ctx* c, LpcNet& net, LpcFeatArgs& fa) {
    IpdgState* s = c->ipdg;
    net.F = s->F;
    net.H = s->H;
    net.linear = s->lpc_linear;
    net.Np = c->Np;
    net.W1 = s->d_W1b;
    net.W2 = s->d_W2b;
    net.perm = s->d_perm;
    if (schwarz_form(s->lpc_form)) {
        net.sw = &s->sw;
        net.U = s->d_U;
    }
    fa.K = c->K;
    fa.Np = c->Np;
    fa.linear = s->lpc_linear;
    fa.zb = s->d_zb;
    fa.conn = c->d_conn;
    fa.geo = c->d_geo;
    fa.perm = s->d_perm;
}

// PCG iterations on S x = b (vectors in v, r = b - S x given) until S->done
// or `limit` iterations.  Every `refresh` host checks (0: never) the
// recurrence residual is replaced by the true FP64 residual b - S x (residual
// replacement: the search direction is kept), and a convergence claim of the
// recurrence is confirmed against the true residual; a claim that fails
// restarts the recurrence from the true residual.
int run_cg(dg_ctx* c, const PcgVecs& v, bool fp32, double tol2, int limit, const double* b, int refresh, int* iters,
           int* stop) {
    IpdgState* s = c->ipdg;
    const size_t n = (size_t)c->K * c->Np;
    PcgScalars h;
    memset(&h, 0, sizeof(h));
    h.tol2 = tol2;
    LpcNet net;
    LpcFeatArgs fa;
    const LpcNet* pnet = nullptr;
    const LpcFeatArgs* pfa = nullptr;
    if (v.zb) {
        lpc_descr(c, net, fa);
        pnet = &net;
        pfa = &fa;
    }
    IP_CUDA(c, cudaMemcpyAsync(s->d_S, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
    IP_CUDA(c, launch_pcg_init(s->args, v, pnet, pfa, c->stream));
    const int CHECK = 16;
    int checks = 0;
    *stop = 0;
    *iters = 0;
    // learned mode: give up when the best residual has not halved over a window
    // (the caller then falls back to block Jacobi instead of running to maxit);
    // with a linear SPD learned form CG cannot break down and the residual norm
    // may plateau for long stretches, so the window is wider
    const int STALL = (schwarz_form(s->lpc_form) && !s->sw.flex) ? 2048 : 256;
    double best_rr = -1.0;
    int best_it = 0;
    // A batch of CHECK iterations is ~20 kernels per iteration; on small
    // operators each is a few microseconds of device work, less than the
    // host's cost of launching it.  From the second full batch on, a batch is
    // one CUDA graph (captured once per solve, parity of the first iteration
    // as its key; the kernels read all vectors and scalars from device memory,
    // so the graph stays valid while this solve's buffers do).  If capture is
    // not possible on this stream the batches are launched directly.
    struct GraphGuard {
        cudaGraphExec_t g = nullptr;
        ~GraphGuard() {
            if (g) cudaGraphExecDestroy(g);
        }
    } graph;
    int gparity = -1;
    bool use_graph = true;
    auto launch_batch = [&](int it0, int count) -> cudaError_t {
        if (use_graph && count == CHECK && checks > 0) {
            const int par = it0 & 1;
            if (graph.g && par != gparity) {
                cudaGraphExecDestroy(graph.g);
                graph.g = nullptr;
            }
            if (!graph.g) {
                cudaGraph_t g = nullptr;
                cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed);
                if (e == cudaSuccess) {
                    for (int j = 0; j < CHECK && e == cudaSuccess; j++)
                        e = launch_pcg_iteration(s->args, v, fp32, (it0 + j) & 1, pnet, pfa, c->stream);
                    const cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
                    if (e == cudaSuccess) e = e2;
                }
                if (e == cudaSuccess) e = cudaGraphInstantiate(&graph.g, g, 0);
                if (g) cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    (void)cudaGetLastError();
                    graph.g = nullptr;
                    use_graph = false;
                } else {
                    gparity = par;
                }
            }
            if (graph.g) return cudaGraphLaunch(graph.g, c->stream);
        }
        for (int j = 0; j < count; j++) {
            const cudaError_t e = launch_pcg_iteration(s->args, v, fp32, (it0 + j) & 1, pnet, pfa, c->stream);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    };
    while (h.it < limit) {
        const int batch = std::min(CHECK, limit - h.it);
        IP_CUDA(c, launch_batch(h.it, batch));
        IP_CUDA(c, cudaMemcpyAsync(&h, s->d_S, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
        IP_CUDA(c, cudaStreamSynchronize(c->stream));
        checks++;
        if (h.done == 2) break;
        if (v.zb && !v.mg && h.done == 0) {
            if (best_rr < 0 || h.rr < 0.5 * best_rr) {
                best_rr = h.rr;
                best_it = h.it;
            } else if (h.it - best_it >= STALL) {
                *iters = h.it;
                *stop = 3;
                return DG_OK;
            }
        }
        const bool claim = h.done == 1;
        const bool periodic = refresh > 0 && checks % refresh == 0;
        if (!b || (!claim && !periodic)) {
            if (claim) break;
            continue;
        }
        // true residual into r (Ap is scratch here: the next iteration recomputes it)
        int rc = apply64(c, v.x, v.Ap);
        if (rc) return rc;
        IP_CUDA(c, launch_xmy(v.r, b, v.Ap, n, c->stream));
        if (claim) {
            double rr = 0;
            rc = dot_host(c, v.r, v.r, &rr);
            if (rc) return rc;
            if (rr <= tol2) break;
            // the recurrence drifted: restart from the true residual (p = z)
            h.done = 0;
            const int zero = 0;
            const double zbeta = 0.0;
            IP_CUDA(c, cudaMemcpyAsync(&s->d_S->done, &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream));
            IP_CUDA(c, cudaMemcpyAsync(&s->d_S->beta, &zbeta, sizeof(double), cudaMemcpyHostToDevice, c->stream));
        }
        IP_CUDA(c, launch_pcg_refresh(s->args, v, pnet, pfa, c->stream));
    }
    *iters = h.it;
    *stop = h.done;
    return DG_OK;
}

}  // namespace

// node permutation (ring order) that rotates a neighbour's face fn onto face 0
std::vector<int> rotation_perms(const dgb::RefOps& o) {
    const int Np = o.Np;
    std::vector<int> perm(3 * Np, -1);
    auto bary = [&](int p, double* l) {
        const double r = o.r[o.ring[p]], t = o.s[o.ring[p]];
        l[0] = -(r + t) / 2;
        l[1] = (1 + r) / 2;
        l[2] = (1 + t) / 2;
    };
    for (int fn = 0; fn < 3; fn++)
        for (int i = 0; i < Np; i++) {
            double mu[3], want[3];
            bary(i, mu);
            for (int m = 0; m < 3; m++) want[(fn + m) % 3] = mu[m];
            for (int j = 0; j < Np; j++) {
                double l[3];
                bary(j, l);
                if (std::fabs(l[0] - want[0]) + std::fabs(l[1] - want[1]) + std::fabs(l[2] - want[2]) < 1e-9) {
                    perm[fn * Np + i] = j;
                    break;
                }
            }
        }
    return perm;
}

template <int N>
static void build_lane_tab(const dg_ctx* c, const std::vector<double>& DrfT, const std::vector<double>& DsfT,
                           const std::vector<double>& Srr, const std::vector<double>& Srs2,
                           const std::vector<double>& Sss, const std::vector<double>& Mr,
                           const std::vector<double>& mrow, std::vector<unsigned char>& blob) {
    using L = IpLaneTab<N>;
    blob.assign(sizeof(L), 0);
    L& t = *reinterpret_cast<L*>(blob.data());
    const dgb::RefOps& o = c->ops;
    for (int p = 0; p < L::Np; p++) {
        for (int fg = 0; fg < L::NF; fg++) {
            t.DrfT[p][fg] = (float)DrfT[(size_t)p * L::NF + fg];
            t.DsfT[p][fg] = (float)DsfT[(size_t)p * L::NF + fg];
        }
        for (int q = 0; q < L::Np; q++) {
            t.Srr[p][q] = (float)Srr[(size_t)p * L::Np + q];
            t.Srs2[p][q] = (float)Srs2[(size_t)p * L::Np + q];
            t.Sss[p][q] = (float)Sss[(size_t)p * L::Np + q];
            t.Mr[p][q] = (float)Mr[(size_t)p * L::Np + q];
        }
        t.mrow[p] = (float)mrow[p];
    }
    for (int g = 0; g < L::Nfq; g++) {
        t.fw[g] = (float)o.fw[g];
        for (int j = 0; j < L::Nfp; j++) t.If[g][j] = (float)o.If[(size_t)g * L::Nfp + j];
    }
}

void ipdg_teardown(dg_ctx* c) {
    if (!c->ipdg) return;
    for (void* p : c->ipdg->allocs) cudaFree(p);
    for (void* p : c->ipdg->mg_allocs) cudaFree(p);
    delete c->ipdg;
    c->ipdg = nullptr;
}

extern "C" {

// block-Jacobi inverse blocks of the current operator
static int build_blocks(dg_ctx* c) {
    IpdgState* s = c->ipdg;
    const IpdgArgs& a = s->args;
    IP_CUDA(c, cudaMemsetAsync(s->d_status, 0, sizeof(int), c->stream));
    IP_CUDA(c, launch_ipdg_diag(a, s->d_blocks, c->stream));
    IP_CUDA(c, launch_invert_blocks(s->d_blocks, nullptr, a.K, a.Np, s->d_status, c->stream));
    IP_CUDA(c, launch_group_blocks(a, s->d_blocks, s->d_P64, s->d_P32, c->stream));
    int st = 0;
    IP_CUDA(c, cudaMemcpyAsync(&st, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    IP_CUDA(c, cudaStreamSynchronize(c->stream));
    if (st) return ifail(c, DG_ERR_NONFINITE, "singular diagonal block in the SIPG operator");
    return DG_OK;
}

// (re)builds the multilevel preconditioner of the current operator
static int mg_setup(dg_ctx* c) {
    IpdgState* s = c->ipdg;
    for (void* p : s->mg_allocs) cudaFree(p);
    s->mg_allocs.clear();
    s->mg_ready = false;
    if (c->etov_host.empty()) {
        s->mg_err = "the mesh descriptor has no vertex ids (EToV)";
        return ifail(c, DG_ERR_UNSUPPORTED, s->mg_err);
    }
    MgBuild b;
    std::string e = mg_build(c->K, c->N, c->Np, c->etov_host.data(), c->geo_host.data(), c->conn_host.data(),
                             s->fc_host, s->btype, s->args.mass_coef, c->ops, b);
    if (!e.empty()) {
        s->mg_err = "multilevel preconditioner: " + e;
        return ifail(c, DG_ERR_UNSUPPORTED, s->mg_err);
    }
    int rc = 0;
    auto up = [&](auto** dst, const auto& h) {
        using T = typename std::remove_reference<decltype(h)>::type::value_type;
        T* p = nullptr;
        if (cudaMalloc((void**)&p, std::max<size_t>(h.size(), 1) * sizeof(T)) != cudaSuccess) { rc = 1; return; }
        s->mg_allocs.push_back(p);
        if (!h.empty() && cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) rc = 1;
        *dst = p;
    };
    auto work = [&](double** dst, int n) {
        double* p = nullptr;
        if (cudaMalloc((void**)&p, std::max(n, 1) * sizeof(double)) != cudaSuccess) { rc = 1; return; }
        s->mg_allocs.push_back(p);
        *dst = p;
    };
    MgLevels& m = s->mg;
    m = MgLevels();
    m.nl = (int)b.levels.size();
    m.K = c->K;
    m.Np = c->Np;
    up((int**)&m.etov, c->etov_host);
    up((double**)&m.lam, b.lam);
    up((int**)&m.vptr, b.vptr);
    up((int**)&m.vinc, b.vinc);
    up((double**)&m.Cinv, b.Cinv);
    for (int l = 0; l < m.nl; l++) {
        const MgBuild::Level& L = b.levels[l];
        MgLevel& d = m.lv[l];
        d.n = L.n;
        up((int**)&d.rowptr, L.rowptr);
        up((int**)&d.col, L.col);
        up((double**)&d.val, L.val);
        up((double**)&d.dinv, L.dinv);
        if (l + 1 < m.nl) {
            up((int**)&d.agg, L.agg);
            up((int**)&d.cptr, L.cptr);
            up((int**)&d.cmem, L.cmem);
        }
        work(&d.r, L.n);
        work(&d.x, L.n);
        work(&d.t, L.n);
    }
    if (!s->d_zb) rc |= ialloc(c, s, &s->d_zb, (size_t)c->K * c->Np);
    if (rc) return ifail(c, DG_ERR_NOMEM, "multilevel preconditioner: device allocation failed");
    s->mg_ready = true;
    return DG_OK;
}

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
    const int NF = 3 * Nfq;
    std::vector<double> DrfT((size_t)Np * NF), DsfT((size_t)Np * NF);
    for (int fg = 0; fg < NF; fg++)
        for (int p = 0; p < Np; p++) {
            DrfT[(size_t)p * NF + fg] = Drf[(size_t)fg * Np + p];
            DsfT[(size_t)p * NF + fg] = Dsf[(size_t)fg * Np + p];
        }
    std::vector<double> J(K), vc((size_t)K * 3), fc((size_t)K * 3 * kFaceCoef);
    const double tau0 = tau_coef * (c->N + 1) * (c->N + 1);
    for (int k = 0; k < K; k++) {
        const double* g = &c->geo_host[4 * (size_t)k];
        const double rx = g[0], sx = g[1], ry = g[2], sy = g[3];
        J[k] = 1.0 / (rx * sy - sx * ry);
        vc[3 * (size_t)k] = J[k] * (rx * rx + ry * ry);
        vc[3 * (size_t)k + 1] = J[k] * (rx * sx + ry * sy);
        vc[3 * (size_t)k + 2] = J[k] * (sx * sx + sy * sy);
        for (int f = 0; f < 3; f++) {
            double nx, ny, fsc;
            face_normal(f, rx, sx, ry, sy, nx, ny, fsc);
            double* out = &fc[((size_t)k * 3 + f) * kFaceCoef];
            out[0] = nx * rx + ny * ry;
            out[1] = nx * sx + ny * sy;
            out[2] = out[3] = 0.0;
            double fmx = fsc;
            const int cn = c->conn_host[(size_t)k * 3 + f];
            if (cn >= 0) {
                const int nb = cn >> 3, fn = cn & 3;
                const double* gn = &c->geo_host[4 * (size_t)nb];
                double nx2, ny2, fsc2;
                face_normal(fn, gn[0], gn[1], gn[2], gn[3], nx2, ny2, fsc2);
                fmx = std::max(fsc, fsc2);
                out[2] = nx * gn[0] + ny * gn[2];
                out[3] = nx * gn[1] + ny * gn[3];
            }
            out[4] = 0.5 * tau0 * fmx;
            out[5] = fsc * J[k];
        }
    }
    std::vector<double> Ifh(o.If.begin(), o.If.end());
    // reference mass matrix in ring order and its row sums
    std::vector<double> Mr((size_t)Np * Np), mrow(Np, 0.0);
    for (int i = 0; i < Np; i++)
        for (int j = 0; j < Np; j++) {
            Mr[(size_t)i * Np + j] = o.Mref[(size_t)o.ring[i] * Np + o.ring[j]];
            mrow[i] += Mr[(size_t)i * Np + j];
        }
    s->fc_host = fc;
    s->btype.assign(c->nb, 0);
    switch (c->N) {
        case 1: build_lane_tab<1>(c, DrfT, DsfT, Srr, Srs2, Sss, Mr, mrow, s->lane_tab); break;
        case 2: build_lane_tab<2>(c, DrfT, DsfT, Srr, Srs2, Sss, Mr, mrow, s->lane_tab); break;
        case 3: build_lane_tab<3>(c, DrfT, DsfT, Srr, Srs2, Sss, Mr, mrow, s->lane_tab); break;
        case 4: build_lane_tab<4>(c, DrfT, DsfT, Srr, Srs2, Sss, Mr, mrow, s->lane_tab); break;
        case 5: build_lane_tab<5>(c, DrfT, DsfT, Srr, Srs2, Sss, Mr, mrow, s->lane_tab); break;
        default: s->lane_tab.clear(); break;
    }
    auto f32 = [](const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); };
    int rc = 0;
    IpdgOps<double>& o64 = s->o64h;
    IpdgOps<float>& o32 = s->o32h;
    rc |= iupload(c, s, &s->d_J, J);
    rc |= iupload(c, s, (double**)&o64.Srr, Srr);
    rc |= iupload(c, s, (double**)&o64.Srs2, Srs2);
    rc |= iupload(c, s, (double**)&o64.Sss, Sss);
    rc |= iupload(c, s, (double**)&o64.Drf, Drf);
    rc |= iupload(c, s, (double**)&o64.Dsf, Dsf);
    rc |= iupload(c, s, (double**)&o64.DrfT, DrfT);
    rc |= iupload(c, s, (double**)&o64.DsfT, DsfT);
    rc |= iupload(c, s, (double**)&o64.If, Ifh);
    rc |= iupload(c, s, (double**)&o64.fw, o.fw);
    rc |= iupload(c, s, (double**)&o64.fc, fc);
    rc |= iupload(c, s, (double**)&o64.vc, vc);
    rc |= iupload(c, s, (double**)&o64.Mr, Mr);
    rc |= iupload(c, s, (double**)&o64.mrow, mrow);
    rc |= iupload(c, s, (float**)&o32.Mr, f32(Mr));
    rc |= iupload(c, s, (float**)&o32.mrow, f32(mrow));
    rc |= iupload(c, s, (float**)&o32.Srr, f32(Srr));
    rc |= iupload(c, s, (float**)&o32.Srs2, f32(Srs2));
    rc |= iupload(c, s, (float**)&o32.Sss, f32(Sss));
    rc |= iupload(c, s, (float**)&o32.Drf, f32(Drf));
    rc |= iupload(c, s, (float**)&o32.Dsf, f32(Dsf));
    rc |= iupload(c, s, (float**)&o32.DrfT, f32(DrfT));
    rc |= iupload(c, s, (float**)&o32.DsfT, f32(DsfT));
    rc |= iupload(c, s, (float**)&o32.If, f32(Ifh));
    rc |= iupload(c, s, (float**)&o32.fw, f32(o.fw));
    rc |= iupload(c, s, (float**)&o32.fc, f32(fc));
    rc |= iupload(c, s, (float**)&o32.vc, f32(vc));
    const size_t n = (size_t)K * Np;
    rc |= ialloc(c, s, &s->d_blocks, n * Np);
    const size_t ng = grouped_blocks_size(K, Np);
    rc |= ialloc(c, s, &s->d_P64, ng);
    rc |= ialloc(c, s, &s->d_P32, ng);
    rc |= ialloc(c, s, &s->d_b, n);
    rc |= ialloc(c, s, &s->d_x, n);
    rc |= ialloc(c, s, &s->d_r, n);
    rc |= ialloc(c, s, &s->d_z, n);
    rc |= ialloc(c, s, &s->d_p, n);
    rc |= ialloc(c, s, &s->d_p2, n);
    rc |= ialloc(c, s, &s->d_dz, n);
    rc |= ialloc(c, s, &s->d_r32, n);
    rc |= ialloc(c, s, &s->d_dp, n);
    rc |= ialloc(c, s, &s->d_dp2, n);
    if (!s->lane_tab.empty()) {
        rc |= ialloc(c, s, &s->d_lane_ftr, (size_t)K * 3 * lane_face_rec(c->N));
        rc |= ialloc(c, s, &s->d_lane_p0, (size_t)K);
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    s->sms = sms > 0 ? sms : 1;
    s->nmax = pcg_max_grid(K, c->N, s->sms);
    rc |= ialloc(c, s, &s->d_ppart, (size_t)3 * s->nmax);
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
    a.sms = s->sms;
    a.mass_coef = 0.0;
    a.o64 = o64;
    a.o32 = o32;
    a.lane_tab = s->lane_tab.empty() ? nullptr : s->lane_tab.data();
    a.lane_ftr = s->d_lane_ftr;
    a.lane_p0 = s->d_lane_p0;
    rc = build_blocks(c);
    if (rc) return rc;
    s->ready = true;
    return DG_OK;
}

int dg_ipdg_set_mass(dg_ctx* c, double alpha) {
    if (!c || !(alpha >= 0)) return DG_ERR_ARG;
    if (!c->ipdg || !c->ipdg->ready) return ifail(c, DG_ERR_ARG, "dg_ipdg_setup not called");
    c->ipdg->args.mass_coef = alpha;
    c->ipdg->mg_ready = false;
    return build_blocks(c);
}

int dg_ipdg_set_boundary_types(dg_ctx* c, const int* btype) {
    if (!c || (!btype && c->nb > 0)) return DG_ERR_ARG;
    if (!c->ipdg || !c->ipdg->ready) return ifail(c, DG_ERR_ARG, "dg_ipdg_setup not called");
    IpdgState* s = c->ipdg;
    for (int i = 0; i < c->nb; i++)
        if (btype[i] < 0 || btype[i] > 2) return ifail(c, DG_ERR_ARG, "boundary type must be 0, 1 or 2");
    std::vector<double> fc = s->fc_host;
    for (int k = 0; k < c->K; k++)
        for (int f = 0; f < 3; f++) {
            const int cn = c->conn_host[(size_t)k * 3 + f];
            if (cn >= 0) continue;
            s->btype[-1 - cn] = btype[-1 - cn];
            // no operator terms on faces without a fixed value: their face weight is zero
            if (btype[-1 - cn] != 0) fc[((size_t)k * 3 + f) * kFaceCoef + 5] = 0.0;
        }
    const size_t nfc = fc.size();
    std::vector<float> fc32(fc.begin(), fc.end());
    IP_CUDA(c, cudaMemcpyAsync((void*)s->o64h.fc, fc.data(), nfc * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    IP_CUDA(c, cudaMemcpyAsync((void*)s->o32h.fc, fc32.data(), nfc * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    IP_CUDA(c, cudaStreamSynchronize(c->stream));
    s->mg_ready = false;
    return build_blocks(c);
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

int dg_ipdg_apply_device(dg_ctx* c, const double* x_dev, double* y_dev) {
    if (!c || !x_dev || !y_dev) return DG_ERR_ARG;
    if (!c->ipdg || !c->ipdg->ready) return ifail(c, DG_ERR_ARG, "dg_ipdg_setup not called");
    IpdgState* s = c->ipdg;
    IP_CUDA(c, launch_permute(x_dev, s->d_p, c->d_ring, c->K, c->Np, true, c->stream));
    int rc = apply64(c, s->d_p, s->d_Ap);
    if (rc) return rc;
    IP_CUDA(c, launch_permute(s->d_Ap, y_dev, c->d_ring, c->K, c->Np, false, c->stream));
    return DG_OK;
}

// The PCG solve behind dg_pcg_solve (host vectors) and dg_pcg_solve_device
// (device vectors): the two differ only in the direction of their copies.
static int pcg_solve_impl(dg_ctx* c, const double* b_host, double* x_host, double rtol, int maxit, int pc,
                          int precision, dg_solve_stats* stats, bool dev) {
    if (!c || !b_host || !x_host || !(rtol > 0) || maxit < 1) return DG_ERR_ARG;
    const cudaMemcpyKind kin = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const cudaMemcpyKind kout = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (!c->ipdg || !c->ipdg->ready) return ifail(c, DG_ERR_ARG, "dg_ipdg_setup not called");
    if (pc != DG_PC_BLOCK_JACOBI && pc != DG_PC_LEARNED && pc != DG_PC_LEARNED_ONLY && pc != DG_PC_MULTILEVEL &&
        pc != DG_PC_LEARNED_MULTILEVEL)
        return ifail(c, DG_ERR_ARG, "unknown preconditioner");
    const bool learned = pc == DG_PC_LEARNED || pc == DG_PC_LEARNED_ONLY || pc == DG_PC_LEARNED_MULTILEVEL;
    const bool mgm = pc == DG_PC_MULTILEVEL || pc == DG_PC_LEARNED_MULTILEVEL;
    if (learned && !c->ipdg->lpc_ready) return ifail(c, DG_ERR_ARG, "dg_lpc_setup not called");
    if (pc == DG_PC_LEARNED_MULTILEVEL && c->ipdg->lpc_form != DG_LPC_SCHWARZ)
        return ifail(c, DG_ERR_ARG, "learned + multilevel needs the linear learned Schwarz form");
    if (mgm && !c->ipdg->mg_ready) {
        const int rcm = mg_setup(c);
        if (rcm) return rcm;
    }
    if (precision != DG_PREC_FP64 && precision != DG_PREC_SPLIT) return ifail(c, DG_ERR_ARG, "unknown precision");
    IpdgState* s = c->ipdg;
    const size_t n = (size_t)c->K * c->Np;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    IP_CUDA(c, cudaMemcpyAsync(s->d_z, b_host, n * sizeof(double), kin, c->stream));
    IP_CUDA(c, launch_permute(s->d_z, s->d_b, c->d_ring, c->K, c->Np, true, c->stream));
    IP_CUDA(c, cudaMemcpyAsync(s->d_z, x_host, n * sizeof(double), kin, c->stream));
    IP_CUDA(c, launch_permute(s->d_z, s->d_x, c->d_ring, c->K, c->Np, true, c->stream));
    cudaEventRecord(e0, c->stream);
    double bb = 0;
    int rc = dot_host(c, s->d_b, s->d_b, &bb);
    if (rc) return rc;
    PcgVecs v{};
    v.r = s->d_r;
    v.z = s->d_z;
    v.p[0] = s->d_p;
    v.p[1] = s->d_p2;
    v.Ap = s->d_Ap;
    v.part = s->d_ppart;
    v.nmax = s->nmax;
    v.P32 = s->d_P32;
    v.P64 = nullptr;
    v.zb = (learned || mgm) ? s->d_zb : nullptr;
    v.mg = mgm ? &s->mg : nullptr;
    if (pc == DG_PC_LEARNED_MULTILEVEL) {
        if (!s->d_zl && ialloc(c, s, &s->d_zl, n)) return ifail(c, DG_ERR_NOMEM, "device allocation failed");
        v.zl = s->d_zl;
    }
    v.S = s->d_S;
    const bool mirrors = precision == DG_PREC_SPLIT;  // the FP32 apply stages from FP32 offset mirrors
    v.dz = mirrors ? s->d_dz : nullptr;
    v.dp[0] = mirrors ? s->d_dp : nullptr;
    v.dp[1] = mirrors ? s->d_dp2 : nullptr;
    v.r32 = (learned && schwarz_form(s->lpc_form)) ? s->d_r32 : nullptr;
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
        if (!v.zb || mgm) v.P64 = s->d_P64;  // FP64 preconditioner: an inexact one stalls CG at high condition numbers
        rc = run_cg(c, v, false, rtol * rtol * bb, maxit, s->d_b, 0, &total_it, &stop);
        if (rc) return rc;
    } else {
        // FP32-arithmetic operator inside CG with FP64 vectors and recurrences;
        // the recurrence residual is replaced by the true FP64 residual every
        // 64 iterations
        rc = apply64(c, s->d_x, s->d_Ap);
        if (rc) return rc;
        IP_CUDA(c, launch_xmy(s->d_r, s->d_b, s->d_Ap, n, c->stream));
        v.x = s->d_x;
        rc = run_cg(c, v, true, rtol * rtol * bb, maxit, s->d_b, 4, &total_it, &stop);
        if (rc) return rc;
    }
    // true FP64 residual
    rc = apply64(c, s->d_x, s->d_Ap);
    if (rc) return rc;
    IP_CUDA(c, launch_xmy(s->d_r, s->d_b, s->d_Ap, n, c->stream));
    double rr = 0;
    rc = dot_host(c, s->d_r, s->d_r, &rr);
    if (rc) return rc;
    cudaEventRecord(e1, c->stream);
    rel = bb > 0 ? std::sqrt(rr / bb) : 0.0;
    if (learned && s->d_tcstatus) {
        int tst = 0;
        IP_CUDA(c, cudaMemcpyAsync(&tst, s->d_tcstatus, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        IP_CUDA(c, cudaStreamSynchronize(c->stream));
        if (tst) {
            cudaMemsetAsync(s->d_tcstatus, 0, sizeof(int), c->stream);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return ifail(c, DG_ERR_TIMEOUT, "learned preconditioner: tensor-core completion wait timed out");
        }
    }
    if (pc == DG_PC_LEARNED && (!(rel == rel) || stop >= 2 || rel > rtol)) {
        // block-Jacobi PCG is the fallback: solve again from the caller's x0;
        // the reported time includes the learned attempt
        IP_CUDA(c, cudaStreamSynchronize(c->stream));
        float ms_learned = 0;
        cudaEventElapsedTime(&ms_learned, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        int rc2 = pcg_solve_impl(c, b_host, x_host, rtol, maxit, DG_PC_BLOCK_JACOBI, precision, stats, dev);
        if (stats) {
            stats->iterations = -stats->iterations;  // negative: the learned solve fell back
            stats->ms += ms_learned;
        }
        return rc2;
    }
    IP_CUDA(c, launch_permute(s->d_x, s->d_z, c->d_ring, c->K, c->Np, false, c->stream));
    IP_CUDA(c, cudaMemcpyAsync(x_host, s->d_z, n * sizeof(double), kout, c->stream));
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

int dg_pcg_solve(dg_ctx* c, const double* b_host, double* x_host, double rtol, int maxit, int pc, int precision,
                 dg_solve_stats* stats) {
    return pcg_solve_impl(c, b_host, x_host, rtol, maxit, pc, precision, stats, false);
}

int dg_pcg_solve_device(dg_ctx* c, const double* b_dev, double* x_dev, double rtol, int maxit, int pc, int precision,
                        dg_solve_stats* stats) {
    return pcg_solve_impl(c, b_dev, x_dev, rtol, maxit, pc, precision, stats, true);
}

}  // extern "C"

// PCG on ring-order device vectors (x holds the initial guess and receives
// the solution); used by the incompressible step.  precision DG_PREC_FP64:
// FP64 operator and blocks; DG_PREC_SPLIT: the mixed-precision iteration of
// dg_pcg_solve (FP32 operator on FP64 offsets, FP32 blocks, FP64 vectors and
// recurrences, true-residual replacement), ending on the true FP64 residual
int ipdg_solve_device(dg_ctx* c, const double* b_dev, double* x_dev, double rtol, int maxit, int* iters,
                      double* rel_out, int pc, int precision) {
    if (precision != DG_PREC_FP64 && precision != DG_PREC_SPLIT) return ifail(c, DG_ERR_ARG, "unknown precision");
    if (!c->ipdg || !c->ipdg->ready) return ifail(c, DG_ERR_ARG, "dg_ipdg_setup not called");
    IpdgState* s = c->ipdg;
    const bool mgm = pc == DG_PC_MULTILEVEL;
    if (mgm && !s->mg_ready) {
        const int rcm = mg_setup(c);
        if (rcm) return rcm;
    }
    const size_t n = (size_t)c->K * c->Np;
    IP_CUDA(c, cudaMemcpyAsync(s->d_b, b_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    IP_CUDA(c, cudaMemcpyAsync(s->d_x, x_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    double bb = 0;
    int rc = dot_host(c, s->d_b, s->d_b, &bb);
    if (rc) return rc;
    int total_it = 0, stop = 0;
    double rr = 0;
    if (bb == 0.0) {
        IP_CUDA(c, cudaMemsetAsync(s->d_x, 0, n * sizeof(double), c->stream));
    } else {
        PcgVecs v{};
        v.r = s->d_r;
        v.z = s->d_z;
        v.p[0] = s->d_p;
        v.p[1] = s->d_p2;
        v.Ap = s->d_Ap;
        v.part = s->d_ppart;
        v.nmax = s->nmax;
        const bool mixed = precision == DG_PREC_SPLIT;
        v.P32 = s->d_P32;
        v.P64 = mixed ? nullptr : s->d_P64;
        v.zb = mgm ? s->d_zb : nullptr;
        v.mg = mgm ? &s->mg : nullptr;
        v.S = s->d_S;
        v.dz = mixed ? s->d_dz : nullptr;  // the FP32 apply stages from FP32 offset mirrors
        v.dp[0] = mixed ? s->d_dp : nullptr;
        v.dp[1] = mixed ? s->d_dp2 : nullptr;
        v.r32 = nullptr;
        v.x = s->d_x;
        rc = apply64(c, s->d_x, s->d_Ap);
        if (rc) return rc;
        IP_CUDA(c, launch_xmy(s->d_r, s->d_b, s->d_Ap, n, c->stream));
        rc = run_cg(c, v, mixed, rtol * rtol * bb, maxit, s->d_b, mixed ? 4 : 0, &total_it, &stop);
        if (rc) return rc;
        rc = apply64(c, s->d_x, s->d_Ap);
        if (rc) return rc;
        IP_CUDA(c, launch_xmy(s->d_r, s->d_b, s->d_Ap, n, c->stream));
        rc = dot_host(c, s->d_r, s->d_r, &rr);
        if (rc) return rc;
    }
    IP_CUDA(c, cudaMemcpyAsync(x_dev, s->d_x, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    const double rel = bb > 0 ? std::sqrt(rr / bb) : 0.0;
    if (iters) *iters = total_it;
    if (rel_out) *rel_out = rel;
    if (!(rel == rel) || stop == 2) return ifail(c, DG_ERR_NONFINITE, "PCG breakdown or non-finite residual");
    if (rel > rtol) return ifail(c, DG_ERR_NOT_CONVERGED, "PCG reached the iteration limit");
    return DG_OK;
}

const dgk::IpdgArgs* ipdg_args(dg_ctx* c) { return (c->ipdg && c->ipdg->ready) ? &c->ipdg->args : nullptr; }
const std::vector<int>* ipdg_btypes(dg_ctx* c) { return c->ipdg ? &c->ipdg->btype : nullptr; }
const std::vector<double>* ipdg_face_coefs(dg_ctx* c) { return c->ipdg ? &c->ipdg->fc_host : nullptr; }

// ---------------------------------------------------------------------------
// learned preconditioner
//
// Training objective (self-supervised, over whole residual vectors r of the
// method's own PCG iterates): the energy loss of one preconditioned step
// with the optimal step length,
//     L(r) = -(r.z)^2 / (z.S z),   z = M(r) = P r + s W2 relu(W1 x),
// which is -1/2 of the largest decrease of the S-norm of the error along z
// (-(r.P r)^2 / (P r.S P r) for block Jacobi alone).  dL/dz is proportional
// to (a/b) S z - r (a = r.z, b = z.S z): one SIPG apply per step, then the
// hand-written backward kernels.  Residuals are scaled to r.P r = 1 when
// they are stored, so every residual weighs the same.

namespace {

__global__ void f32_to_bf16_kernel(const float* in, __nv_bfloat16* out, long long n) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        out[t] = __float2bfloat16(in[t]);
}

__global__ void scale_kernel(double* x, const double* part, int G, size_t n) {
    __shared__ double s_f;
    if (threadIdx.x < 32) {
        double a = 0;
        for (int i = threadIdx.x; i < G; i += 32) a += part[i];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (threadIdx.x == 0) s_f = a > 0 ? rsqrt(a) : 0.0;
    }
    __syncthreads();
    const double f = s_f;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) x[t] *= f;
}

// forward pass of the learned preconditioner on the ring-order residual r:
// zb = P r, features, hidden layer, z = zb + s y (into s->d_zt), w = S z
// (FP32-arithmetic apply) and the partials of a = r.z, b = z.w
int lpc_forward_vec(dg_ctx* c, const double* r, bool with_bj_loss) {
    IpdgState* s = c->ipdg;
    const int K = c->K, Np = c->Np;
    const size_t n = (size_t)K * Np;
    LpcNet net;
    LpcFeatArgs fa;
    lpc_descr(c, net, fa);
    IP_CUDA(c, launch_bj(s->args, s->d_P32, r, s->d_zb, c->stream));
    if (with_bj_loss) {
        // the reference loss: block Jacobi, with the coarse-space correction when training under it
        const double* zref = s->d_zb;
        if (s->lpc_coarse) {
            IP_CUDA(c, launch_mg_correction(s->mg, r, s->d_zb, s->d_zt, nullptr, LPC_PCG_INIT, s->d_S, s->d_ppart,
                                            s->nmax, nullptr, c->stream));
            zref = s->d_zt;
        }
        IP_CUDA(c, launch_ipdg_apply(s->args, true, zref, s->d_w, c->stream));
        IP_CUDA(c, launch_dot(r, zref, n, s->d_lpart + 2 * s->G, s->G, c->stream));
        IP_CUDA(c, launch_dot(zref, s->d_w, n, s->d_lpart + 3 * s->G, s->G, c->stream));
    }
    if (schwarz_form(s->lpc_form)) {
        IP_CUDA(c, launch_schwarz_local(s->sw, r, nullptr, s->d_U, nullptr, c->stream));
        IP_CUDA(c, launch_schwarz_collect(s->sw, s->d_zb, s->d_U, nullptr, s->d_zt, nullptr, LPC_APPLY, nullptr,
                                          nullptr, c->stream));
        if (s->lpc_coarse)  // z = learned local stage + P V(P^T r), in place (the preconditioner it is trained for)
            IP_CUDA(c, launch_mg_correction(s->mg, r, s->d_zt, s->d_zt, nullptr, LPC_PCG_INIT, s->d_S, s->d_ppart,
                                            s->nmax, nullptr, c->stream));
    } else {
        IP_CUDA(c, launch_lpc_features(fa, s->d_X, s->d_sc, c->stream));
        IP_CUDA(c, launch_lpc_forward(net, s->d_X, nullptr, K, s->d_Hs, s->d_y, s->d_lpart + 4 * s->G, s->G,
                                      c->stream));
        IP_CUDA(c, launch_lpc_combine(s->d_zb, s->d_sc, s->d_y, K, Np, s->d_zt, c->stream));
    }
    IP_CUDA(c, launch_ipdg_apply(s->args, true, s->d_zt, s->d_w, c->stream));
    IP_CUDA(c, launch_dot(r, s->d_zt, n, s->d_lpart, s->G, c->stream));
    IP_CUDA(c, launch_dot(s->d_zt, s->d_w, n, s->d_lpart + s->G, s->G, c->stream));
    return DG_OK;
}

// gradients of L(r) into s->d_g1 / d_g2
int lpc_backward_vec(dg_ctx* c, const double* r) {
    IpdgState* s = c->ipdg;
    if (s->lpc_form == DG_LPC_SCHWARZ_MLP) {
        // dL/dW = (2a/b) sum_m h_m a_m^T + (D_m W a_m) x_m^T, x_m = G_m r, a_m = G_m g,
        // g = (a/b) S z - r: per-CTA partials on the tensor cores, then their sum
        const size_t n = (size_t)c->K * c->Np;
        IP_CUDA(c, launch_schwarz_outgrad(r, s->d_w, s->d_lpart, s->d_lpart + s->G, s->G, n, s->d_gvec, c->stream));
        IP_CUDA(c, launch_schwarz_mlp_wgrad(s->sw, r, s->d_gvec, s->d_wpart, s->d_tcstatus, c->stream));
        IP_CUDA(c, launch_schwarz_mlp_wreduce(s->d_wpart, schwarz_mlp_wgrad_ctas(s->sw), s->H, s->F, s->d_lpart,
                                              s->d_lpart + s->G, s->G, s->d_g1, c->stream));
        return DG_OK;
    }
    if (schwarz_form(s->lpc_form)) {
        // dL/dW = (2a/b) W (X^T A + A^T X), X = G r, A = G g, g = (a/b) S z - r
        const size_t n = (size_t)c->K * c->Np;
        IP_CUDA(c, launch_schwarz_outgrad(r, s->d_w, s->d_lpart, s->d_lpart + s->G, s->G, n, s->d_gvec, c->stream));
        IP_CUDA(c, launch_schwarz_gather_rows(s->sw, r, s->d_Xs, c->stream));
        IP_CUDA(c, launch_schwarz_gather_rows(s->sw, s->d_gvec, s->d_As, c->stream));
        IP_CUDA(c, launch_schwarz_cross(s->d_Xs, s->d_As, c->K, s->F, s->d_C, c->stream));
        IP_CUDA(c, launch_schwarz_wgrad(s->d_W1, s->d_C, s->H, s->F, s->d_lpart, s->d_lpart + s->G, s->G, s->d_g1,
                                        c->stream));
        return DG_OK;
    }
    LpcNet net;
    LpcFeatArgs fa;
    lpc_descr(c, net, fa);
    IP_CUDA(c, launch_lpc_energy_dy(r, s->d_w, s->d_sc, s->d_lpart, s->d_lpart + s->G, s->G, c->K, c->Np, s->d_dY,
                                    c->stream));
    IP_CUDA(c, launch_lpc_backward(net, s->d_X, s->d_Hs, s->d_dY, c->K, s->d_g1, s->d_g2, c->stream));
    return DG_OK;
}

// host value of a partial sum block
int lpc_sum(dg_ctx* c, const double* part, double* out) {
    IpdgState* s = c->ipdg;
    IP_CUDA(c, launch_reduce_to(part, s->G, s->d_scal, c->stream));
    IP_CUDA(c, cudaMemcpyAsync(out, s->d_scal, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    IP_CUDA(c, cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int lpc_losses(dg_ctx* c, double* loss, double* loss_bj) {
    IpdgState* s = c->ipdg;
    double a = 0, b = 0;
    int rc = lpc_sum(c, s->d_lpart, &a);
    if (!rc) rc = lpc_sum(c, s->d_lpart + s->G, &b);
    if (rc) return rc;
    if (loss) *loss = b > 0 ? -(a * a) / b : 0.0;
    if (loss_bj) {
        double a0 = 0, b0 = 0;
        rc = lpc_sum(c, s->d_lpart + 2 * s->G, &a0);
        if (!rc) rc = lpc_sum(c, s->d_lpart + 3 * s->G, &b0);
        if (rc) return rc;
        *loss_bj = b0 > 0 ? -(a0 * a0) / b0 : 0.0;
    }
    return DG_OK;
}

int lpc_adam_step(dg_ctx* c, double lr) {
    IpdgState* s = c->ipdg;
    const int n1 = s->H * s->F, n2 = schwarz_form(s->lpc_form) ? 0 : c->Np * s->H;
    s->adam_step++;
    IP_CUDA(c, launch_lpc_adam(s->d_W1, s->d_m1, s->d_v1, s->d_g1, s->d_W1b, n1, (float)lr, 0.9f, 0.999f, 1e-8f,
                               s->adam_step, 1.f, c->stream));
    if (n2 > 0)
        IP_CUDA(c, launch_lpc_adam(s->d_W2, s->d_m2, s->d_v2, s->d_g2, s->d_W2b, n2, (float)lr, 0.9f, 0.999f, 1e-8f,
                                   s->adam_step, 1.f, c->stream));
    return DG_OK;
}

// BF16 copies of the master weights (an Adam step with zero gradient and zero
// learning rate only converts)
int lpc_refresh_bf16(dg_ctx* c) {
    IpdgState* s = c->ipdg;
    const int n1 = s->H * s->F, n2 = schwarz_form(s->lpc_form) ? 0 : c->Np * s->H;
    IP_CUDA(c, cudaMemsetAsync(s->d_g1, 0, n1 * sizeof(float), c->stream));
    IP_CUDA(c, launch_lpc_adam(s->d_W1, s->d_m1, s->d_v1, s->d_g1, s->d_W1b, n1, 0.f, 0.9f, 0.999f, 1e-8f, 1, 1.f,
                               c->stream));
    if (n2 > 0) {
        IP_CUDA(c, cudaMemsetAsync(s->d_g2, 0, n2 * sizeof(float), c->stream));
        IP_CUDA(c, launch_lpc_adam(s->d_W2, s->d_m2, s->d_v2, s->d_g2, s->d_W2b, n2, 0.f, 0.9f, 0.999f, 1e-8f, 1,
                                   1.f, c->stream));
    }
    return DG_OK;
}

// host residual (reference order) -> ring order into dst
int lpc_upload_residual(dg_ctx* c, const double* r_host, double* dst) {
    IpdgState* s = c->ipdg;
    const size_t n = (size_t)c->K * c->Np;
    IP_CUDA(c, cudaMemcpyAsync(s->d_z, r_host, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    IP_CUDA(c, launch_permute(s->d_z, dst, c->d_ring, c->K, c->Np, true, c->stream));
    return DG_OK;
}

bool lpc_ok(dg_ctx* c) { return c && c->ipdg && c->ipdg->lpc_ready; }

}  // namespace

extern "C" {

int dg_lpc_setup(dg_ctx* c, int hidden, unsigned long long seed, int capacity, int form) {
    if (!c || hidden < 8 || hidden > 256 || capacity < 0) return DG_ERR_ARG;
    if (form != DG_LPC_RELU && form != DG_LPC_LINEAR && form != DG_LPC_SCHWARZ && form != DG_LPC_SCHWARZ_MLP)
        return DG_ERR_ARG;
    if (!c->ipdg || !c->ipdg->ready) return ifail(c, DG_ERR_ARG, "dg_ipdg_setup not called");
    IpdgState* s = c->ipdg;
    if (s->lpc_ready) return ifail(c, DG_ERR_ARG, "learned preconditioner already set up");
    const int Np = c->Np, K = c->K;
    const bool schwarz = schwarz_form(form), mlp = form == DG_LPC_SCHWARZ_MLP;
    if (Np > 36) return ifail(c, DG_ERR_UNSUPPORTED, "learned preconditioner supports N <= 7");
    if (form == DG_LPC_SCHWARZ && (Np > 28 || (hidden != 32 && hidden != 64)))
        return ifail(c, DG_ERR_UNSUPPORTED, "the Schwarz form supports N <= 6 and hidden width 32 or 64");
    if (mlp && (Np > 28 || Np < 3 || hidden != kSchwarzMlpH))
        return ifail(c, DG_ERR_UNSUPPORTED, "the two-layer Schwarz form supports N = 1..6 and hidden width 128");
    s->H = hidden;
    s->F = schwarz ? 4 * Np : 4 * Np + 4;
    s->lpc_form = form;
    s->lpc_linear = form == DG_LPC_LINEAR ? 1 : 0;
    const int n1 = s->H * s->F, n2 = schwarz ? 0 : Np * s->H;
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    std::vector<float> W1(n1), W2(n2);
    // Schwarz form: a small start keeps M close to block Jacobi
    for (auto& w : W1) w = nd(rng) * (schwarz ? 1e-3f : std::sqrt(2.0f / s->F));
    for (auto& w : W2) w = nd(rng) * 0.01f / std::sqrt((float)s->H);
    std::vector<int> perm = rotation_perms(c->ops);
    for (int v : perm)
        if (v < 0) return ifail(c, DG_ERR_ARG, "node set is not rotation symmetric");
    std::vector<int> iperm(perm.size());
    for (int f = 0; f < 3; f++)
        for (int i = 0; i < Np; i++) iperm[f * Np + perm[f * Np + i]] = i;
    const size_t n = (size_t)K * Np;
    int rc = 0;
    rc |= iupload(c, s, &s->d_W1, W1);
    rc |= iupload(c, s, &s->d_perm, perm);
    rc |= ialloc(c, s, &s->d_m1, n1);
    rc |= ialloc(c, s, &s->d_v1, n1);
    rc |= ialloc(c, s, &s->d_g1, n1);
    rc |= ialloc(c, s, &s->d_W1b, n1);
    rc |= ialloc(c, s, &s->d_zb, n);
    rc |= ialloc(c, s, &s->d_zt, n);
    rc |= ialloc(c, s, &s->d_w, n);
    rc |= ialloc(c, s, &s->d_lpart, (size_t)5 * s->G);
    if (schwarz) {
        rc |= iupload(c, s, &s->d_iperm, iperm);
        rc |= ialloc(c, s, &s->d_U, (size_t)K * s->F);
        rc |= ialloc(c, s, &s->d_gvec, n);
        if (mlp) {
            const int nctas = std::min((K + 127) / 128, s->sms);
            rc |= ialloc(c, s, &s->d_wpart, (size_t)nctas * s->H * s->F);
        } else {
            rc |= ialloc(c, s, &s->d_Xs, (size_t)K * s->F);
            rc |= ialloc(c, s, &s->d_As, (size_t)K * s->F);
            rc |= ialloc(c, s, &s->d_C, (size_t)s->F * s->F);
        }
    } else {
        rc |= iupload(c, s, &s->d_W2, W2);
        rc |= ialloc(c, s, &s->d_m2, n2);
        rc |= ialloc(c, s, &s->d_v2, n2);
        rc |= ialloc(c, s, &s->d_g2, n2);
        rc |= ialloc(c, s, &s->d_W2b, n2);
        rc |= ialloc(c, s, &s->d_sc, (size_t)K);
        rc |= ialloc(c, s, &s->d_X, (size_t)K * s->F);
        rc |= ialloc(c, s, &s->d_Hs, (size_t)2 * K * s->H);
        rc |= ialloc(c, s, &s->d_y, n);
        rc |= ialloc(c, s, &s->d_dY, n);
    }
    s->cap = (size_t)capacity;
    if (s->cap) rc |= ialloc(c, s, &s->d_R, s->cap * n);
    if (rc) return DG_ERR_NOMEM;
    s->sw.K = K;
    s->sw.Np = Np;
    s->sw.H = s->H;
    s->sw.sms = s->sms;
    s->sw.W = s->d_W1b;
    s->sw.conn = c->d_conn;
    s->sw.perm = s->d_perm;
    s->sw.iperm = s->d_iperm;
    s->sw.tc_status = nullptr;
    s->sw.mlp = mlp ? 1 : 0;
    s->sw.flex = mlp ? 1 : 0;  // M(r) is not linear: flexible beta in the PCG
    s->sw.slope = 0.f;
    if ((form == DG_LPC_SCHWARZ && s->H == 32) || mlp) {
        if (ialloc(c, s, &s->d_tcstatus, 1)) return DG_ERR_NOMEM;
        IP_CUDA(c, cudaMemsetAsync(s->d_tcstatus, 0, sizeof(int), c->stream));
        s->sw.tc_status = s->d_tcstatus;  // the tensor-core local stage
    }
    IP_CUDA(c, cudaMemsetAsync(s->d_m1, 0, n1 * sizeof(float), c->stream));
    IP_CUDA(c, cudaMemsetAsync(s->d_v1, 0, n1 * sizeof(float), c->stream));
    if (n2 > 0) {
        IP_CUDA(c, cudaMemsetAsync(s->d_m2, 0, n2 * sizeof(float), c->stream));
        IP_CUDA(c, cudaMemsetAsync(s->d_v2, 0, n2 * sizeof(float), c->stream));
    }
    rc = lpc_refresh_bf16(c);
    if (rc) return rc;
    IP_CUDA(c, cudaStreamSynchronize(c->stream));
    s->count = 0;
    s->adam_step = 0;
    s->lpc_ready = true;
    return DG_OK;
}

int dg_lpc_set_coarse(dg_ctx* c, int on) {
    if (!c) return DG_ERR_ARG;
    if (!lpc_ok(c)) return ifail(c, DG_ERR_ARG, "dg_lpc_setup not called");
    IpdgState* s = c->ipdg;
    if (on && s->lpc_form != DG_LPC_SCHWARZ)
        return ifail(c, DG_ERR_ARG, "training under the coarse space takes the linear Schwarz form");
    if (on && !s->mg_ready) {
        const int rc = mg_setup(c);
        if (rc) return rc;
    }
    s->lpc_coarse = on != 0;
    return DG_OK;
}

int dg_lpc_set_slope(dg_ctx* c, double slope) {
    if (!c || !(slope >= 0.0 && slope <= 1.0)) return DG_ERR_ARG;
    if (!lpc_ok(c)) return ifail(c, DG_ERR_ARG, "dg_lpc_setup not called");
    IpdgState* s = c->ipdg;
    if (s->lpc_form != DG_LPC_SCHWARZ_MLP) return ifail(c, DG_ERR_ARG, "the slope belongs to the two-layer Schwarz form");
    s->sw.slope = (float)slope;
    s->sw.flex = slope < 1.0 ? 1 : 0;  // slope 1: linear and symmetric, the standard beta applies
    return DG_OK;
}

int dg_lpc_add_residual(dg_ctx* c, const double* r_host) {
    if (!c || !r_host) return DG_ERR_ARG;
    if (!lpc_ok(c)) return ifail(c, DG_ERR_ARG, "dg_lpc_setup not called");
    IpdgState* s = c->ipdg;
    if (s->count >= s->cap) return ifail(c, DG_ERR_ARG, "training set capacity reached");
    const size_t n = (size_t)c->K * c->Np;
    double* dst = s->d_R + s->count * n;
    int rc = lpc_upload_residual(c, r_host, dst);
    if (rc) return rc;
    // scale to r.P r = 1
    IP_CUDA(c, launch_bj(s->args, s->d_P32, dst, s->d_zb, c->stream));
    IP_CUDA(c, launch_dot(dst, s->d_zb, n, s->d_lpart, s->G, c->stream));
    double rpr = 0;
    rc = lpc_sum(c, s->d_lpart, &rpr);
    if (rc) return rc;
    if (!(rpr > 0) || !std::isfinite(rpr)) return ifail(c, DG_ERR_ARG, "residual is zero or not finite");
    scale_kernel<<<608, 256, 0, c->stream>>>(dst, s->d_lpart, s->G, n);
    IP_CUDA(c, cudaGetLastError());
    IP_CUDA(c, cudaStreamSynchronize(c->stream));
    s->count++;
    return DG_OK;
}

int dg_lpc_train(dg_ctx* c, int epochs, double lr, unsigned long long seed, double* final_loss,
                 double* final_loss_bj) {
    if (!c || epochs < 1 || !(lr >= 0)) return DG_ERR_ARG;
    if (!lpc_ok(c)) return ifail(c, DG_ERR_ARG, "dg_lpc_setup not called");
    IpdgState* s = c->ipdg;
    if (s->count < 1) return ifail(c, DG_ERR_ARG, "no training residuals");
    const size_t n = (size_t)c->K * c->Np;
    std::vector<size_t> order(s->count);
    for (size_t i = 0; i < s->count; i++) order[i] = i;
    std::mt19937_64 rng(seed);
    int rc = DG_OK;
    for (int ep = 0; ep < epochs && !rc; ep++) {
        std::shuffle(order.begin(), order.end(), rng);
        for (size_t j = 0; j < s->count && !rc; j++) {
            const double* r = s->d_R + order[j] * n;
            rc = lpc_forward_vec(c, r, false);
            if (!rc) rc = lpc_backward_vec(c, r);
            if (!rc) rc = lpc_adam_step(c, lr);
        }
    }
    if (rc) return rc;
    // mean loss over the stored residuals (learned and block Jacobi alone)
    double L = 0, Lbj = 0;
    for (size_t j = 0; j < s->count && !rc; j++) {
        double l = 0, lb = 0;
        rc = lpc_forward_vec(c, s->d_R + j * n, true);
        if (!rc) rc = lpc_losses(c, &l, &lb);
        L += l;
        Lbj += lb;
    }
    if (rc) return rc;
    if (final_loss) *final_loss = L / s->count;
    if (final_loss_bj) *final_loss_bj = Lbj / s->count;
    if (!std::isfinite(L)) return ifail(c, DG_ERR_NONFINITE, "training diverged");
    return DG_OK;
}

int dg_lpc_loss(dg_ctx* c, const double* r_host, double* loss, double* loss_bj) {
    if (!c || !r_host) return DG_ERR_ARG;
    if (!lpc_ok(c)) return ifail(c, DG_ERR_ARG, "dg_lpc_setup not called");
    IpdgState* s = c->ipdg;
    int rc = lpc_upload_residual(c, r_host, s->d_r);
    if (!rc) rc = lpc_forward_vec(c, s->d_r, true);
    if (!rc) rc = lpc_losses(c, loss, loss_bj);
    return rc;
}

int dg_lpc_energy_gradients(dg_ctx* c, const double* r_host, float* gW1, float* gW2, double* loss) {
    if (!c || !r_host || !gW1) return DG_ERR_ARG;
    if (c->ipdg && !schwarz_form(c->ipdg->lpc_form) && !gW2) return DG_ERR_ARG;
    if (!lpc_ok(c)) return ifail(c, DG_ERR_ARG, "dg_lpc_setup not called");
    IpdgState* s = c->ipdg;
    int rc = lpc_upload_residual(c, r_host, s->d_r);
    if (!rc) rc = lpc_forward_vec(c, s->d_r, false);
    if (!rc) rc = lpc_backward_vec(c, s->d_r);
    if (!rc) rc = lpc_losses(c, loss, nullptr);
    if (rc) return rc;
    IP_CUDA(c, cudaMemcpyAsync(gW1, s->d_g1, (size_t)s->H * s->F * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    if (!schwarz_form(s->lpc_form))
        IP_CUDA(c, cudaMemcpyAsync(gW2, s->d_g2, (size_t)c->Np * s->H * sizeof(float), cudaMemcpyDeviceToHost,
                                   c->stream));
    IP_CUDA(c, cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_lpc_get_weights(dg_ctx* c, float* W1, float* W2) {
    if (!c || !W1) return DG_ERR_ARG;
    if (!lpc_ok(c)) return ifail(c, DG_ERR_ARG, "dg_lpc_setup not called");
    IpdgState* s = c->ipdg;
    const bool two = !schwarz_form(s->lpc_form);
    if (two && !W2) return DG_ERR_ARG;
    IP_CUDA(c, cudaMemcpyAsync(W1, s->d_W1, (size_t)s->H * s->F * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    if (two)
        IP_CUDA(c, cudaMemcpyAsync(W2, s->d_W2, (size_t)c->Np * s->H * sizeof(float), cudaMemcpyDeviceToHost,
                                   c->stream));
    IP_CUDA(c, cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_lpc_set_weights(dg_ctx* c, const float* W1, const float* W2) {
    if (!c || !W1) return DG_ERR_ARG;
    if (!lpc_ok(c)) return ifail(c, DG_ERR_ARG, "dg_lpc_setup not called");
    IpdgState* s = c->ipdg;
    const bool two = !schwarz_form(s->lpc_form);
    if (two && !W2) return DG_ERR_ARG;
    const int n1 = s->H * s->F, n2 = two ? c->Np * s->H : 0;
    IP_CUDA(c, cudaMemcpyAsync(s->d_W1, W1, n1 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    IP_CUDA(c, cudaMemsetAsync(s->d_m1, 0, n1 * sizeof(float), c->stream));
    IP_CUDA(c, cudaMemsetAsync(s->d_v1, 0, n1 * sizeof(float), c->stream));
    if (two) {
        IP_CUDA(c, cudaMemcpyAsync(s->d_W2, W2, n2 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        IP_CUDA(c, cudaMemsetAsync(s->d_m2, 0, n2 * sizeof(float), c->stream));
        IP_CUDA(c, cudaMemsetAsync(s->d_v2, 0, n2 * sizeof(float), c->stream));
    }
    s->adam_step = 0;
    int rc = lpc_refresh_bf16(c);
    if (rc) return rc;
    IP_CUDA(c, cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_lpc_gradients(dg_ctx* c, const float* X_host, const float* T_host, int B, float* gW1, float* gW2,
                     double* loss) {
    if (!c || !X_host || !T_host || B < 1 || !gW1 || !gW2) return DG_ERR_ARG;
    if (!lpc_ok(c)) return ifail(c, DG_ERR_ARG, "dg_lpc_setup not called");
    IpdgState* s = c->ipdg;
    if (schwarz_form(s->lpc_form))
        return ifail(c, DG_ERR_UNSUPPORTED, "batch gradients are defined for the two-layer forms");
    const int Np = c->Np;
    float *Xf = nullptr, *Td = nullptr, *Hs = nullptr, *dY = nullptr;
    __nv_bfloat16* Xb = nullptr;
    bool ok = cudaMalloc(&Xf, (size_t)B * s->F * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&Xb, (size_t)B * s->F * sizeof(__nv_bfloat16)) == cudaSuccess &&
              cudaMalloc(&Td, (size_t)B * Np * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&Hs, (size_t)2 * B * s->H * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&dY, (size_t)B * Np * sizeof(float)) == cudaSuccess;
    int rc = DG_OK;
    if (!ok) rc = ifail(c, DG_ERR_NOMEM, "dg_lpc_gradients: allocation failed");
    if (rc == DG_OK) {
        LpcNet net;
        LpcFeatArgs fa;
        lpc_descr(c, net, fa);
        cudaMemcpyAsync(Xf, X_host, (size_t)B * s->F * sizeof(float), cudaMemcpyHostToDevice, c->stream);
        cudaMemcpyAsync(Td, T_host, (size_t)B * Np * sizeof(float), cudaMemcpyHostToDevice, c->stream);
        f32_to_bf16_kernel<<<256, 256, 0, c->stream>>>(Xf, Xb, (long long)B * s->F);
        cudaError_t e = launch_lpc_forward(net, Xb, Td, B, Hs, dY, s->d_lpart, s->G, c->stream);
        if (e == cudaSuccess) e = launch_lpc_backward(net, Xb, Hs, dY, B, s->d_g1, s->d_g2, c->stream);
        double l = 0;
        if (e != cudaSuccess) rc = ifail(c, DG_ERR_CUDA, std::string("lpc kernels: ") + cudaGetErrorString(e));
        if (rc == DG_OK) rc = lpc_sum(c, s->d_lpart, &l);
        if (rc == DG_OK) {
            cudaMemcpyAsync(gW1, s->d_g1, (size_t)s->H * s->F * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
            cudaMemcpyAsync(gW2, s->d_g2, (size_t)Np * s->H * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
            cudaStreamSynchronize(c->stream);
            if (loss) *loss = l / (2.0 * B * Np);
        }
    }
    cudaFree(Xf);
    cudaFree(Xb);
    cudaFree(Td);
    cudaFree(Hs);
    cudaFree(dY);
    return rc;
}

int dg_lpc_apply(dg_ctx* c, const double* r_host, double* z_host) {
    if (!c || !r_host || !z_host) return DG_ERR_ARG;
    if (!lpc_ok(c)) return ifail(c, DG_ERR_ARG, "dg_lpc_setup not called");
    IpdgState* s = c->ipdg;
    const int K = c->K, Np = c->Np;
    const size_t n = (size_t)K * Np;
    int rc = lpc_upload_residual(c, r_host, s->d_r);
    if (rc) return rc;
    IP_CUDA(c, launch_bj(s->args, s->d_P32, s->d_r, s->d_zb, c->stream));
    LpcNet net;
    LpcFeatArgs fa;
    lpc_descr(c, net, fa);
    IP_CUDA(c, cudaMemsetAsync(s->d_z, 0, n * sizeof(double), c->stream));
    if (schwarz_form(s->lpc_form)) {
        IP_CUDA(c, launch_schwarz_local(s->sw, s->d_r, nullptr, s->d_U, nullptr, c->stream));
        IP_CUDA(c, launch_schwarz_collect(s->sw, s->d_zb, s->d_U, nullptr, s->d_z, nullptr, LPC_APPLY, nullptr,
                                          nullptr, c->stream));
    } else {
        IP_CUDA(c, launch_lpc_precond(net, fa, s->d_r, s->d_z, LPC_APPLY, nullptr, nullptr, nullptr, c->stream));
    }
    IP_CUDA(c, launch_permute(s->d_z, s->d_p, c->d_ring, K, Np, false, c->stream));
    IP_CUDA(c, cudaMemcpyAsync(z_host, s->d_p, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    IP_CUDA(c, cudaStreamSynchronize(c->stream));
    return DG_OK;
}

}  // extern "C"
