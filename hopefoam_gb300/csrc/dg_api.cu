// dg_api.cu -- C ABI of libdgcu (declared in include/dgcu.h).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dgcu.h"
#include "dg_ctx.hpp"

using namespace dgk;

namespace {

const double kRk4a[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                         -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
const double kRk4b[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                         1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                         2277821191437.0 / 14882151754819.0};

int fail(dg_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(dg_ctx* c, cudaError_t e, const char* where) {
    return fail(c, DG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define DG_CUDA(ctx, call)                                       \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

template <typename T>
int dmalloc(dg_ctx* c, T** p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(c, DG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    c->bytes += n * sizeof(T);
    c->allocs.push_back((void*)*p);
    return DG_OK;
}

template <typename T>
int upload(dg_ctx* c, T** p, const std::vector<T>& h) {
    int rc = dmalloc(c, p, h.size());
    if (rc) return rc;
    DG_CUDA(c, cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return DG_OK;
}

EulerArgs base_args(dg_ctx* c, int flux) {
    EulerArgs a;
    memset(&a, 0, sizeof(a));
    a.dtk = c->d_dtk;
    a.dtk32 = c->d_dtk32;
    a.geo = c->d_geo;
    a.conn = c->d_conn;
    a.btrace = c->d_btrace;
    a.ops = EulerOps{c->d_Vg, c->d_Sr, c->d_Ss, c->d_Lift, c->d_If};
    a.K = c->K;
    a.flux = flux;
    a.gamma = c->gamma;
    return a;
}

int run_stage(dg_ctx* c, const EulerArgs& a, int precision) {
    cudaError_t e;
    if (precision == DG_PREC_FP64) e = launch_euler_fp64(c->N, a, c->stream);
    else if (precision == DG_PREC_SPLIT) e = launch_euler_split(c->N, a, c->split, c->stream);
    else return fail(c, DG_ERR_ARG, "unknown precision");
    if (e != cudaSuccess) return cuda_fail(c, e, "euler stage launch");
    return DG_OK;
}

// The split kernel reports bounded-wait timeouts in a device status word.
int split_status_impl(dg_ctx* c, int precision) {
    if (precision != DG_PREC_SPLIT) return DG_OK;
    int st = 0;
    DG_CUDA(c, cudaMemcpyAsync(&st, c->split.d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    DG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (st != 0) {
        cudaMemsetAsync(c->split.d_status, 0, sizeof(int), c->stream);
        return fail(c, DG_ERR_TIMEOUT, "split kernel: tensor-core completion wait timed out");
    }
    return DG_OK;
}

int run_args_impl(dg_ctx* c, int flux, int precision) {
    if (!c) return DG_ERR_ARG;
    if (flux != DG_FLUX_LF && flux != DG_FLUX_ROE) return fail(c, DG_ERR_ARG, "unknown flux");
    if (precision != DG_PREC_FP64 && precision != DG_PREC_SPLIT) return fail(c, DG_ERR_ARG, "unknown precision");
    if (precision == DG_PREC_SPLIT && !c->split.ready) return fail(c, DG_ERR_UNSUPPORTED, "split path not built for this order");
    if (c->nb > 0 && !c->btrace_set) return fail(c, DG_ERR_ARG, "boundary traces not set");
    return DG_OK;
}

}  // namespace

int check_split_status(dg_ctx* c, int precision) { return split_status_impl(c, precision); }
int check_run_args(dg_ctx* c, int flux, int precision) { return run_args_impl(c, flux, precision); }

int euler_stage_mode(dg_ctx* c, const double* qin, double* qout, const double* qold, int mode, double dt, int flux,
                     int precision, const double* btrace) {
    EulerArgs a = base_args(c, flux);
    a.qin = qin;
    a.qout = qout;
    a.qold = qold;
    a.mode = mode;
    a.dt = dt;
    if (btrace) a.btrace = btrace;
    return run_stage(c, a, precision);
}

int lserk_stage_args(dg_ctx* c, double dt, int stage, int flux, EulerArgs* out) {
    EulerArgs a = base_args(c, flux);
    a.res = c->d_res;
    a.mode = MODE_LSERK;
    a.dt = dt;
    a.qin = c->d_q[c->cur];
    a.qout = c->d_q[c->cur ^ 1];
    a.rka = kRk4a[stage];
    a.rkb = kRk4b[stage];
    *out = a;
    return DG_OK;
}

int lserk_stage(dg_ctx* c, double dt, int stage, int flux, int precision) {
    EulerArgs a = base_args(c, flux);
    a.res = c->d_res;
    a.mode = MODE_LSERK;
    a.dt = dt;
    a.qin = c->d_q[c->cur];
    a.qout = c->d_q[c->cur ^ 1];
    a.rka = kRk4a[stage];
    a.rkb = kRk4b[stage];
    int rc = refresh_boundary_traces(c, a.qin);
    if (rc) return rc;
    rc = run_stage(c, a, precision);
    if (rc) return rc;
    c->cur ^= 1;
    return DG_OK;
}

extern "C" {

int dg_ctx_create(const dg_mesh_desc* m, const dg_opts* o, dg_ctx** out) {
    if (!out) return DG_ERR_ARG;
    *out = nullptr;
    if (!m || !o || m->K <= 0 || !m->VXY || !m->EToE || !m->EToF) return DG_ERR_ARG;
    dg_ctx* c = new dg_ctx();
    if (cudaGetDevice(&c->device) != cudaSuccess) {
        delete c;
        return DG_ERR_CUDA;
    }
    c->K = m->K;
    c->N = o->order;
    c->gamma = o->gamma > 0 ? o->gamma : 1.4;
    int expect = dgb::cubature_points_for_order(o->order);
    if (expect == 0) { dg_ctx_destroy(c); return DG_ERR_UNSUPPORTED; }
    if (o->n_cubature != expect || !o->cubature) {
        dg_ctx_destroy(c);
        return DG_ERR_ARG;
    }
    std::string e = dgb::build_ref_ops(o->order, o->cubature, o->n_cubature, c->ops);
    if (!e.empty()) { dg_ctx_destroy(c); return DG_ERR_ARG; }
    c->Np = c->ops.Np;
    c->Ng = c->ops.Ng;
    c->Nfp = c->ops.Nfp;
    c->Nfq = c->ops.Nfq;
    const int K = c->K;

    // geometry (affine metrics) and connectivity
    std::vector<double> geo((size_t)K * 4);
    std::vector<int> conn((size_t)K * 3);
    double minh = 1e300;
    for (int k = 0; k < K; k++) {
        const double* v = m->VXY + 6 * (size_t)k;
        double xr = 0.5 * (v[2] - v[0]), yr = 0.5 * (v[3] - v[1]);
        double xs = 0.5 * (v[4] - v[0]), ys = 0.5 * (v[5] - v[1]);
        double J = xr * ys - xs * yr;
        if (!(J > 0)) {
            delete c;
            return DG_ERR_ARG;  // vertices must be counter-clockwise and non-degenerate
        }
        geo[4 * (size_t)k + 0] = ys / J;
        geo[4 * (size_t)k + 1] = -yr / J;
        geo[4 * (size_t)k + 2] = -xs / J;
        geo[4 * (size_t)k + 3] = xr / J;
        double emax = 0;
        for (int f = 0; f < 3; f++) {
            double dx = v[2 * ((f + 1) % 3)] - v[2 * f], dy = v[2 * ((f + 1) % 3) + 1] - v[2 * f + 1];
            emax = std::max(emax, std::sqrt(dx * dx + dy * dy));
        }
        minh = std::min(minh, 2.0 * (2.0 * J) / emax);  // area = 2J
    }
    c->min_h = minh;
    int nb = 0;
    for (int k = 0; k < K; k++)
        for (int f = 0; f < 3; f++) {
            int n = m->EToE[3 * (size_t)k + f], fn = m->EToF[3 * (size_t)k + f];
            if (n < 0) {
                conn[3 * (size_t)k + f] = -1 - nb;
                nb++;
                continue;
            }
            if (n >= K || fn < 0 || fn > 2 || m->EToE[3 * (size_t)n + fn] != k || m->EToF[3 * (size_t)n + fn] != f) {
                delete c;
                return DG_ERR_ARG;  // inconsistent face connectivity
            }
            int rot;
            if (m->ROT) rot = m->ROT[3 * (size_t)k + f];
            else if (m->EToV) rot = (m->EToV[3 * (size_t)k + f] == m->EToV[3 * (size_t)n + (fn + 1) % 3]) ? 1 : 0;
            else rot = 1;
            if (n >= (1 << 28)) { delete c; return DG_ERR_UNSUPPORTED; }
            conn[3 * (size_t)k + f] = (n << 3) | ((rot & 1) << 2) | fn;
        }
    c->nb = nb;

    // stream
    if (o->stream) {
        c->stream = (cudaStream_t)o->stream;
        c->own_stream = false;
    } else {
        cudaError_t ce = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (ce != cudaSuccess) { delete c; return DG_ERR_CUDA; }
        c->own_stream = true;
    }
    // device buffers
    size_t n = (size_t)K * 4 * c->Np;
    int rc = 0;
    rc |= dmalloc(c, &c->d_q[0], n);
    rc |= dmalloc(c, &c->d_q[1], n);
    rc |= dmalloc(c, &c->d_res, n);
    rc |= dmalloc(c, &c->d_stage, n);
    rc |= upload(c, &c->d_geo, geo);
    rc |= upload(c, &c->d_conn, conn);
    rc |= upload(c, &c->d_ring, c->ops.ring);
    rc |= upload(c, &c->d_Vg, c->ops.dVg);
    rc |= upload(c, &c->d_Sr, c->ops.dSr);
    rc |= upload(c, &c->d_Ss, c->ops.dSs);
    rc |= upload(c, &c->d_Lift, c->ops.dLift);
    rc |= upload(c, &c->d_If, c->ops.If);
    rc |= dmalloc(c, &c->d_btrace, (size_t)std::max(nb, 1) * 4 * c->Nfp);
    if (rc) { dg_ctx_destroy(c); return DG_ERR_NOMEM; }
    if (cudaMemset(c->d_res, 0, n * sizeof(double)) != cudaSuccess ||
        cudaMemset(c->d_q[0], 0, n * sizeof(double)) != cudaSuccess) {
        dg_ctx_destroy(c);
        return DG_ERR_CUDA;
    }
    c->geo_host = geo;
    c->conn_host = conn;
    if (m->EToV) c->etov_host.assign(m->EToV, m->EToV + 3 * (size_t)K);
    c->vxy_host.assign(m->VXY, m->VXY + 6 * (size_t)K);
    if (split_setup(c) != DG_OK) c->split.ready = false;
    if (cudaDeviceSynchronize() != cudaSuccess) { dg_ctx_destroy(c); return DG_ERR_CUDA; }
    *out = c;
    return DG_OK;
}

int dg_ctx_destroy(dg_ctx* c) {
    if (!c) return DG_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    split_teardown(c);
    ipdg_teardown(c);
    limiter_teardown(c);
    for (void* p : c->allocs) cudaFree(p);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return DG_OK;
}

int dg_get_info(const dg_ctx* c, dg_info* info) {
    if (!c || !info) return DG_ERR_ARG;
    info->K = c->K;
    info->order = c->N;
    info->Np = c->Np;
    info->Ng = c->Ng;
    info->Nfp = c->Nfp;
    info->Nfq = c->Nfq;
    info->n_bfaces = c->nb;
    info->stream = (void*)c->stream;
    info->device_bytes = c->bytes;
    return DG_OK;
}

const char* dg_last_error(const dg_ctx* c) { return c ? c->err.c_str() : "null context"; }

int dg_set_element_dt(dg_ctx* c, const double* dtk_host) {
    if (!c) return DG_ERR_ARG;
    if (!dtk_host) {
        c->d_dtk = nullptr;  // the buffers stay allocated for a later call
        c->d_dtk32 = nullptr;
        return DG_OK;
    }
    for (int k = 0; k < c->K; k++)
        if (!(dtk_host[k] > 0) || !std::isfinite(dtk_host[k])) return fail(c, DG_ERR_ARG, "time-step factors must be positive");
    if (!c->dtk_buf) {
        int rc = dmalloc(c, &c->dtk_buf, (size_t)c->K);
        if (rc) return rc;
    }
    DG_CUDA(c, cudaMemcpy(c->dtk_buf, dtk_host, (size_t)c->K * sizeof(double), cudaMemcpyHostToDevice));
    c->d_dtk = c->dtk_buf;
    if (!c->dtk32_buf) {
        int rc = dmalloc(c, &c->dtk32_buf, (size_t)c->K);
        if (rc) return rc;
    }
    std::vector<float> f32(dtk_host, dtk_host + c->K);
    DG_CUDA(c, cudaMemcpy(c->dtk32_buf, f32.data(), (size_t)c->K * sizeof(float), cudaMemcpyHostToDevice));
    c->d_dtk32 = c->dtk32_buf;
    return DG_OK;
}

int dg_upload_state_device(dg_ctx* c, const double* q_dev) {
    if (!c || !q_dev) return DG_ERR_ARG;
    cudaError_t e = launch_to_internal(q_dev, c->d_q[c->cur], c->d_ring, c->K, c->Np, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "to_internal");
    DG_CUDA(c, cudaMemsetAsync(c->d_res, 0, (size_t)c->K * 4 * c->Np * sizeof(double), c->stream));
    return DG_OK;
}

int dg_download_state_device(dg_ctx* c, double* q_dev) {
    if (!c || !q_dev) return DG_ERR_ARG;
    cudaError_t e = launch_to_reference(c->d_q[c->cur], q_dev, c->d_ring, c->K, c->Np, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "to_reference");
    return DG_OK;
}

int dg_upload_state(dg_ctx* c, const double* q_host) {
    if (!c || !q_host) return DG_ERR_ARG;
    size_t n = (size_t)c->K * 4 * c->Np;
    DG_CUDA(c, cudaMemcpyAsync(c->d_stage, q_host, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    int rc = dg_upload_state_device(c, c->d_stage);
    if (rc) return rc;
    DG_CUDA(c, cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_download_state(dg_ctx* c, double* q_host) {
    if (!c || !q_host) return DG_ERR_ARG;
    size_t n = (size_t)c->K * 4 * c->Np;
    int rc = dg_download_state_device(c, c->d_stage);
    if (rc) return rc;
    DG_CUDA(c, cudaMemcpyAsync(q_host, c->d_stage, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    DG_CUDA(c, cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_set_boundary_traces(dg_ctx* c, const double* tr) {
    if (!c || (!tr && c->nb > 0)) return DG_ERR_ARG;
    if (c->nb > 0)
        DG_CUDA(c, cudaMemcpyAsync(c->d_btrace, tr, (size_t)c->nb * 4 * c->Nfp * sizeof(double), cudaMemcpyHostToDevice,
                                   c->stream));
    DG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->btrace_set = true;
    return DG_OK;
}

int dg_euler_rhs(dg_ctx* c, int flux, int precision, double* rhs_host) {
    int rc = check_run_args(c, flux, precision);
    if (rc) return rc;
    if (!rhs_host) return fail(c, DG_ERR_ARG, "rhs_host is NULL");
    EulerArgs a = base_args(c, flux);
    a.qin = c->d_q[c->cur];
    a.rhs = c->d_q[c->cur ^ 1];  // scratch: the spare state buffer
    a.mode = MODE_RHS;
    if ((rc = refresh_boundary_traces(c, a.qin))) return rc;
    rc = run_stage(c, a, precision);
    if (rc) return rc;
    rc = check_split_status(c, precision);
    if (rc) return rc;
    cudaError_t e = launch_to_reference(a.rhs, c->d_stage, c->d_ring, c->K, c->Np, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "to_reference");
    DG_CUDA(c, cudaMemcpyAsync(rhs_host, c->d_stage, (size_t)c->K * 4 * c->Np * sizeof(double), cudaMemcpyDeviceToHost,
                               c->stream));
    DG_CUDA(c, cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_euler_rhs_device(dg_ctx* c, int flux, int precision, double* rhs_dev) {
    int rc = check_run_args(c, flux, precision);
    if (rc) return rc;
    if (!rhs_dev) return fail(c, DG_ERR_ARG, "rhs_dev is NULL");
    EulerArgs a = base_args(c, flux);
    a.qin = c->d_q[c->cur];
    a.rhs = c->d_q[c->cur ^ 1];  // scratch: the spare state buffer
    a.mode = MODE_RHS;
    if ((rc = refresh_boundary_traces(c, a.qin))) return rc;
    rc = run_stage(c, a, precision);
    if (rc) return rc;
    cudaError_t e = launch_to_reference(a.rhs, rhs_dev, c->d_ring, c->K, c->Np, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "to_reference");
    return DG_OK;
}

int dg_forward_euler_stage(dg_ctx* c, double dt, int flux, int precision) {
    int rc = check_run_args(c, flux, precision);
    if (rc) return rc;
    if (!(dt > 0)) return fail(c, DG_ERR_ARG, "bad dt");
    EulerArgs a = base_args(c, flux);
    a.dt = dt;
    a.mode = MODE_EULER;
    a.qin = c->d_q[c->cur];
    a.qout = c->d_q[c->cur ^ 1];
    if ((rc = refresh_boundary_traces(c, a.qin))) return rc;
    rc = run_stage(c, a, precision);
    if (rc) return rc;
    c->cur ^= 1;
    return DG_OK;
}

int dg_sync(dg_ctx* c) {
    if (!c) return DG_ERR_ARG;
    if (c->split.ready) return check_split_status(c, DG_PREC_SPLIT);
    DG_CUDA(c, cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_lserk4_step(dg_ctx* c, double dt, int nsteps, int flux, int precision) {
    int rc = check_run_args(c, flux, precision);
    if (rc) return rc;
    if (nsteps < 0 || !(dt > 0)) return fail(c, DG_ERR_ARG, "bad dt / nsteps");
    EulerArgs a = base_args(c, flux);
    a.res = c->d_res;
    a.mode = MODE_LSERK;
    a.dt = dt;
    for (int s = 0; s < nsteps; s++)
        for (int st = 0; st < 5; st++) {
            a.qin = c->d_q[c->cur];
            a.qout = c->d_q[c->cur ^ 1];
            a.rka = kRk4a[st];
            a.rkb = kRk4b[st];
            rc = refresh_boundary_traces(c, a.qin);
            if (rc) return rc;
            rc = run_stage(c, a, precision);
            if (rc) return rc;
            c->cur ^= 1;
        }
    return check_split_status(c, precision);
}

int dg_ssprk2_step(dg_ctx* c, double dt, int nsteps, int flux, int precision) {
    int rc = check_run_args(c, flux, precision);
    if (rc) return rc;
    if (nsteps < 0 || !(dt > 0)) return fail(c, DG_ERR_ARG, "bad dt / nsteps");
    EulerArgs a = base_args(c, flux);
    a.dt = dt;
    for (int s = 0; s < nsteps; s++) {
        // stage 1: q1 = q + dt R(q)  -> spare buffer
        a.qin = c->d_q[c->cur];
        a.qout = c->d_q[c->cur ^ 1];
        a.mode = MODE_EULER;
        if ((rc = refresh_boundary_traces(c, a.qin))) return rc;
        rc = run_stage(c, a, precision);
        if (rc) return rc;
        // stage 2: q = q/2 + (q1 + dt R(q1))/2, written over q (element-local reads of q only)
        a.qin = c->d_q[c->cur ^ 1];
        a.qold = c->d_q[c->cur];
        a.qout = c->d_q[c->cur];
        a.mode = MODE_SSP2;
        if ((rc = refresh_boundary_traces(c, a.qin))) return rc;
        rc = run_stage(c, a, precision);
        if (rc) return rc;
    }
    return check_split_status(c, precision);
}

int dg_cfl_dt(dg_ctx* c, double cfl, double* dt) {
    if (!c || !dt || !(cfl > 0)) return DG_ERR_ARG;
    size_t n = (size_t)c->K * 4 * c->Np;
    std::vector<double> q(n);
    int rc = dg_download_state(c, q.data());
    if (rc) return rc;
    size_t KN = (size_t)c->K * c->Np;
    double smax = 0;
    for (size_t i = 0; i < KN; i++) {
        double rho = q[i], u = q[KN + i] / rho, v = q[2 * KN + i] / rho;
        double p = (c->gamma - 1) * (q[3 * KN + i] - 0.5 * rho * (u * u + v * v));
        double s = std::sqrt(u * u + v * v) + std::sqrt(std::fabs(c->gamma * p / rho));
        if (!std::isfinite(s)) return fail(c, DG_ERR_NONFINITE, "non-finite state in dg_cfl_dt");
        smax = std::max(smax, s);
    }
    *dt = cfl * c->min_h / ((c->N + 1) * (c->N + 1) * smax);
    return DG_OK;
}

int dg_reference_operators(int order, const double* cub, int n_cub, double* r, double* s, double* Dr, double* Ds,
                           double* Vg, double* If, double* Mref) {
    if (dgb::cubature_points_for_order(order) == 0) return DG_ERR_UNSUPPORTED;
    if (!cub || n_cub != dgb::cubature_points_for_order(order)) return DG_ERR_ARG;
    dgb::RefOps o;
    if (!dgb::build_ref_ops(order, cub, n_cub, o).empty()) return DG_ERR_ARG;
    auto put = [](double* dst, const std::vector<double>& v) {
        if (dst) std::copy(v.begin(), v.end(), dst);
    };
    put(r, o.r);
    put(s, o.s);
    put(Dr, o.Dr);
    put(Ds, o.Ds);
    put(Vg, o.Vg);
    put(If, o.If);
    put(Mref, o.Mref);
    return DG_OK;
}

}  // extern "C"
