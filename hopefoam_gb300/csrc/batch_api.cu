// batch_api.cu -- many independent Euler cases advanced together: groups of
// same-order cases (each group one context over the cases' disjoint meshes,
// with per-element time-step factors), all stages of all groups captured
// into one CUDA graph, the launch shapes chosen by a measuring autotuner.
//
// No counterpart in the reference (it runs one case per process).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dgcu.h"
#include "dg_ctx.hpp"
#include "euler_split.cuh"

struct dg_batch {
    std::vector<dg_ctx*> groups;
    std::vector<cudaStream_t> streams;  // one per group
    std::vector<cudaStream_t> saved;    // the groups' own streams
    cudaStream_t main = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> joins;
    // schedule
    // 0: groups one after another on the whole GPU; 1: side by side on
    // streams; 2: every stage of every group in one launch (the mixed-order
    // kernel, each group on its share of the SMs)
    int concurrent = 0;
    std::vector<int> ctas_per_sm;    // per group
    std::vector<int> sm_budget;      // per group (concurrent schedule)
    // captured graph
    cudaGraphExec_t exec = nullptr;
    int g_steps = -1, g_flux = -1, g_prec = -1;
    double g_dt = 0;
    std::vector<int> g_cur;          // buffer parity each group started from when captured
    int sms = 0;
    std::string err;
};

namespace {

int bfail(dg_batch* b, int code, const std::string& m) {
    if (b) b->err = m;
    return code;
}

#define B_CUDA(b, call)                                                                                   \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return bfail(b, DG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

void apply_shape(dg_batch* b) {
    for (size_t g = 0; g < b->groups.size(); g++) {
        b->groups[g]->split.ctas_per_sm = b->ctas_per_sm[g];
        b->groups[g]->split.sm_budget = b->concurrent == 1 ? b->sm_budget[g] : 0;
    }
}

void drop_graph(dg_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->g_steps = -1;
}

// the mixed-order single launch per stage needs split precision, orders
// 1..6 on the pipelined body, 16-byte aligned states and no per-stage
// boundary-trace refresh
bool fused_ok(const dg_batch* b, int precision) {
    if (precision != DG_PREC_SPLIT || b->groups.size() > (size_t)dgk::SplitBatchArgs::MAXG) return false;
    for (const dg_ctx* c : b->groups) {
        if (c->N > 6 || !c->split.ready || c->split.variant == dgk::SplitPlan::CLASSIC) return false;
        if (has_dynamic_traces(c)) return false;
        if ((reinterpret_cast<uintptr_t>(c->d_q[0]) & 15u) || (reinterpret_cast<uintptr_t>(c->d_q[1]) & 15u))
            return false;
    }
    return true;
}

int issue_steps_fused(dg_batch* b, double dt, int nsteps, int flux) {
    const int G = (int)b->groups.size();
    for (int s = 0; s < nsteps; s++)
        for (int k = 0; k < 5; k++) {
            dgk::SplitBatchArgs P;
            memset(&P, 0, sizeof(P));
            P.ngroups = G;
            int acc = 0;
            for (int g = 0; g < G; g++) {
                dg_ctx* c = b->groups[g];
                dgk::EulerArgs a;
                lserk_stage_args(c, dt, k, flux, &a);
                dgk::split_fill_args(a, c->split, &P.sa[g]);
                P.order[g] = c->N;
                const int ntiles = (c->K + dgk::SplitDims<1>::E - 1) / dgk::SplitDims<1>::E;
                acc += std::max(1, std::min(ntiles, b->sm_budget[g]));
                P.cta_end[g] = acc;
            }
            B_CUDA(b, dgk::launch_split_batch(P, b->main));
            for (int g = 0; g < G; g++) b->groups[g]->cur ^= 1;
        }
    return DG_OK;
}

// issues nsteps LSERK4 steps of every group into the batch streams
int issue_steps(dg_batch* b, double dt, int nsteps, int flux, int precision) {
    const int G = (int)b->groups.size();
    if (b->concurrent == 2) return issue_steps_fused(b, dt, nsteps, flux);
    B_CUDA(b, cudaEventRecord(b->fork, b->main));
    for (int g = 0; g < G; g++) {
        cudaStream_t st = b->concurrent ? b->streams[g] : b->main;
        if (b->concurrent) B_CUDA(b, cudaStreamWaitEvent(st, b->fork, 0));
        dg_ctx* c = b->groups[g];
        c->stream = st;
        for (int s = 0; s < nsteps; s++)
            for (int k = 0; k < 5; k++) {
                int rc = lserk_stage(c, dt, k, flux, precision);
                if (rc) {
                    b->err = c->err;
                    return rc;
                }
            }
        if (b->concurrent) {
            B_CUDA(b, cudaEventRecord(b->joins[g], st));
            B_CUDA(b, cudaStreamWaitEvent(b->main, b->joins[g], 0));
        }
    }
    return DG_OK;
}

void restore_streams(dg_batch* b) {
    for (size_t g = 0; g < b->groups.size(); g++) b->groups[g]->stream = b->saved[g];
}

int check_groups(dg_batch* b, int precision) {
    for (size_t g = 0; g < b->groups.size(); g++) {
        int rc = check_split_status(b->groups[g], precision);
        if (rc) {
            b->err = b->groups[g]->err;
            return rc;
        }
    }
    return DG_OK;
}

// milliseconds for nsteps (events on the main stream), state advanced
int time_steps(dg_batch* b, double dt, int nsteps, int flux, int precision, float* ms) {
    cudaEvent_t e0, e1;
    B_CUDA(b, cudaEventCreate(&e0));
    B_CUDA(b, cudaEventCreate(&e1));
    B_CUDA(b, cudaEventRecord(e0, b->main));
    int rc = issue_steps(b, dt, nsteps, flux, precision);
    restore_streams(b);
    if (!rc) {
        B_CUDA(b, cudaEventRecord(e1, b->main));
        B_CUDA(b, cudaEventSynchronize(e1));
        B_CUDA(b, cudaEventElapsedTime(ms, e0, e1));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

}  // namespace

extern "C" {

int dg_batch_create(dg_ctx* const* groups, int n_groups, dg_batch** out) {
    if (!groups || n_groups < 1 || !out) return DG_ERR_ARG;
    dg_batch* b = new dg_batch();
    for (int g = 0; g < n_groups; g++) {
        if (!groups[g]) {
            delete b;
            return DG_ERR_ARG;
        }
        for (int h = 0; h < g; h++)
            if (groups[h] == groups[g]) {
                delete b;
                return DG_ERR_ARG;
            }
        b->groups.push_back(groups[g]);
        b->saved.push_back(groups[g]->stream);
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    bool ok = cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
    for (int g = 0; g < n_groups && ok; g++) {
        cudaStream_t s;
        cudaEvent_t e;
        ok = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
        if (ok) {
            b->streams.push_back(s);
            b->joins.push_back(e);
        }
    }
    b->ctas_per_sm.assign(n_groups, 1);
    b->sm_budget.assign(n_groups, b->sms);
    if (!ok) {
        dg_batch_destroy(b);
        return DG_ERR_CUDA;
    }
    *out = b;
    return DG_OK;
}

int dg_batch_destroy(dg_batch* b) {
    if (!b) return DG_OK;
    if (b->main) cudaStreamSynchronize(b->main);
    drop_graph(b);
    restore_streams(b);
    for (dg_ctx* c : b->groups) {
        c->split.ctas_per_sm = 1;
        c->split.sm_budget = 0;
    }
    for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
    for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->main) cudaStreamDestroy(b->main);
    delete b;
    return DG_OK;
}

const char* dg_batch_last_error(const dg_batch* b) { return b ? b->err.c_str() : "null batch"; }

int dg_batch_tune(dg_batch* b, double dt, int flux, int precision, int steps_per_trial, dg_batch_tuning* result) {
    if (!b || !(dt > 0) || steps_per_trial < 1) return DG_ERR_ARG;
    const int G = (int)b->groups.size();
    for (dg_ctx* c : b->groups) {
        int rc = check_run_args(c, flux, precision);
        if (rc) return bfail(b, rc, c->err);
        B_CUDA(b, cudaStreamSynchronize(c->stream));
    }
    drop_graph(b);
    // the trials advance the state: keep a copy of every group's current state
    std::vector<double*> keep(G, nullptr);
    for (int g = 0; g < G; g++) {
        dg_ctx* c = b->groups[g];
        const size_t n = (size_t)c->K * 4 * c->Np;
        B_CUDA(b, cudaMalloc(&keep[g], n * sizeof(double)));
        B_CUDA(b, cudaMemcpy(keep[g], c->d_q[c->cur], n * sizeof(double), cudaMemcpyDeviceToDevice));
    }
    // work weights: one stage of each group alone on the whole GPU
    b->concurrent = 0;
    std::vector<int> cps_best(G, 1);
    std::vector<float> t_alone(G, 0.f);
    int rc = DG_OK;
    for (int g = 0; g < G && !rc; g++) {
        dg_ctx* c = b->groups[g];
        // CTAs per SM: 1, and 2 where two CTAs fit (split kernel, small orders)
        const int max_cps = (precision == DG_PREC_SPLIT && c->N <= 2) ? 2 : 1;
        float best = 1e30f;
        for (int cps = 1; cps <= max_cps && !rc; cps++) {
            std::vector<dg_ctx*> only{c};
            dg_batch one;  // a one-group view sharing the streams
            one.groups = only;
            one.saved = {c->stream};
            one.main = b->main;
            one.fork = b->fork;
            one.joins = {b->joins[g]};
            one.streams = {b->streams[g]};
            one.concurrent = 0;
            one.ctas_per_sm = {cps};
            one.sm_budget = {b->sms};
            apply_shape(&one);
            float ms = 0;
            rc = time_steps(&one, dt, 1, flux, precision, &ms);  // warm
            if (!rc) rc = time_steps(&one, dt, steps_per_trial, flux, precision, &ms);
            one.main = nullptr;  // not owned
            one.fork = nullptr;
            one.joins.clear();
            one.streams.clear();
            if (!rc && ms < best) {
                best = ms;
                cps_best[g] = cps;
            }
        }
        t_alone[g] = best;
    }
    float t_seq = 0, t_conc = 1e30f;
    if (!rc) {
        b->ctas_per_sm = cps_best;
        b->concurrent = 0;
        apply_shape(b);
        rc = time_steps(b, dt, steps_per_trial, flux, precision, &t_seq);
    }
    std::vector<int> budget(G, b->sms);
    if (!rc && G > 1) {
        // side by side: SMs split in proportion to each group's time alone
        double tot = 0;
        for (float t : t_alone) tot += t;
        int used = 0;
        for (int g = 0; g < G; g++) {
            budget[g] = std::max(1, (int)std::floor(b->sms * t_alone[g] / tot));
            used += budget[g];
        }
        for (int g = 0; used < b->sms; g = (g + 1) % G, used++) budget[g]++;
        b->sm_budget = budget;
        b->concurrent = 1;
        apply_shape(b);
        rc = time_steps(b, dt, steps_per_trial, flux, precision, &t_conc);
    }
    float t_fused = 1e30f;
    if (!rc && fused_ok(b, precision)) {
        // one launch per stage, each group on its share of the SMs
        b->sm_budget = budget;
        b->concurrent = 2;
        apply_shape(b);
        rc = time_steps(b, dt, steps_per_trial, flux, precision, &t_fused);
    }
    if (!rc) {
        b->concurrent = 0;
        float best = t_seq;
        if (G > 1 && t_conc < best) {
            b->concurrent = 1;
            best = t_conc;
        }
        if (t_fused < best) b->concurrent = 2;
        b->sm_budget = budget;
        apply_shape(b);
        if (result) {
            result->concurrent = b->concurrent;
            result->ms_sequential = t_seq / steps_per_trial;
            result->ms_concurrent = G > 1 ? t_conc / steps_per_trial : t_seq / steps_per_trial;
            result->ms_fused = t_fused < 1e29f ? t_fused / steps_per_trial : 0.0;
        }
    }
    // restore the states
    for (int g = 0; g < G; g++) {
        dg_ctx* c = b->groups[g];
        const size_t n = (size_t)c->K * 4 * c->Np;
        if (keep[g]) {
            cudaMemcpy(c->d_q[c->cur], keep[g], n * sizeof(double), cudaMemcpyDeviceToDevice);
            cudaFree(keep[g]);
        }
    }
    if (!rc) rc = check_groups(b, precision);
    return rc;
}

int dg_batch_set_schedule(dg_batch* b, int schedule, int precision) {
    if (!b || schedule < 0 || schedule > 2) return DG_ERR_ARG;
    if (schedule == 2 && !fused_ok(b, precision))
        return bfail(b, DG_ERR_UNSUPPORTED, "one launch per stage needs split precision, orders <= 6, <= 8 groups");
    const int G = (int)b->groups.size();
    if (schedule != 0 && b->sm_budget.size() == (size_t)G) {
        // SM shares in proportion to the groups' element-node counts unless tuned before
        int sum = 0;
        for (int v : b->sm_budget) sum += v;
        if (sum != b->sms) {
            double tot = 0;
            for (const dg_ctx* c : b->groups) tot += (double)c->K * c->Np;
            int used = 0;
            for (int g = 0; g < G; g++) {
                b->sm_budget[g] = std::max(1, (int)std::floor(b->sms * (double)b->groups[g]->K * b->groups[g]->Np / tot));
                used += b->sm_budget[g];
            }
            for (int g = 0; used < b->sms; g = (g + 1) % G, used++) b->sm_budget[g]++;
        }
    }
    drop_graph(b);
    b->concurrent = schedule;
    apply_shape(b);
    return DG_OK;
}

int dg_batch_get_shape(const dg_batch* b, int group, int* ctas_per_sm, int* sm_budget, int* concurrent) {
    if (!b || group < 0 || group >= (int)b->groups.size()) return DG_ERR_ARG;
    if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm[group];
    if (sm_budget) *sm_budget = b->concurrent ? b->sm_budget[group] : b->sms;  // schedules 1 and 2: its share
    if (concurrent) *concurrent = b->concurrent;
    return DG_OK;
}

int dg_batch_run(dg_batch* b, double dt, int nsteps, int flux, int precision, double* ms) {
    if (!b || !(dt > 0) || nsteps < 0) return DG_ERR_ARG;
    const int G = (int)b->groups.size();
    for (dg_ctx* c : b->groups) {
        int rc = check_run_args(c, flux, precision);
        if (rc) return bfail(b, rc, c->err);
        B_CUDA(b, cudaStreamSynchronize(c->stream));  // the group's own work is done before the batch runs
    }
    if (nsteps == 0) return DG_OK;
    apply_shape(b);
    bool same = b->exec && b->g_steps == nsteps && b->g_flux == flux && b->g_prec == precision && b->g_dt == dt;
    for (int g = 0; g < G && same; g++) same = b->g_cur[g] == b->groups[g]->cur;
    if (!same) {
        drop_graph(b);
        std::vector<int> start(G);
        for (int g = 0; g < G; g++) start[g] = b->groups[g]->cur;
        B_CUDA(b, cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal));
        int rc = issue_steps(b, dt, nsteps, flux, precision);
        restore_streams(b);
        cudaGraph_t graph = nullptr;
        cudaError_t ce = cudaStreamEndCapture(b->main, &graph);
        if (rc || ce != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            for (int g = 0; g < G; g++) b->groups[g]->cur = start[g];
            return rc ? rc : bfail(b, DG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
        }
        ce = cudaGraphInstantiate(&b->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) {
            b->exec = nullptr;
            for (int g = 0; g < G; g++) b->groups[g]->cur = start[g];
            return bfail(b, DG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
        }
        b->g_steps = nsteps;
        b->g_flux = flux;
        b->g_prec = precision;
        b->g_dt = dt;
        b->g_cur = start;
        // capture advanced the host-side buffer parity; the launch below starts from `start`
        for (int g = 0; g < G; g++) b->groups[g]->cur = start[g];
    }
    cudaEvent_t e0, e1;
    B_CUDA(b, cudaEventCreate(&e0));
    B_CUDA(b, cudaEventCreate(&e1));
    B_CUDA(b, cudaEventRecord(e0, b->main));
    B_CUDA(b, cudaGraphLaunch(b->exec, b->main));
    B_CUDA(b, cudaEventRecord(e1, b->main));
    B_CUDA(b, cudaEventSynchronize(e1));
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms) *ms = t;
    // buffer parity after the replay: 5 stages per step
    for (int g = 0; g < G; g++) b->groups[g]->cur = b->g_cur[g] ^ ((5 * nsteps) & 1);
    return check_groups(b, precision);
}

}  // extern "C"
