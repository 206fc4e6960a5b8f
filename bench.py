"""Benchmark of the DG Euler hot path on one GB300 (one JSON line on stdout).

Workload (the configuration the headline metric is quoted on): isentropic
vortex (gamma 1.4, strength 5, free stream rho=1, u=1, v=0, p=1) on a periodic
[0,10]^2 256x256x2 triangulation (K = 131072) with vertices perturbed by
U(-0.1h, 0.1h) (seed 0), order N = 5 (Np = 21), Lax-Friedrichs flux, LSERK4 at
CFL 0.5.  One bench step = one LSERK4 time step (5 RK stages) over the whole
mesh.  Metric: DOF-stage updates/s, DOF = K*Np*4 conserved node values.

--impl reference times the CPU oracle (the reference's algorithm restated in
C++, OpenMP over all host threads) on the same mesh and metric.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DG DOF-stage updates/s (isentropic vortex N=5, K=131072, LSERK4)"
UNIT = "DOF-stage/s"


def workload(nx=256, order=5):
    from hopefoam_gb300.mesh import periodic_square

    return periodic_square(nx, nx, 10.0, 10.0, perturb=0.1, seed=0)


def initial_state(mesh, order):
    """The vortex at the product's nodes (libdgcu's reference element)."""
    from hopefoam_gb300 import euler

    ops = euler.reference_operators(order)
    x, y = euler.node_coords(mesh, ops["r"], ops["s"])
    return euler.isentropic_vortex(x, y, x0=5.0, y0=5.0), x, y


def initial_state_oracle(orc):
    """The vortex at the oracle's own nodes: the reference arm never loads
    libdgcu."""
    from hopefoam_gb300 import euler

    x, y = orc.nodes()
    return euler.isentropic_vortex(x, y, x0=5.0, y0=5.0)


def host_cfl_dt(mesh, order, q, cfl=0.5, gamma=1.4):
    """The CFL rule of dg_cfl_dt, evaluated on the host from the initial
    state: dt = cfl * min_k(2 * area_k / longest edge_k) / ((N+1)^2 *
    max(|u| + c)).  Both bench arms use this dt, so they run the same
    configuration."""
    v = np.asarray(mesh.VXY, np.float64)
    e = np.stack([np.hypot(*(v[:, (f + 1) % 3] - v[:, f]).T) for f in range(3)], 1)
    xr, yr = 0.5 * (v[:, 1, 0] - v[:, 0, 0]), 0.5 * (v[:, 1, 1] - v[:, 0, 1])
    xs, ys = 0.5 * (v[:, 2, 0] - v[:, 0, 0]), 0.5 * (v[:, 2, 1] - v[:, 0, 1])
    J = xr * ys - xs * yr
    min_h = float(np.min(4.0 * J / e.max(1)))
    q = np.asarray(q, np.float64).reshape(4, -1)
    rho, u, w = q[0], q[1] / q[0], q[2] / q[0]
    p = (gamma - 1.0) * (q[3] - 0.5 * rho * (u * u + w * w))
    smax = float(np.max(np.hypot(u, w) + np.sqrt(np.abs(gamma * p / rho))))
    return cfl * min_h / ((order + 1) ** 2 * smax)


def headline_config(mesh, order, dt):
    """The workload the headline metric is quoted on (identical in both arms)."""
    return {"workload": "isentropic vortex, periodic 256x256x2 perturbed 10%%, N=%d (Np=%d), LF flux, LSERK4 CFL 0.5"
                        % (order, (order + 1) * (order + 2) // 2),
            "K": int(mesh.K), "order": order, "flux": "LF", "dt": float("%.12e" % dt),
            "step": "one LSERK4 time step = 5 RK stages over the whole mesh",
            "l2": "working set (q in/out + RK register) > 129 MB L2, no flush"}


def alg_bytes_per_elem_stage_fp64res(order):
    """The same minimum with an FP64 RK register and 5 FP64 metrics:
    128 Np + 96 Nfp + 124 bytes per element-stage."""
    Np = (order + 1) * (order + 2) // 2
    return 128 * Np + 96 * (order + 1) + 124


def alg_bytes_per_elem_stage(order, split=True):
    """Minimum HBM bytes one element moves per RK stage in the fused kernel:
    q read + q write (4 vars x Np x 8 B each), the RK register read + write
    (FP32 in the split path, FP64 in the FP64 path), the three neighbour face
    traces (3 x 4 x Nfp x 8 B), 4 FP64 metrics and 3 int32 neighbour words."""
    Np = (order + 1) * (order + 2) // 2
    Nfp = order + 1
    res = 4 if split else 8
    return 4 * Np * (8 + 8 + 2 * res) + 96 * Nfp + 32 + 12


# dram__bytes_read.sum + dram__bytes_write.sum of one split-stage launch at
# the headline workload (one ncu capture of euler_stage_split_pipe_kernel<5>)
SPLIT_STAGE_TRAFFIC_N5 = 220.8e6


class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if not self.samples:
            return out
        try:
            sm = [float(s[0]) for s in self.samples]
            out["sm_mhz"] = float(np.median(sm))
            out["sm_max_mhz"] = float(self.samples[0][1])
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            reasons = set()
            for s in self.samples:
                for n, v in zip(names, s[4:8]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            out["reasons"] = sorted(reasons)
            out["samples"] = len(sm)
        except Exception:
            pass
        return out


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline(mesh, order, q0, dt, threads, one_thread=True):
    """Oracle LSERK4 (one time step = 5 stages) on the full mesh with all host
    threads, and one stage on one thread; returns DOF-stage/s for both and the
    seconds each sample took."""
    from hopefoam_gb300.mesh import load_cubature
    from oracle import oracle

    oracle.set_threads(threads)
    orc = oracle.Oracle(mesh, order, load_cubature(3 * (order + 1)))
    q = q0.reshape(-1)
    t = time.perf_counter()
    orc.lserk4(q, dt, 1, flux=0)
    el = time.perf_counter() - t
    dofs = mesh.K * orc.Np * 4
    out = {"value": dofs * 5 / el, "seconds": el}
    if one_thread:
        oracle.set_threads(1)
        t = time.perf_counter()
        orc.euler_rhs(q, flux=0)
        el1 = time.perf_counter() - t
        oracle.set_threads(threads)
        out["value_1thread"] = dofs / el1
        out["seconds_1thread"] = el1
    return out


def run_reference(args):
    """The reference arm: the oracle (the reference's algorithm restated in
    C++, OpenMP over all host threads) on the headline workload, its initial
    state built at the oracle's own nodes and stepped at the same dt.  Nothing
    here loads libdgcu."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    order = args.order
    mesh = workload(args.nx, order)
    from oracle import oracle

    from hopefoam_gb300.mesh import load_cubature

    threads = oracle.max_threads()
    oracle.set_threads(threads)
    orc = oracle.Oracle(mesh, order, load_cubature(3 * (order + 1)))
    q0 = initial_state_oracle(orc)
    dt = host_cfl_dt(mesh, order, q0)
    q = q0.reshape(-1)
    res = None
    for _ in range(args.warmup):
        q, res = orc.lserk4(q, dt, 1, flux=0, res=res)
    vals = []
    for _ in range(args.steps):
        t = time.perf_counter()
        q, res = orc.lserk4(q, dt, 1, flux=0, res=res)
        vals.append(time.perf_counter() - t)
    Np = (order + 1) * (order + 2) // 2
    dofs_stage = mesh.K * Np * 4 * 5
    tot = float(np.sum(vals))
    value = dofs_stage * args.steps / tot
    # one right-hand side on one thread (a bounded sample of the same work)
    oracle.set_threads(1)
    t = time.perf_counter()
    orc.euler_rhs(q, flux=0)
    el1 = time.perf_counter() - t
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": headline_config(mesh, order, dt),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "one LSERK4 step (5 stages) over all %d elements per bench step" % mesh.K,
                             "value_1thread": mesh.K * Np * 4 / el1,
                             "sample_1thread": "one right-hand side over all %d elements on 1 thread, %.1f s"
                                               % (mesh.K, el1),
                             "build": "g++ -O3 -fopenmp (portable flags: the same source builds on x86 and Arm)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "split"])
    ap.add_argument("--nx", type=int, default=256)
    ap.add_argument("--order", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-poisson", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip timing the plain FP64 path beside the split path")
    ap.add_argument("--no-configs", action="store_true")
    ap.add_argument("--kh-steps", type=int, default=2)
    ap.add_argument("--no-ins", action="store_true", help="skip the incompressible (Chorin) step benchmark")
    ap.add_argument("--c5-study", action="store_true", help="500-step shear-layer accuracy study (reduced size)")
    ap.add_argument("--c5-study-n", type=int, default=128)
    ap.add_argument("--c5-study-only", action="store_true", help="run only the shear-layer accuracy study and exit")
    ap.add_argument("--c5-study-cfl", type=float, default=0.5)
    ap.add_argument("--profile-target", default=None, choices=sorted(PROFILE_TARGETS),
                    help="run one workload of the line alone (the command the ncu summaries profile) and exit")
    ap.add_argument("--profile-size", default="full", choices=["full", "small"],
                    help="small: a reduced case of the same kernels for multi-pass ncu captures")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_target:
        return profile_target(args.profile_target, args.profile_size == "small")
    if args.c5_study_only:
        import torch

        torch.cuda.set_device(0)
        print(json.dumps({"c5_study": c5_study(n=args.c5_study_n, cfl=args.c5_study_cfl)}))
        return

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300 import euler

    order = args.order
    mesh = workload(args.nx, order)
    q0, x, y = initial_state(mesh, order)
    dt = host_cfl_dt(mesh, order, q0)
    ctx = euler.EulerContext(mesh, order)
    ctx.upload(q0)
    prec_name = args.precision
    if prec_name == "auto":
        prec_name = "split" if _split_ready(ctx) else "fp64"
    prec = L.DG_PREC_SPLIT if prec_name == "split" else L.DG_PREC_FP64
    stream = torch.cuda.ExternalStream(ctx.stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # device-resident timing
    for _ in range(args.warmup):
        ctx.lserk4(dt, 1, flux=L.DG_FLUX_LF, precision=prec)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler()
    clocks.start()
    time.sleep(0.3)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    ctx.lserk4(dt, args.steps, flux=L.DG_FLUX_LF, precision=prec)
    ev1.record(stream)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1)
    ck = clocks.stop()
    torch.cuda.synchronize()
    barrier()
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    Np = ctx.Np
    dof_stage = mesh.K * Np * 4 * 5 * args.steps
    value = dof_stage * world / (ms * 1e-3)
    launches = 5 * args.steps
    per_launch_s = ms * 1e-3 / launches
    bpe = alg_bytes_per_elem_stage(order, split=(prec_name == "split"))
    bpe_survey = alg_bytes_per_elem_stage_fp64res(order)
    achieved = bpe * mesh.K / per_launch_s / 1e9
    peak, peak_kind = peaks()
    qfin = ctx.download()
    finite = bool(np.isfinite(qfin).all())

    # the plain FP64 path on the same workload (same dt, same state)
    fp64 = None
    if prec_name == "split" and not args.no_fp64:
        ctx.upload(q0)
        ctx.lserk4(dt, 1, flux=L.DG_FLUX_LF, precision=L.DG_PREC_FP64)  # warm-up
        ctx.upload(q0)
        n64 = max(2, min(args.steps, 4))
        ms64 = _timed_lserk4(ctx, dt, n64, L.DG_FLUX_LF, L.DG_PREC_FP64)
        fp64 = {"value": mesh.K * Np * 4 * 5 * n64 / (ms64 * 1e-3), "unit": UNIT, "ms_per_step": ms64 / n64,
                "steps": n64, "split_speedup": (ms64 / n64) / (ms / args.steps)}

    # precision of the timed path against the FP64 path (itself equal to the
    # oracle to 1e-12, tests/test_euler_gpu.py) from the benchmark state: the
    # right-hand side, and the state after one LSERK4 step
    precision_check = None
    if prec_name == "split":
        ctx.upload(qfin)
        r64 = ctx.rhs(flux=L.DG_FLUX_LF, precision=L.DG_PREC_FP64)
        rsp = ctx.rhs(flux=L.DG_FLUX_LF, precision=L.DG_PREC_SPLIT)
        ctx.lserk4(dt, 1, flux=L.DG_FLUX_LF, precision=L.DG_PREC_FP64)
        q64 = ctx.download()
        ctx.upload(qfin)
        ctx.lserk4(dt, 1, flux=L.DG_FLUX_LF, precision=prec)
        qsp = ctx.download()
        d = (qsp - q64).reshape(4, -1)
        r64v = q64.reshape(4, -1)
        dr = rsp - r64
        precision_check = {
            "against": "FP64 GPU path from the benchmark state after the timed steps",
            "rhs_rel_l2": float(np.linalg.norm(dr) / np.linalg.norm(r64)),
            "rhs_rel_linf": float(np.abs(dr).max() / np.abs(r64).max()),
            "step_rel_l2": float(np.linalg.norm(d) / np.linalg.norm(r64v)),
            "step_rel_linf": float(np.abs(d).max() / np.abs(r64v).max()),
            "step_rel_l2_per_variable": [float(np.linalg.norm(d[v]) / np.linalg.norm(r64v[v])) for v in range(4)],
            "reading": "the 1e-9 target is met by the state after one step (step_rel_l2); the right-hand side "
                       "itself carries FP32 flux round-off times the volume/surface cancellation (rhs_rel_l2)"}

    # end to end through the public API with pinned host buffers
    n = 4 * mesh.K * Np
    hin = torch.from_numpy(q0.reshape(-1).copy()).pin_memory()
    hout = torch.empty(n, dtype=torch.float64).pin_memory()
    import ctypes

    lib = L.lib()

    def e2e_step():
        lib.dg_upload_state(ctx.h, ctypes.cast(hin.data_ptr(), L._dp))
        ctx.lserk4(dt, 1, flux=L.DG_FLUX_LF, precision=prec)
        lib.dg_download_state(ctx.h, ctypes.cast(hout.data_ptr(), L._dp))

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    e2e_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_value = mesh.K * Np * 4 * 5 * e2e_steps * world / e2e_s

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec_name == "fp64" else "tf32x3+f32acc, f64 state", "data": "synthetic",
        "config": headline_config(mesh, order, dt),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": SPLIT_STAGE_TRAFFIC_N5 if (prec_name == "split" and order == 5 and args.nx == 256)
                     else None, "peak_kind": peak_kind, "bytes_per_elem_stage": bpe,
                     "frac_at_fp64_register_bytes": bpe_survey * mesh.K / per_launch_s / 1e9 / peak,
                     "kernel": ("euler_stage_split_pipe_kernel<%d>" % order if prec_name == "split" and order <= 6
                                else "euler_stage_%s_kernel<%d>" % (prec_name, order))},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8},
        "gpu_launches": launches,
        "clocks": ck,
        "state_finite": finite,
        "precision": prec_name,
        "precision_check": precision_check,
        "fp64": fp64,
    }
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle

        threads = oracle.max_threads()
        cb = cpu_baseline(mesh, order, q0, dt, threads)
        line["cpu_baseline"] = {"value": cb["value"], "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "one LSERK4 step (5 stages) over all %d elements, %.1f s"
                                          % (mesh.K, cb["seconds"]),
                                "value_1thread": cb.get("value_1thread"),
                                "sample_1thread": "one right-hand side over all %d elements on 1 thread, %.1f s"
                                                  % (mesh.K, cb.get("seconds_1thread", 0.0))}
    ctx.close()
    if rank == 0 and not args.no_poisson:
        try:
            line["poisson"] = poisson_bench(with_cpu=not args.no_cpu_baseline)
        except Exception as exc:  # reported, never hides the Euler line
            line["poisson"] = {"error": str(exc)}
    if rank == 0 and not args.no_configs:
        for key, fn in (("c1", c1_bench), ("c5", c5_bench)):
            try:
                line[key] = fn(with_oracle=not args.no_cpu_baseline) if key == "c1" else fn(nsteps=args.kh_steps)
            except Exception as exc:
                line[key] = {"error": str(exc)}
    if rank == 0 and not args.no_configs:
        try:
            line["shock"] = shock_bench(with_cpu=not args.no_cpu_baseline)
        except Exception as exc:
            line["shock"] = {"error": str(exc)}
    if rank == 0 and not args.no_ins:
        try:
            line["ins"] = ins_bench(with_cpu=not args.no_cpu_baseline)
        except Exception as exc:
            line["ins"] = {"error": str(exc)}
        try:
            line["cylinder"] = cylinder_bench(with_cpu=not args.no_cpu_baseline)
        except Exception as exc:
            line["cylinder"] = {"error": str(exc)}
    if rank == 0 and args.c5_study:
        try:
            line["c5_study"] = c5_study(n=args.c5_study_n)
        except Exception as exc:
            line["c5_study"] = {"error": str(exc)}
    if rank == 0 and not args.no_batch:
        try:
            line["batched"] = batch_bench(prec)
        except Exception as exc:
            line["batched"] = {"error": str(exc)}
    if rank == 0:
        line["summary"] = summary(line)  # last key: the end of the line is what a log tail shows
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def summary(line):
    """A compact digest of every workload of the line (3 significant digits)."""
    def g(d, *path):
        for p in path:
            if not isinstance(d, dict) or p not in d:
                return None
            d = d[p]
        if isinstance(d, float):
            return float("%.3g" % d)
        return d

    out = {"headline": {"value": g(line, "value"), "e2e": g(line, "e2e", "value"), "frac": g(line, "roofline", "frac"),
                        "ms_per_step": g(line, "ms_per_step"), "cpu": g(line, "cpu_baseline", "value"),
                        "cpu_1thread": g(line, "cpu_baseline", "value_1thread")},
           "fp64_path": {"value": g(line, "fp64", "value"), "split_speedup": g(line, "fp64", "split_speedup")},
           "split_vs_fp64": {k: g(line, "precision_check", k) for k in ("rhs_rel_l2", "rhs_rel_linf", "step_rel_l2",
                                                                           "step_rel_linf")}}
    p = line.get("poisson")
    if isinstance(p, dict):
        out["poisson_ms"] = {"block_jacobi": g(p, "bj_mixed", "ms"), "bj_iters": g(p, "bj_mixed", "iterations"),
                             "bj_frac": g(p, "bj_mixed", "roofline", "frac"),
                             "multilevel": g(p, "multilevel_mixed", "ms"),
                             "ml_iters": g(p, "multilevel_mixed", "iterations"),
                             "learned": g(p, "learned", "ms"), "learned_iters": g(p, "learned", "iterations"),
                             "learned_vs_bj": g(p, "learned", "speedup_vs_block_jacobi"),
                             "learned_multilevel": g(p, "learned_multilevel", "ms"),
                             "cpu": g(p, "cpu_baseline", "ms")}
    for k in ("c1", "c5", "batched", "shock", "ins", "cylinder"):
        d = line.get(k)
        if not isinstance(d, dict):
            continue
        if "error" in d:
            out[k] = {"error": str(d["error"])[:120]}
            continue
        out[k] = {kk: g(d, *pp) for kk, pp in {
            "c1": {"value": ("value",), "rho_err_l2": ("rho_err_l2",), "state_vs_oracle": ("state_vs_oracle",)},
            "c5": {"split_ms": ("split", "ms_per_step"), "fp64_ms": ("fp64", "ms_per_step"),
                   "speedup": ("split_speedup_vs_fp64",), "frac": ("split", "roofline", "frac"),
                   "step_l2": ("split_step_error", "rel_l2")},
            "batched": {"value": ("value",), "frac": ("roofline", "frac"), "ms": ("ms",)},
            "shock": {"fp64_ms": ("fp64", "ms_per_step"), "split_ms": ("split", "ms_per_step"),
                      "cpu_ms": ("cpu_baseline", "ms_per_step")},
            "ins": {"ms": ("ms_per_step",), "mixed_ms": ("mixed_solves", "ms_per_step"),
                    "cpu_ms": ("cpu_baseline", "ms_per_step")},
            "cylinder": {"ms": ("ms_per_step",), "cpu_ms": ("cpu_baseline", "ms_per_step"),
                         "vs_oracle": ("state_vs_oracle",)}}[k].items()}
    return out


def c1_bench(nsteps=100, order=3, with_oracle=True):
    """The reference's CPU-sized case: isentropic vortex on the periodic
    40x40x2 mesh of [0,10]^2 (K = 3200), N = 3, LF flux, LSERK4 at CFL 0.5,
    100 steps on the FP64 path; L2 / Linf errors of density against the exact
    advected vortex, and the throughput (the working set fits in L2: a latency
    case, not a roofline case)."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300 import euler
    from hopefoam_gb300.mesh import periodic_square

    mesh = periodic_square(40, 40, 10.0, 10.0)
    ops = euler.reference_operators(order)
    x, y = euler.node_coords(mesh, ops["r"], ops["s"])
    q0 = euler.isentropic_vortex(x, y, x0=5.0, y0=5.0)
    ctx = euler.EulerContext(mesh, order)
    ctx.upload(q0)
    dt = ctx.cfl_dt(0.5)
    ctx.lserk4(dt, 1, flux=L.DG_FLUX_LF, precision=L.DG_PREC_FP64)
    ctx.upload(q0)
    import torch

    stream = torch.cuda.ExternalStream(ctx.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.lserk4(dt, nsteps, flux=L.DG_FLUX_LF, precision=L.DG_PREC_FP64)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    q = ctx.download()
    ex = euler.isentropic_vortex(x, y, t=nsteps * dt, x0=5.0, y0=5.0)
    d = q[0] - ex[0]
    ctx.close()
    out = {"workload": "isentropic vortex, periodic 40x40x2 (K=3200), N=3, LF, LSERK4 CFL 0.5, %d steps, FP64"
                       % nsteps, "dt": dt, "t": nsteps * dt,
           "rho_err_l2": float(np.linalg.norm(d) / np.linalg.norm(ex[0])), "rho_err_linf": float(np.abs(d).max()),
           "value": mesh.K * ops["r"].size * 4 * 5 * nsteps / (ms * 1e-3), "unit": UNIT, "ms": ms}
    if with_oracle:
        # the same 100 steps on the oracle: FP64 state parity at the configured size
        from hopefoam_gb300.mesh import load_cubature
        from oracle import oracle

        orc = oracle.Oracle(mesh, order, load_cubature(3 * (order + 1)))
        t0 = time.perf_counter()
        qo, _ = orc.lserk4(q0.reshape(-1), dt, nsteps, flux=0)
        out["oracle_s"] = time.perf_counter() - t0
        out["state_vs_oracle"] = float(np.linalg.norm(q.reshape(-1) - qo) / np.linalg.norm(qo))
    return out


def _kh_context(n, order):
    from hopefoam_gb300 import euler
    from hopefoam_gb300.mesh import periodic_square

    mesh = periodic_square(n, n, 1.0, 1.0)
    ops = euler.reference_operators(order)
    x, y = euler.node_coords(mesh, ops["r"], ops["s"])
    q0 = euler.kelvin_helmholtz(x, y, seed=0)
    return mesh, q0


def _timed_lserk4(ctx, dt, nsteps, flux, prec):
    import torch

    stream = torch.cuda.ExternalStream(ctx.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.lserk4(dt, nsteps, flux=flux, precision=prec)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def c5_bench(nsteps=None, order=7, n=708):
    """Large shear layer: periodic [0,1]^2, 708x708x2 = 1,002,528 triangles,
    N = 7 (Np = 36), Kelvin-Helmholtz initial state, Roe flux, LSERK4 at CFL
    0.5; the FP64 path and the split path (streamed-operator kernel) each
    timed over a few steps from the initial state, and the split path's
    one-step state error against the FP64 path from the same state.  The
    500-step accuracy study is c5_study (--c5-study)."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300 import euler

    nsteps = nsteps or 2
    t0 = time.perf_counter()
    mesh, q0 = _kh_context(n, order)
    ctx = euler.EulerContext(mesh, order)
    ctx.upload(q0)
    dt = ctx.cfl_dt(0.5)
    setup_s = time.perf_counter() - t0
    K, Np = mesh.K, ctx.Np
    out = {"workload": "Kelvin-Helmholtz, periodic 708x708x2 (K=%d), N=7, Roe, LSERK4 CFL 0.5" % K,
           "steps": nsteps, "setup_s": setup_s, "dt": dt, "unit": UNIT}
    peak, peak_kind = peaks()
    for name, prec in (("fp64", L.DG_PREC_FP64), ("split", L.DG_PREC_SPLIT)):
        ctx.upload(q0)
        ctx.lserk4(dt, 1, flux=L.DG_FLUX_ROE, precision=prec)  # warm-up
        ctx.upload(q0)
        ms = _timed_lserk4(ctx, dt, nsteps, L.DG_FLUX_ROE, prec)
        bpe = alg_bytes_per_elem_stage(order, split=(name == "split"))
        out[name] = {"ms_per_step": ms / nsteps, "value": K * Np * 4 * 5 * nsteps / (ms * 1e-3),
                     "roofline": {"achieved": bpe * K * 5 * nsteps / (ms * 1e-3) / 1e9, "peak": peak,
                                  "unit": "GB/s", "peak_kind": peak_kind, "bytes_per_elem_stage": bpe}}
        out[name]["roofline"]["frac"] = out[name]["roofline"]["achieved"] / peak
        out[name]["state_finite"] = bool(np.isfinite(ctx.download()).all())
    out["split_speedup_vs_fp64"] = out["fp64"]["ms_per_step"] / out["split"]["ms_per_step"]
    ctx.upload(q0)
    ctx.lserk4(dt, 1, flux=L.DG_FLUX_ROE, precision=L.DG_PREC_FP64)
    q64 = ctx.download()
    ctx.upload(q0)
    ctx.lserk4(dt, 1, flux=L.DG_FLUX_ROE, precision=L.DG_PREC_SPLIT)
    qsp = ctx.download()
    ctx.close()
    d = qsp - q64
    out["split_step_error"] = {"against": "FP64 path, one LSERK4 step from the initial state",
                               "rel_l2": float(np.linalg.norm(d) / np.linalg.norm(q64)),
                               "rel_linf": float(np.abs(d).max() / np.abs(q64).max())}
    out["value"] = out["split"]["value"]
    out["ms_per_step"] = out["split"]["ms_per_step"]
    return out


def c5_study(order=7, n=128, checkpoints=(100, 250, 500), n_full=708, cfl=0.5):
    """The shear layer's accuracy study at reduced size (n x n x 2 elements,
    the full-size workload's setup otherwise) and at the full-size
    workload's time step (its CFL-0.5 step on the n_full grid, so that 500
    steps cover the same physical time; the unlimited scheme on the
    discontinuous initial state does not survive 500 steps at the coarse
    grid's own CFL step): the split path and the FP64 path advanced side by
    side from the same initial state; density error of the split path
    against the FP64 path (relative L2 and Linf) at each checkpoint, and
    both paths' device time."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300 import euler

    mesh, q0 = _kh_context(n, order)
    c64 = euler.EulerContext(mesh, order)
    csp = euler.EulerContext(mesh, order)
    c64.upload(q0)
    csp.upload(q0)
    dt = c64.cfl_dt(cfl) * n / n_full  # min h scales with 1/n on this grid family
    rows, done, ms64, mssp = [], 0, 0.0, 0.0
    for cp in checkpoints:
        ms64 += _timed_lserk4(c64, dt, cp - done, L.DG_FLUX_ROE, L.DG_PREC_FP64)
        mssp += _timed_lserk4(csp, dt, cp - done, L.DG_FLUX_ROE, L.DG_PREC_SPLIT)
        done = cp
        r64, rsp = c64.download()[0], csp.download()[0]
        d = rsp - r64
        rows.append({"step": cp, "t": cp * dt, "rho_rel_l2": float(np.linalg.norm(d) / np.linalg.norm(r64)),
                     "rho_rel_linf": float(np.abs(d).max() / np.abs(r64).max()),
                     "finite_fp64": bool(np.isfinite(r64).all()), "finite_split": bool(np.isfinite(rsp).all())})
    c64.close()
    csp.close()
    return {"workload": "Kelvin-Helmholtz, periodic %dx%dx2 (K=%d), N=7, Roe, LSERK4 at the %dx%dx2 grid's "
                        "CFL-%g step, %d steps" % (n, n, mesh.K, n_full, n_full, cfl, checkpoints[-1]),
            "dt": dt, "density_error_split_vs_fp64": rows, "ms_per_step_fp64": ms64 / checkpoints[-1],
            "ms_per_step_split": mssp / checkpoints[-1]}


def ins_bench(n=128, order=2, steps=4, warmup=2, with_cpu=True, cpu_steps=2):
    """Incompressible Chorin step (dg_ins_step) on the Pearson-vortex case of
    the reference's dgChorinFoam tutorial, refined: [-0.5, 0.5]^2 as n x n x 2
    triangles (K = 2 n^2) with the tutorial's inlet / outlet pattern, N = 2
    (its baseOrder), nu = 0.01, dt = 1e-3, tau = 20 (N+1)^2 fscale; solves to a
    relative residual of 1e-10.  Device time per step from CUDA events on the
    solver's stream; the CPU baseline is the oracle's step (C++ operators,
    scipy sparse LU factorised once) on the same mesh."""
    from hopefoam_gb300.ins import ChorinSolver, PearsonVortex, pearson_mesh

    mesh = pearson_mesh(n)
    g = ChorinSolver(mesh, order, nu=0.01, dt=1e-3)
    pv = PearsonVortex(g)
    g.set_state(*pv.initial_state())
    t = 0.0
    for _ in range(warmup):
        g.step(pv.bdata(t), rtol=1e-10)
        t += g.dt
    sts = []
    for _ in range(steps):
        sts.append(g.step(pv.bdata(t), rtol=1e-10))
        t += g.dt
    _, p = g.get_state()
    err = pv.pressure_error(p, t)
    ms = float(np.mean([s["ms"] for s in sts]))
    Np = g.Np
    # PCG iteration bytes (FP64 vectors x 11 passes, FP64 block inverse, geometry)
    bytes_it = mesh.K * (8 * Np * 11 + 8 * Np * Np + 136)
    its = float(np.mean([s["iterations_p"] + sum(s["iterations_u"]) for s in sts]))
    peak, peak_kind = peaks()
    out = {"workload": "Pearson vortex (dgChorinFoam tutorial case refined), %dx%dx2 (K=%d), N=%d, dt=1e-3, "
                       "nu=0.01, rtol 1e-10" % (n, n, mesh.K, order),
           "ms_per_step": ms, "steps": steps, "iterations_p": [s["iterations_p"] for s in sts],
           "iterations_u": [list(s["iterations_u"]) for s in sts], "pressure_error_avg_max": err,
           "value": mesh.K * Np * 3 / (ms * 1e-3), "unit": "DOF-steps/s (3 fields)",
           "roofline": {"bound": "hbm", "achieved": bytes_it * its / (ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": bytes_it * its / (ms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind,
                        "bytes_per_pcg_iteration": bytes_it,
                        "note": "PCG iteration bytes x iterations of the step's three solves / step time"}}
    g.close()
    # the same steps with mixed-precision linear solves (FP32 operator on FP64
    # offsets, FP64 vectors and recurrences, the same 1e-10 on the true residual)
    try:
        from hopefoam_gb300 import _lib as L

        gm = ChorinSolver(mesh, order, nu=0.01, dt=1e-3, precision=L.DG_PREC_SPLIT)
        pvm = PearsonVortex(gm)
        gm.set_state(*pvm.initial_state())
        tm = 0.0
        for _ in range(warmup):
            gm.step(pvm.bdata(tm), rtol=1e-10)
            tm += gm.dt
        stm = []
        for _ in range(steps):
            stm.append(gm.step(pvm.bdata(tm), rtol=1e-10))
            tm += gm.dt
        _, pm = gm.get_state()
        out["mixed_solves"] = {"ms_per_step": float(np.mean([s["ms"] for s in stm])),
                               "pressure_error_avg_max": pvm.pressure_error(pm, tm),
                               "iterations_p": [s["iterations_p"] for s in stm]}
        gm.close()
    except Exception as exc:
        out["mixed_solves"] = {"error": str(exc)}
    if with_cpu:
        from hopefoam_gb300.mesh import load_cubature
        from oracle import oracle
        from oracle.ins_oracle import ChorinOracle

        threads = oracle.max_threads()
        t0 = time.perf_counter()
        o = ChorinOracle(mesh, order, load_cubature(3 * (order + 1)), nu=0.01, dt=1e-3)
        setup = time.perf_counter() - t0
        o.step()  # first step (BDF1) factorises its Helmholtz operator
        t0 = time.perf_counter()
        for _ in range(cpu_steps):
            o.step()
        el = (time.perf_counter() - t0) / cpu_steps
        out["cpu_baseline"] = {"value": mesh.K * Np * 3 / el, "unit": out["unit"], "cores": threads, "kind": "port",
                               "ms_per_step": el * 1e3, "setup_s": setup,
                               "sample": "%d oracle steps on the same mesh (sparse LU factorised at setup)" % cpu_steps}
    return out


def shock_bench(steps=200, warmup=5, with_cpu=True, cpu_steps=3):
    """The reference's double-Mach-reflection tutorial (5390 triangles, N = 4,
    Roe flux, dt = 1e-5, limited SSP-RK2 with reflective wall and the moving
    shock's boundary values): device ms per step through
    dg_limited_ssprk2_step (the boundary data are host arrays uploaded each
    step, as the reference sets them each step), FP64 and split precision;
    CPU baseline: the oracle's limited step on the same state."""
    import ctypes

    import torch

    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300 import euler
    from hopefoam_gb300.mesh import Mesh, connect
    from hopefoam_gb300.shock import DoubleMach

    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "doublemach.npz"))
    EToE, EToF, ROT, BC = connect(d["EToV"])
    mesh = Mesh(d["EToV"], d["VXY"], EToE, EToF, ROT, BC, name="doubleMach", patch=d["patch"],
                patch_names=tuple(str(x) for x in d["patch_names"]))
    mesh.patch_first_face = d["patch_first_face"]
    N, dt = 4, 1e-5
    dm = DoubleMach(mesh, N)
    out = {"workload": "double Mach reflection (tutorial mesh, K=%d), N=%d, Roe, dt=1e-5, limited SSP-RK2" % (mesh.K, N)}
    for name, prec in (("fp64", L.DG_PREC_FP64), ("split", L.DG_PREC_SPLIT)):
        ctx = euler.EulerContext(mesh, N)
        ctx.upload(dm.initial_state())
        ctx.set_boundary_traces(dm.bdata(0.0))
        ctx.set_boundary_kinds(dm.kinds, dm.gref)
        t = 0.0
        bd = [np.ascontiguousarray(dm.bdata(t + i * dt)) for i in range(warmup + steps)]
        for i in range(warmup):
            ctx.limited_ssprk2(dt, bd[i], precision=prec)
        stream = torch.cuda.ExternalStream(ctx.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(steps):
            ctx.limited_ssprk2(dt, bd[warmup + i], precision=prec)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        q = ctx.download()
        out[name] = {"ms_per_step": ms, "value": mesh.K * ctx.Np * 4 * 2 / (ms * 1e-3), "unit": "DOF-stage/s",
                     "state_finite": bool(np.isfinite(q).all()), "rho_min_max": [float(q[0].min()), float(q[0].max())]}
        ctx.close()
    if with_cpu:
        from hopefoam_gb300.mesh import load_cubature
        from oracle import oracle
        from oracle.limited_oracle import LimitedSSPOracle

        lo = LimitedSSPOracle(mesh, N, load_cubature(3 * (N + 1)), dm.kinds, dm.gref)
        q = dm.initial_state()
        q = lo.step(q, dt, dm.bdata(0.0))
        t0 = time.perf_counter()
        for i in range(cpu_steps):
            q = lo.step(q, dt, dm.bdata((i + 1) * dt))
        el = (time.perf_counter() - t0) / cpu_steps
        out["cpu_baseline"] = {"ms_per_step": el * 1e3, "kind": "port", "cores": oracle.max_threads(),
                               "sample": "%d oracle limited steps on the same mesh" % cpu_steps}
    return out


def cylinder_bench(steps=100, warmup=5, with_cpu=True, cpu_steps=3):
    """The reference's cylinder tutorial as it stands (tutorials/DG/2D/cylinder:
    its polyMesh of 1840 triangles with the two arc patches of the cylinder,
    order 3, nu = 0.001, dt = 2e-4, time-varying inflow): device ms per Chorin
    step through dg_ins_step (PCG to a relative residual of 1e-10, about the
    FP64 floor of this case's pressure systems) and the oracle's step (sparse
    LU, the reference's preonly + LU) on the same case; after the timed steps,
    the state is compared with the oracle run for the same number of steps."""
    from hopefoam_gb300.curved import ArcCurve
    from hopefoam_gb300.ins import ChorinSolver, CylinderFlow
    from hopefoam_gb300.mesh import Mesh, connect

    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "cylinder.npz"))
    EToE, EToF, ROT, BC = connect(d["EToV"])
    mesh = Mesh(d["EToV"], d["VXY"], EToE, EToF, ROT, BC, name="cylinder", patch=d["patch"],
                patch_names=tuple(str(x) for x in d["patch_names"]))
    mesh.curves = {str(n): ArcCurve.from_code(str(c), tuple(u), name=str(n))
                   for n, c, u in zip(d["arc_names"], d["arc_codes"], d["arc_u_range"])}
    N, nu, dt = CylinderFlow.ORDER, CylinderFlow.NU, CylinderFlow.DT
    uk, pk = CylinderFlow.kinds(mesh)
    g = ChorinSolver(mesh, N, nu=nu, dt=dt, u_kind=uk, p_kind=pk)
    cf = CylinderFlow(g)
    g.set_state(*cf.initial_state())
    t = 0.0
    sts = []
    for i in range(warmup + steps):
        st = g.step(cf.bdata(t), rtol=1e-10)
        if i >= warmup:
            sts.append(st)
        t += dt
    U, p = g.get_state()
    ms = float(np.mean([s["ms"] for s in sts]))
    out = {"workload": "cylinder tutorial (polyMesh K=%d, arc patches), N=%d, nu=%g, dt=%g, rtol 1e-10"
                       % (mesh.K, N, nu, dt),
           "ms_per_step": ms, "steps": steps, "value": mesh.K * g.Np * 3 / (ms * 1e-3),
           "unit": "DOF-steps/s (3 fields)",
           "iterations_p_u": [sts[-1]["iterations_p"], list(sts[-1]["iterations_u"])],
           "max_speed": float(np.hypot(U[0], U[1]).max())}
    g.close()
    if with_cpu:
        from hopefoam_gb300.mesh import load_cubature
        from oracle import oracle
        from oracle.ins_oracle import ChorinOracle, CylinderCase

        o = ChorinOracle(mesh, N, load_cubature(3 * (N + 1)), nu=nu, dt=dt, case=CylinderCase(nu, dt))
        o.step()  # first step (BDF1) factorises its Helmholtz operator
        t0 = time.perf_counter()
        for _ in range(cpu_steps):
            o.step()
        el = (time.perf_counter() - t0) / cpu_steps
        out["cpu_baseline"] = {"ms_per_step": el * 1e3, "kind": "port", "cores": oracle.max_threads(),
                               "sample": "%d oracle steps on the same case (sparse LU at setup)" % cpu_steps}
        for _ in range(warmup + steps - 1 - cpu_steps):
            o.step()
        out["state_vs_oracle"] = float(max(np.linalg.norm(U - o.U) / np.linalg.norm(o.U),
                                           np.linalg.norm(p - o.p) / max(np.linalg.norm(o.p), 1e-300)))
    return out


def batch_bench(prec, n_cases=512, nsteps=100):
    """Batched workload: 512 seeded isentropic-vortex cases (strength U(1,6),
    Mach U(0.1,0.8), N uniform in 2..6, K log-uniform in [800, 20000] as
    m x m x 2 perturbed periodic grids), each at its own CFL-0.5 step, all
    advanced nsteps LSERK4 steps in one CUDA-graph launch after autotuning."""
    from hopefoam_gb300.batch import EulerBatch, batch_cases

    t0 = time.perf_counter()
    cases = batch_cases(n_cases, seed=0)
    b = EulerBatch(cases)
    setup_s = time.perf_counter() - t0
    tune = b.tune(precision=prec, steps_per_trial=2)
    b.run(nsteps, precision=prec)  # capture + warm-up launch
    ms = b.run(nsteps, precision=prec)  # graph replay, device time
    dof_stage = b.dofs * 5 * nsteps
    bytes_stage = sum(g["ctx"].K * alg_bytes_per_elem_stage(g["order"], split=True) for g in b.groups)
    peak, peak_kind = peaks()
    finite = all(bool(np.isfinite(q).all()) for q in b.states())
    out = {"workload": "%d isentropic-vortex cases, N in 2..6, K in [800,20000] log-uniform, %d LSERK4 steps, "
                       "one CUDA-graph launch" % (n_cases, nsteps),
           "elements": b.elements, "dofs": b.dofs, "value": dof_stage / (ms * 1e-3), "unit": UNIT,
           "ms": ms, "setup_s": setup_s, "tuning": tune, "state_finite": finite,
           "roofline": {"bound": "hbm", "achieved": bytes_stage * 5 * nsteps / (ms * 1e-3) / 1e9, "peak": peak,
                        "unit": "GB/s", "peak_kind": peak_kind},
           "groups": [{"order": g["order"], "cases": len(g["cases"]), "K": g["ctx"].K} for g in b.groups]}
    out["roofline"]["frac"] = out["roofline"]["achieved"] / peak
    b.close()
    return out


def poisson_bench(with_cpu, n_interior=50000, order=4, tau_coef=1.0, rtol=1e-10):
    """Pressure-Poisson workload: SIPG (tau = (N+1)^2 / h, i.e. tau_coef 1 with
    h = J/sJ) on a seeded ~100k-triangle Delaunay mesh of [0, 2pi]^2, N = 4,
    Dirichlet boundary, Taylor-Green + random Fourier RHS; wall ms of the
    block-Jacobi PCG to 1e-10 (true FP64 residual), mixed-precision and
    plain-FP64 arithmetic, and the learned preconditioner when one is loaded."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.mesh import delaunay_square
    from hopefoam_gb300.poisson import PressureSolver, poisson_rhs

    mesh = delaunay_square(n_interior, seed=0)
    ps = PressureSolver(mesh, order, tau_coef=tau_coef)
    b, _ = poisson_rhs(mesh, order, seed=1)
    out = {"workload": "SIPG N=%d, Delaunay [0,2pi]^2 K=%d, tau=(N+1)^2/h, Dirichlet, TG+Fourier(k<=16) rhs"
                       % (order, mesh.K), "rtol": rtol}
    ps.solve(b, rtol=1e-4, precision=L.DG_PREC_SPLIT, raise_on_fail=False)  # warm-up
    x, st = ps.solve(b, rtol=rtol, precision=L.DG_PREC_SPLIT, raise_on_fail=False)
    out["bj_mixed"] = {"ms": st["ms"], "iterations": st["iterations"], "rel_residual": st["rel_residual"]}
    x, st64 = ps.solve(b, rtol=rtol, precision=L.DG_PREC_FP64, maxit=20000, raise_on_fail=False)
    out["bj_fp64"] = {"ms": st64["ms"], "iterations": st64["iterations"], "rel_residual": st64["rel_residual"]}
    # algorithmic bytes per iteration (FP64 vectors x 11 passes, FP32 block inverse)
    Np = ps.Np
    bytes_it = mesh.K * (8 * Np * 11 + 4 * Np * Np + 136)
    if st["iterations"]:
        per_it = st["ms"] * 1e-3 / st["iterations"]
        peak, peak_kind = peaks()
        out["bj_mixed"]["roofline"] = {"bound": "hbm", "achieved": bytes_it / per_it / 1e9, "peak": peak,
                                       "unit": "GB/s", "frac": bytes_it / per_it / 1e9 / peak,
                                       "bytes_per_iteration": bytes_it, "peak_kind": peak_kind}
    # multilevel coarse-space preconditioner (block Jacobi + P1 Galerkin
    # coarse space with an aggregation V-cycle); the first solve includes its
    # host construction, the timed ones reuse it
    try:
        t0 = time.perf_counter()
        ps.solve(b, rtol=1e-4, pc=L.DG_PC_MULTILEVEL, precision=L.DG_PREC_SPLIT, raise_on_fail=False)
        setup_s = time.perf_counter() - t0
        _, stm = ps.solve(b, rtol=rtol, pc=L.DG_PC_MULTILEVEL, precision=L.DG_PREC_SPLIT, raise_on_fail=False)
        _, stm64 = ps.solve(b, rtol=rtol, pc=L.DG_PC_MULTILEVEL, precision=L.DG_PREC_FP64, raise_on_fail=False)
        out["multilevel_mixed"] = {"ms": stm["ms"], "iterations": stm["iterations"],
                                   "rel_residual": stm["rel_residual"], "first_solve_with_setup_s": setup_s,
                                   "speedup_vs_block_jacobi": st["ms"] / stm["ms"] if stm["ms"] else None}
        out["multilevel_fp64"] = {"ms": stm64["ms"], "iterations": stm64["iterations"],
                                  "rel_residual": stm64["rel_residual"]}
    except Exception as exc:
        out["multilevel_mixed"] = {"error": str(exc)}
    # learned preconditioner: trained on a small mesh from the solver's own
    # residuals, transferred, then the learned solve alone and with its
    # block-Jacobi fallback
    try:
        from hopefoam_gb300.poisson import train_learned_preconditioner

        W1, W2, info = train_learned_preconditioner(order, tau_coef=tau_coef)
        ps.lpc_setup(hidden=info["hidden"], seed=0, capacity=0, form=info["form"])
        ps.lpc_set_weights(W1, W2)
        _, stl = ps.solve(b, rtol=rtol, maxit=20000, pc=L.DG_PC_LEARNED_ONLY, precision=L.DG_PREC_SPLIT,
                          raise_on_fail=False)
        _, stf = ps.solve(b, rtol=rtol, maxit=20000, pc=L.DG_PC_LEARNED, precision=L.DG_PREC_SPLIT,
                          raise_on_fail=False)
        out["learned"] = {"training": info, "ms": stf["ms"], "iterations": stf["iterations"],
                          "rel_residual": stf["rel_residual"],
                          "learned_only": {"ms": stl["ms"], "iterations": stl["iterations"],
                                           "rel_residual": stl["rel_residual"], "converged": stl["status"] == L.DG_OK},
                          "speedup_vs_block_jacobi": st["ms"] / stf["ms"] if stf["ms"] else None,
                          "note": "negative iterations: the learned solve stalled and block Jacobi finished it"}
        # the learned local preconditioner in place of block Jacobi under the coarse-space
        # correction, trained for that combination (its loss includes the coarse correction)
        Wc, _, infoc = train_learned_preconditioner(order, tau_coef=tau_coef, coarse=True)
        ps.lpc_set_weights(Wc)
        ps.solve(b, rtol=rtol, maxit=20000, pc=L.DG_PC_LEARNED_MULTILEVEL, precision=L.DG_PREC_SPLIT)  # warm-up
        _, stlm = ps.solve(b, rtol=rtol, maxit=20000, pc=L.DG_PC_LEARNED_MULTILEVEL, precision=L.DG_PREC_SPLIT)
        out["learned_multilevel"] = {"ms": stlm["ms"], "iterations": stlm["iterations"],
                                     "rel_residual": stlm["rel_residual"], "training": infoc,
                                     "speedup_vs_block_jacobi": st["ms"] / stlm["ms"] if stlm["ms"] else None}
    except Exception as exc:
        out["learned"] = out.get("learned", {"error": str(exc)})
        out["learned_multilevel"] = {"error": str(exc)}
    # the two-layer network of width 128 (tied weights, relu, BF16 tensor-core
    # training and inference kernels) in the same Schwarz form, flexible PCG
    try:
        out["learned_mlp"] = learned_mlp_solve(mesh, order, b, tau_coef, rtol, st["ms"])
    except Exception as exc:
        out["learned_mlp"] = {"error": str(exc)}
    if with_cpu:
        from hopefoam_gb300.mesh import load_cubature
        from oracle import oracle

        orc = oracle.Oracle(mesh, order, load_cubature(3 * (order + 1)))
        diag, off, _ = orc.ipdg_blocks(tau_coef=tau_coef)
        t = time.perf_counter()
        _, it, _ = orc.pcg_bj(diag, off, b, rtol=1e-30, maxit=20)
        per = (time.perf_counter() - t) / max(it, 1)
        out["cpu_baseline"] = {"ms": per * 1e3 * st64["iterations"] if st64["iterations"] else None,
                               "kind": "port", "cores": oracle.max_threads(),
                               "sample": "20 oracle block-Jacobi CG iterations on the same system, scaled to the FP64 "
                                         "iteration count"}
    ps.ctx.close()
    return out


def learned_mlp_solve(mesh, order, b, tau_coef, rtol, ms_block_jacobi):
    """Trains the two-layer Schwarz form on a small mesh, transfers it, and
    solves S x = b with it (learned alone, then with the block-Jacobi
    fallback)."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.poisson import PressureSolver, train_learned_preconditioner

    W, _, info = train_learned_preconditioner(order, tau_coef=tau_coef, form="mlp", hidden=128)
    ps = PressureSolver(mesh, order, tau_coef=tau_coef)
    try:
        ps.lpc_setup(hidden=128, seed=0, capacity=0, form="mlp")
        ps.lpc_set_weights(W)
        _, stl = ps.solve(b, rtol=rtol, maxit=20000, pc=L.DG_PC_LEARNED_ONLY, precision=L.DG_PREC_SPLIT,
                          raise_on_fail=False)
        _, stf = ps.solve(b, rtol=rtol, maxit=20000, pc=L.DG_PC_LEARNED, precision=L.DG_PREC_SPLIT,
                          raise_on_fail=False)
    finally:
        ps.ctx.close()
    return {"training": info, "ms": stf["ms"], "iterations": stf["iterations"], "rel_residual": stf["rel_residual"],
            "learned_only": {"ms": stl["ms"], "iterations": stl["iterations"], "rel_residual": stl["rel_residual"],
                             "converged": stl["status"] == L.DG_OK},
            "speedup_vs_block_jacobi": ms_block_jacobi / stf["ms"] if stf["ms"] else None}


def _prof_pcg(small, pcs=("bj",)):
    """The pressure system of the Poisson workload (Delaunay [0,2pi]^2, N = 4,
    tau = (N+1)^2/h): a warm-up solve, then 64 iterations of each requested
    preconditioner in mixed precision (block Jacobi also in FP64)."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.mesh import delaunay_square
    from hopefoam_gb300.poisson import PressureSolver, poisson_rhs

    mesh = delaunay_square(12000 if small else 50000, seed=0)
    ps = PressureSolver(mesh, 4, tau_coef=1.0)
    b, _ = poisson_rhs(mesh, 4, seed=1)
    out = {"K": mesh.K}
    warm = L.DG_PC_MULTILEVEL if pcs[0] == "multilevel" else L.DG_PC_BLOCK_JACOBI
    ps.solve(b, rtol=1e-4, pc=warm, precision=L.DG_PREC_SPLIT, raise_on_fail=False)  # warm-up (and setup)
    for name in pcs:
        if name == "bj":
            for pn, prec in (("bj_mixed", L.DG_PREC_SPLIT), ("bj_fp64", L.DG_PREC_FP64)):
                _, st = ps.solve(b, rtol=1e-30, maxit=64, precision=prec, raise_on_fail=False)
                out[pn] = {"iterations": st["iterations"], "ms": st["ms"]}
        elif name == "multilevel":
            _, st = ps.solve(b, rtol=1e-10, pc=L.DG_PC_MULTILEVEL, precision=L.DG_PREC_SPLIT, raise_on_fail=False)
            out["multilevel"] = {"iterations": st["iterations"], "ms": st["ms"]}
    ps.ctx.close()
    return out


def profile_target(name, small=False):
    """One workload of the bench line on its own, for the ncu summaries (each
    summary names the command it ran).  Prints one JSON line."""
    import torch

    torch.cuda.set_device(0)
    from hopefoam_gb300 import _lib as L

    out = {"profile_target": name, "size": "small" if small else "full"}
    if name == "pcg":
        out.update(_prof_pcg(small))
    elif name == "multilevel":
        out.update(_prof_pcg(small, pcs=("multilevel",)))
    elif name == "learned":
        from hopefoam_gb300.mesh import delaunay_square
        from hopefoam_gb300.poisson import PressureSolver, poisson_rhs, train_learned_preconditioner

        W1, W2, info = train_learned_preconditioner(4, tau_coef=1.0)
        mesh = delaunay_square(12000 if small else 50000, seed=0)
        ps = PressureSolver(mesh, 4, tau_coef=1.0)
        ps.lpc_setup(hidden=info["hidden"], seed=0, capacity=0, form=info["form"])
        ps.lpc_set_weights(W1, W2)
        b, _ = poisson_rhs(mesh, 4, seed=1)
        _, st = ps.solve(b, rtol=1e-30, maxit=64, pc=L.DG_PC_LEARNED_ONLY, precision=L.DG_PREC_SPLIT,
                         raise_on_fail=False)
        out.update({"K": mesh.K, "training": info, "iterations": st["iterations"], "ms": st["ms"]})
        ps.ctx.close()
    elif name == "learned_solve":
        # the learned iteration's kernels without the training phase: small
        # random weights (the kernels' cost does not depend on their values)
        from hopefoam_gb300.mesh import delaunay_square
        from hopefoam_gb300.poisson import PressureSolver, poisson_rhs

        mesh = delaunay_square(12000 if small else 50000, seed=0)
        ps = PressureSolver(mesh, 4, tau_coef=1.0)
        ps.lpc_setup(hidden=32, seed=0, capacity=0, form="schwarz")
        W = np.random.default_rng(0).standard_normal((32, 4 * ps.Np)).astype(np.float32) * 1e-3
        ps.lpc_set_weights(W)
        b, _ = poisson_rhs(mesh, 4, seed=1)
        _, st = ps.solve(b, rtol=1e-30, maxit=64, pc=L.DG_PC_LEARNED_ONLY, precision=L.DG_PREC_SPLIT,
                         raise_on_fail=False)
        out.update({"K": mesh.K, "iterations": st["iterations"], "ms": st["ms"]})
        ps.ctx.close()
    elif name == "learned_mlp":
        # the two-layer form's tensor-core kernels: two applies and two
        # energy-gradient evaluations with random weights
        from hopefoam_gb300.mesh import delaunay_square
        from hopefoam_gb300.poisson import PressureSolver

        mesh = delaunay_square(12000 if small else 50000, seed=0)
        ps = PressureSolver(mesh, 4, tau_coef=1.0)
        ps.lpc_setup(hidden=128, seed=0, capacity=0, form="mlp")
        rng = np.random.default_rng(0)
        ps.lpc_set_weights((rng.standard_normal((128, 4 * ps.Np)) * 0.05).astype(np.float32))
        r = rng.standard_normal(mesh.K * ps.Np)
        for _ in range(2):
            ps.lpc_apply(r)
        for _ in range(2):
            _, _, loss = ps.lpc_energy_gradients(r)
        out.update({"K": mesh.K, "loss": loss})
        ps.ctx.close()
    elif name == "ins":
        out.update(ins_bench(n=64 if small else 128, steps=2, warmup=1, with_cpu=False))
    elif name == "cylinder":
        out.update(cylinder_bench(steps=3 if small else 8, warmup=0, with_cpu=False))
    elif name == "limiter":
        out.update(shock_bench(steps=10 if small else 50, warmup=2, with_cpu=False))
    elif name == "batch":
        prec = L.DG_PREC_SPLIT
        out.update(batch_bench(prec, n_cases=32 if small else 512, nsteps=2 if small else 10))
        # the one-launch-per-stage schedule as well, whatever the tuner kept
        from hopefoam_gb300.batch import EulerBatch, batch_cases

        b = EulerBatch(batch_cases(32 if small else 512, seed=0))
        b.set_schedule(2, precision=prec)
        b.run(2, precision=prec)
        out["fused_ms_2_steps"] = b.run(2, precision=prec)
        b.close()
    elif name == "split":
        from hopefoam_gb300 import euler

        order = 5
        mesh = workload(128 if small else 256, order)
        q0, _, _ = initial_state(mesh, order)
        ctx = euler.EulerContext(mesh, order)
        ctx.upload(q0)
        dt = host_cfl_dt(mesh, order, q0)
        ctx.lserk4(dt, 2, flux=L.DG_FLUX_LF, precision=L.DG_PREC_SPLIT)
        torch.cuda.synchronize()
        out.update({"K": mesh.K, "steps": 2})
        ctx.close()
    print(json.dumps(out))


PROFILE_TARGETS = ("pcg", "multilevel", "learned", "learned_solve", "learned_mlp", "ins", "cylinder", "limiter", "batch",
                   "split")


def _split_ready(ctx):
    from hopefoam_gb300 import _lib as L

    try:
        ctx.rhs(flux=L.DG_FLUX_LF, precision=L.DG_PREC_SPLIT)
        return True
    except L.DGError:
        return False


if __name__ == "__main__":
    main()
