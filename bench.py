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
    from hopefoam_gb300 import euler

    ops = euler.reference_operators(order)
    x, y = euler.node_coords(mesh, ops["r"], ops["s"])
    return euler.isentropic_vortex(x, y, x0=5.0, y0=5.0), x, y


def alg_bytes_per_elem_stage(order):
    """Minimum HBM bytes one element moves per RK stage in the fused kernel:
    q read + q write + res read + res write (4 vars x Np x 8 B each), the three
    neighbour face traces (3 x 4 x Nfp x 8 B), 4 FP64 metrics and 3 int32
    neighbour words."""
    Np = (order + 1) * (order + 2) // 2
    Nfp = order + 1
    return 128 * Np + 96 * Nfp + 32 + 12


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


def cpu_baseline(mesh, order, q0, dt, threads):
    """Oracle LSERK4 (one time step = 5 stages) on the full mesh with all host
    threads; returns DOF-stage/s."""
    from hopefoam_gb300.mesh import load_cubature
    from oracle import oracle

    oracle.set_threads(threads)
    orc = oracle.Oracle(mesh, order, load_cubature(3 * (order + 1)))
    q = q0.reshape(-1)
    t = time.perf_counter()
    orc.lserk4(q, dt, 1, flux=0)
    el = time.perf_counter() - t
    dofs = mesh.K * orc.Np * 4
    return dofs * 5 / el, el


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    order = 5
    mesh = workload()
    q0, _, _ = initial_state(mesh, order)
    from oracle import oracle

    from hopefoam_gb300.mesh import load_cubature

    threads = oracle.max_threads()
    oracle.set_threads(threads)
    orc = oracle.Oracle(mesh, order, load_cubature(3 * (order + 1)))
    dt = 1e-4
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
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "isentropic vortex, periodic 256x256x2 perturbed, N=5, LSERK4, LF flux",
                       "K": mesh.K, "order": order},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "one LSERK4 step (5 stages) over all 131072 elements per bench step"},
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
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

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
    ctx = euler.EulerContext(mesh, order)
    ctx.upload(q0)
    dt = ctx.cfl_dt(0.5)
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
    bpe = alg_bytes_per_elem_stage(order)
    achieved = bpe * mesh.K / per_launch_s / 1e9
    peak, peak_kind = peaks()
    qfin = ctx.download()
    finite = bool(np.isfinite(qfin).all())

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
        "config": {"workload": "isentropic vortex, periodic 256x256x2 perturbed 10%, N=5 (Np=21), LF flux, LSERK4 "
                               "CFL 0.5", "K": mesh.K, "order": order, "precision": prec_name,
                   "l2": "working set (q in/out + res) %.0f MB > 129 MB L2, no flush" % (3 * n * 8 / 1e6)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_kind": peak_kind, "bytes_per_elem_stage": bpe,
                     "kernel": "euler_stage_%s" % prec_name},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8},
        "gpu_launches": launches,
        "clocks": ck,
        "state_finite": finite,
    }
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle

        threads = oracle.max_threads()
        v, el = cpu_baseline(mesh, order, q0, dt, threads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "one LSERK4 step (5 stages) over all %d elements, %.1f s" % (mesh.K, el)}
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def _split_ready(ctx):
    from hopefoam_gb300 import _lib as L

    try:
        ctx.rhs(flux=L.DG_FLUX_LF, precision=L.DG_PREC_SPLIT)
        return True
    except L.DGError:
        return False


if __name__ == "__main__":
    main()
