"""dg_euler_rhs_noalloc: the allocation-free right-hand side for callers that
may not allocate device memory while they run (stream capture, pool-owned
device memory, real-time loops).  Checked through the C ABI against the
existing entry point dg_euler_rhs (FP64), on two calls in a row with
different states, within the FP64 path's tolerance, on a periodic mesh and on
the double-Mach mesh with reflective-wall slots (whose traces the call
recomputes from the state it is given); and the size limit of its fixed
scratch array is enforced.  This file sorts last so that a run stopping
at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # same kernel as dg_euler_rhs: agreement is expected to be exact


def _ctx(nx, N):
    from hopefoam_gb300 import euler
    from hopefoam_gb300.mesh import periodic_square

    m = periodic_square(nx, nx, 10.0, 10.0, perturb=0.1, seed=5)
    ctx = euler.EulerContext(m, N)
    ops = euler.reference_operators(N)
    x, y = euler.node_coords(m, ops["r"], ops["s"])
    return ctx, x, y


def test_noalloc_rhs_matches_dg_euler_rhs_on_two_calls(gpu_lib):
    import torch

    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300 import euler

    lib = L.lib()
    ctx, x, y = _ctx(12, 3)
    for call, (beta, flux) in enumerate([(5.0, L.DG_FLUX_LF), (2.5, L.DG_FLUX_ROE)]):
        q = euler.isentropic_vortex(x, y, x0=5.0, y0=5.0, beta=beta, uinf=0.6 + 0.1 * call, vinf=0.2)
        ctx.upload(q)
        ref = ctx.rhs(flux=flux, precision=L.DG_PREC_FP64)
        q_dev = torch.from_numpy(q.reshape(-1).copy()).cuda()
        out = torch.full_like(q_dev, float("nan"))
        torch.cuda.synchronize()
        rc = lib.dg_euler_rhs_noalloc(ctx.h, ctypes.c_void_p(q_dev.data_ptr()), ctypes.c_void_p(out.data_ptr()), flux)
        assert rc == L.DG_OK, lib.dg_last_error(ctx.h)
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(ref.shape)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        print("call %d: no-alloc rhs vs dg_euler_rhs rel L2 %.3e" % (call, err))
        assert np.isfinite(got).all()
        assert err < TOL


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu_lib):
    import torch

    from hopefoam_gb300 import _lib as L

    lib = L.lib()
    ctx, x, y = _ctx(64, 5)  # 4 * 8192 * 21 values > 524288
    assert 4 * ctx.K * ctx.Np > L.DG_NOALLOC_MAX_VALUES
    q_dev = torch.ones(4 * ctx.K * ctx.Np, dtype=torch.float64, device="cuda")
    out = torch.empty_like(q_dev)
    rc = lib.dg_euler_rhs_noalloc(ctx.h, ctypes.c_void_p(q_dev.data_ptr()), ctypes.c_void_p(out.data_ptr()), 0)
    assert rc == L.DG_ERR_ARG
    assert b"exceeds the fixed scratch" in lib.dg_last_error(ctx.h)


def test_noalloc_rhs_with_wall_slots(gpu_lib):
    """Reflective-wall boundary slots: the call recomputes their traces from
    the state it is given, as dg_euler_rhs does from the context's state."""
    import os

    import torch

    from conftest import GOLDEN
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300 import euler
    from hopefoam_gb300.mesh import Mesh, connect
    from hopefoam_gb300.shock import DoubleMach

    lib = L.lib()
    d = np.load(os.path.join(GOLDEN, "doublemach.npz"))
    EToE, EToF, ROT, BC = connect(d["EToV"])
    mesh = Mesh(d["EToV"], d["VXY"], EToE, EToF, ROT, BC, name="doubleMach", patch=d["patch"],
                patch_names=tuple(str(x) for x in d["patch_names"]))
    mesh.patch_first_face = d["patch_first_face"]
    N = 4
    dm = DoubleMach(mesh, N)
    ctx = euler.EulerContext(mesh, N)
    assert 4 * ctx.K * ctx.Np <= L.DG_NOALLOC_MAX_VALUES
    ctx.set_boundary_traces(dm.bdata(0.0))
    ctx.set_boundary_kinds(dm.kinds, dm.gref)
    rng = np.random.default_rng(7)
    for call in range(2):
        q = dm.initial_state()
        q = q * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, size=q.shape))  # walls see a non-trivial interior trace
        ctx.upload(q)
        ref = ctx.rhs(flux=L.DG_FLUX_ROE, precision=L.DG_PREC_FP64)
        q_dev = torch.from_numpy(q.reshape(-1).copy()).cuda()
        out = torch.full_like(q_dev, float("nan"))
        torch.cuda.synchronize()
        rc = lib.dg_euler_rhs_noalloc(ctx.h, ctypes.c_void_p(q_dev.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                      L.DG_FLUX_ROE)
        assert rc == L.DG_OK, lib.dg_last_error(ctx.h)
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(ref.shape)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        print("wall slots, call %d: no-alloc rhs vs dg_euler_rhs rel L2 %.3e" % (call, err))
        assert np.isfinite(got).all()
        assert err < TOL
    ctx.close()
