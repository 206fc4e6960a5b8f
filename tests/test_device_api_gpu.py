"""The device-pointer, stream-ordered entry points of the boundary
(include/dgcu.h: dg_euler_rhs_device, dg_forward_euler_stage, dg_sync,
dg_ipdg_apply_device, dg_pcg_solve_device) through ctypes, against their
host-array counterparts: the same kernels on the same data, so the results
agree bit for bit."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("precision", [0, 1])
def test_euler_rhs_device_matches_host_variant(gpu_lib, precision):
    import torch

    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300 import euler
    from hopefoam_gb300.mesh import periodic_square

    lib = L.lib()
    N = 5
    m = periodic_square(20, 20, 10.0, 10.0, perturb=0.1, seed=3)
    ctx = euler.EulerContext(m, N)
    ops = euler.reference_operators(N)
    x, y = euler.node_coords(m, ops["r"], ops["s"])
    q = euler.isentropic_vortex(x, y, x0=5.0, y0=5.0, uinf=0.7, vinf=0.2)
    ctx.upload(q)
    for flux in (L.DG_FLUX_LF, L.DG_FLUX_ROE):
        ref = ctx.rhs(flux=flux, precision=precision)
        out = torch.full((q.size,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        assert lib.dg_euler_rhs_device(ctx.h, flux, precision, _vp(out)) == L.DG_OK, lib.dg_last_error(ctx.h)
        assert lib.dg_sync(ctx.h) == L.DG_OK, lib.dg_last_error(ctx.h)
        got = out.cpu().numpy().reshape(ref.shape)
        assert np.array_equal(got, ref), np.abs(got - ref).max()
    ctx.close()


def test_forward_euler_stage(gpu_lib):
    """q <- q + dt R(q) on the device, against the host-side update from the
    host right-hand side (FMA contraction aside, the same arithmetic)."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300 import euler
    from hopefoam_gb300.mesh import periodic_square

    lib = L.lib()
    N = 3
    m = periodic_square(16, 16, 10.0, 10.0, perturb=0.1, seed=4)
    ctx = euler.EulerContext(m, N)
    ops = euler.reference_operators(N)
    x, y = euler.node_coords(m, ops["r"], ops["s"])
    q = euler.isentropic_vortex(x, y, x0=5.0, y0=5.0)
    ctx.upload(q)
    dt = 1e-3
    r = ctx.rhs(flux=L.DG_FLUX_ROE, precision=L.DG_PREC_FP64)
    assert lib.dg_forward_euler_stage(ctx.h, dt, L.DG_FLUX_ROE, L.DG_PREC_FP64) == L.DG_OK
    assert lib.dg_sync(ctx.h) == L.DG_OK
    got = ctx.download()
    want = q + dt * r
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err < 1e-15, err
    ctx.close()


def test_ipdg_apply_and_pcg_device_match_host_variants(gpu_lib):
    import torch

    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.mesh import delaunay_square
    from hopefoam_gb300.poisson import PressureSolver, poisson_rhs

    lib = L.lib()
    N = 4
    mesh = delaunay_square(600, seed=2)
    ps = PressureSolver(mesh, N, tau_coef=1.0)
    h = ps.ctx.h
    n = mesh.K * ps.Np
    rng = np.random.default_rng(5)
    xh = rng.standard_normal(n)
    yh = np.empty(n)
    assert lib.dg_ipdg_apply(h, L.dptr(xh), L.dptr(yh)) == L.DG_OK
    xd = torch.from_numpy(xh.copy()).cuda()
    yd = torch.full_like(xd, float("nan"))
    torch.cuda.synchronize()
    assert lib.dg_ipdg_apply_device(h, _vp(xd), _vp(yd)) == L.DG_OK, lib.dg_last_error(h)
    torch.cuda.synchronize()
    assert np.array_equal(yd.cpu().numpy(), yh)

    b, _ = poisson_rhs(mesh, N, seed=1)
    b = np.ascontiguousarray(b, np.float64).reshape(-1)
    for pc, prec in ((L.DG_PC_BLOCK_JACOBI, L.DG_PREC_FP64), (L.DG_PC_BLOCK_JACOBI, L.DG_PREC_SPLIT),
                     (L.DG_PC_MULTILEVEL, L.DG_PREC_SPLIT)):
        x_host = np.zeros(n)
        st_h = L.SolveStats()
        assert lib.dg_pcg_solve(h, L.dptr(b), L.dptr(x_host), 1e-10, 5000, pc, prec, ctypes.byref(st_h)) == L.DG_OK
        bd = torch.from_numpy(b.copy()).cuda()
        xd = torch.zeros_like(bd)
        st_d = L.SolveStats()
        torch.cuda.synchronize()
        rc = lib.dg_pcg_solve_device(h, _vp(bd), _vp(xd), 1e-10, 5000, pc, prec, ctypes.byref(st_d))
        assert rc == L.DG_OK, lib.dg_last_error(h)
        torch.cuda.synchronize()
        assert st_d.iterations == st_h.iterations
        assert st_d.rel_residual == st_h.rel_residual
        assert np.array_equal(xd.cpu().numpy(), x_host)
    ps.ctx.close()
