"""SIPG operator and PCG solve on the GPU against the oracle's assembled
element blocks (the reference's laplacianFunc restated), through the C ABI.
Tolerances: operator apply 1e-12 relative L2 (FP64 round-off); solves must
reach ||b - S x|| / ||b|| <= 1e-10 (true FP64 residual) and agree with the
oracle's CG solution to 1e-8 relative."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _setup(mesh, N, tau=20.0):
    from hopefoam_gb300.mesh import load_cubature
    from hopefoam_gb300.poisson import PressureSolver
    from oracle import oracle

    ps = PressureSolver(mesh, N, tau_coef=tau)
    orc = oracle.Oracle(mesh, N, load_cubature(3 * (N + 1)))
    diag, off, _ = orc.ipdg_blocks(tau_coef=tau)
    return ps, orc, diag, off


def _vertex_ulp_sensitivity(mesh, N, x, ref):
    """Relative change of the oracle's assembled apply when every vertex
    coordinate moves by one ulp: the geometry round-off floor of the
    comparison (unstructured meshes have near-degenerate elements)."""
    from hopefoam_gb300.mesh import Mesh, load_cubature
    from oracle import oracle

    rng = np.random.default_rng(7)
    v = mesh.VXY * (1 + rng.uniform(-1.1e-16, 1.1e-16, mesh.VXY.shape))
    o2 = oracle.Oracle(Mesh(mesh.EToV, v, mesh.EToE, mesh.EToF, mesh.ROT, mesh.BC), N, load_cubature(3 * (N + 1)))
    d2, f2, _ = o2.ipdg_blocks(tau_coef=20.0)
    return rel_l2(-o2.blk_apply(d2, f2, x), ref)


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 6, 7])
def test_apply_matches_assembled_operator(gpu_lib, N):
    from hopefoam_gb300.mesh import delaunay_square

    m = delaunay_square(60, seed=N)
    ps, orc, diag, off = _setup(m, N)
    rng = np.random.default_rng(N)
    x = rng.standard_normal(m.K * ps.Np)
    y = ps.apply(x)
    ref = -orc.blk_apply(diag, off, x)
    err = rel_l2(y, ref)
    tol = max(1e-12, 10 * _vertex_ulp_sensitivity(m, N, x, ref))
    print("N=%d SIPG apply rel L2 %.3e (tol %.1e)" % (N, err, tol))
    assert err < tol


def test_apply_periodic_interior_only(gpu_lib):
    from hopefoam_gb300.mesh import periodic_square

    m = periodic_square(5, 4, 2.0, 2.0, perturb=0.1, seed=3)
    ps, orc, diag, off = _setup(m, 4, tau=10.0)
    x = np.random.default_rng(0).standard_normal(m.K * ps.Np)
    assert rel_l2(ps.apply(x), -orc.blk_apply(diag, off, x)) < 1e-12


@pytest.mark.parametrize("precision", [0, 1])
def test_pcg_reaches_tolerance_and_matches_oracle(gpu_lib, precision):
    from hopefoam_gb300.mesh import delaunay_square

    N = 4
    m = delaunay_square(400, seed=11)
    ps, orc, diag, off = _setup(m, N)
    rng = np.random.default_rng(5)
    b = rng.standard_normal(m.K * ps.Np)
    x, st = ps.solve(b, rtol=1e-10, precision=precision)
    print("precision %d: iterations %d rel residual %.3e (%.2f ms)" % (precision, st["iterations"],
                                                                       st["rel_residual"], st["ms"]))
    assert st["rel_residual"] <= 1e-10
    # independent check of the residual with the oracle's assembled operator
    r = b - (-orc.blk_apply(diag, off, x))
    assert np.linalg.norm(r) / np.linalg.norm(b) < 2e-10
    xo, it, rr = orc.pcg_bj(diag, off, b, rtol=1e-12)
    assert rel_l2(x, xo) < 1e-8


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5])
def test_mixed_pcg_every_lane_order(gpu_lib, N):
    """Mixed-precision PCG at every order of the two-pass FP32 apply (N <= 5):
    the true FP64 residual reaches 1e-10, the solution matches the FP64 solve
    to 1e-8, and the FP32 operator costs at most a quarter more
    iterations than the FP64 one (a wrong face exchange would not converge
    or would need many more)."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.mesh import delaunay_square

    m = delaunay_square(300, seed=13)
    ps, orc, diag, off = _setup(m, N, tau=1.0)
    b = np.random.default_rng(N).standard_normal(m.K * ps.Np)
    x64, st64 = ps.solve(b, rtol=1e-10, precision=L.DG_PREC_FP64)
    xmx, stmx = ps.solve(b, rtol=1e-10, precision=L.DG_PREC_SPLIT)
    print("N=%d K=%d: FP64 %d its, mixed %d its" % (N, m.K, st64["iterations"], stmx["iterations"]))
    assert stmx["rel_residual"] <= 1e-10
    r = b - (-orc.blk_apply(diag, off, xmx))
    assert np.linalg.norm(r) / np.linalg.norm(b) < 2e-10
    assert rel_l2(xmx, x64) < 1e-8
    assert stmx["iterations"] <= 1.25 * st64["iterations"] + 20


def test_pcg_errors(gpu_lib):
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.mesh import delaunay_square

    m = delaunay_square(100, seed=2)
    ps, orc, diag, off = _setup(m, 3)
    b = np.ones(m.K * ps.Np)
    x, st = ps.solve(b, rtol=1e-14, maxit=3, raise_on_fail=False)
    assert st["status"] == L.DG_ERR_NOT_CONVERGED
    with pytest.raises(L.DGError):
        ps.solve(b, pc=L.DG_PC_LEARNED + 5)
