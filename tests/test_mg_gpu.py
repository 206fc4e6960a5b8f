"""Block-Jacobi PCG with the multilevel coarse-space correction
(DG_PC_MULTILEVEL) on the SIPG pressure operator, through the C ABI:
same solution as block Jacobi (both to rtol 1e-10: the solutions agree to
1e-8 relative), iteration counts that do not grow with the mesh, both
arithmetic modes, and the mixed boundary types / Helmholtz form of the
incompressible step."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _solver(n_interior, N, tau):
    from hopefoam_gb300.mesh import delaunay_square
    from hopefoam_gb300.poisson import PressureSolver, poisson_rhs

    m = delaunay_square(n_interior, seed=1)
    ps = PressureSolver(m, N, tau_coef=tau)
    b, _ = poisson_rhs(m, N, seed=3)
    return ps, b


@pytest.mark.parametrize("N,tau", [(4, 1.0), (2, 20.0), (7, 1.0)])
def test_multilevel_matches_block_jacobi(gpu_lib, N, tau):
    from hopefoam_gb300 import _lib as L

    ps, b = _solver(3000, N, tau)
    x_bj, st_bj = ps.solve(b, rtol=1e-10, pc=L.DG_PC_BLOCK_JACOBI, precision=L.DG_PREC_FP64)
    x_mg, st_mg = ps.solve(b, rtol=1e-10, pc=L.DG_PC_MULTILEVEL, precision=L.DG_PREC_FP64)
    x_mx, st_mx = ps.solve(b, rtol=1e-10, pc=L.DG_PC_MULTILEVEL, precision=L.DG_PREC_SPLIT)
    print("N=%d tau=%g K=%d: block Jacobi %d its %.1f ms, multilevel %d its %.1f ms (mixed %d its %.1f ms)" %
          (N, tau, ps.mesh.K if hasattr(ps, "mesh") else -1, st_bj["iterations"], st_bj["ms"], st_mg["iterations"],
           st_mg["ms"], st_mx["iterations"], st_mx["ms"]))
    assert st_mg["rel_residual"] <= 1e-10 and st_mx["rel_residual"] <= 1e-10
    assert rel_l2(x_mg, x_bj) < 1e-8 and rel_l2(x_mx, x_bj) < 1e-8
    assert st_mg["iterations"] * 4 < st_bj["iterations"]


def test_multilevel_iterations_do_not_grow(gpu_lib):
    from hopefoam_gb300 import _lib as L

    its = []
    for n in (2000, 8000, 32000):
        ps, b = _solver(n, 4, 1.0)
        _, st = ps.solve(b, rtol=1e-10, pc=L.DG_PC_MULTILEVEL, precision=L.DG_PREC_FP64)
        its.append(st["iterations"])
    print("multilevel iterations at 2k / 8k / 32k interior points:", its)
    assert max(its) < 1.6 * min(its)
