"""The Chorin-step oracle (oracle/ins_oracle.py) on the reference's
Pearson-vortex case: operator identities and convergence of the pressure
error under mesh refinement (the tutorial has no published numbers; the
scheme at N = 2 must converge at about third order)."""
import numpy as np
import pytest

from conftest import golden_mesh


def _oracle(mesh, N=2, **kw):
    from hopefoam_gb300.mesh import load_cubature
    from oracle.ins_oracle import ChorinOracle

    return ChorinOracle(mesh, N, load_cubature(3 * (N + 1)), **kw)


def test_nodal_operators_exact_on_polynomials():
    from hopefoam_gb300.ins import pearson_mesh

    N = 3
    c = _oracle(pearson_mesh(3), N=N)
    x, y = c.x, c.y
    u = np.stack([x ** 2 * y + y ** 3, x * y ** 2 - x ** 3])  # degree 3 <= N
    div = c.O.div_nodal(u)
    assert np.allclose(div, 2 * x * y + 2 * x * y, atol=1e-11)
    p = x ** 3 - 2 * x * y ** 2
    g = c.O.grad_nodal(p)
    assert np.allclose(g[0], 3 * x ** 2 - 2 * y ** 2, atol=1e-11) and np.allclose(g[1], -4 * x * y, atol=1e-11)
    # w = dv/dx - du/dy = (y^2 - 3x^2) - (x^2 + 3y^2) = -4x^2 - 2y^2; curl w = (dw/dy, -dw/dx) = (-4y, 8x)
    cc = c.O.curlcurl(u)
    assert np.allclose(cc[0], -4 * y, atol=1e-10) and np.allclose(cc[1], 8 * x, atol=1e-10)


def test_convection_of_a_uniform_field_is_zero():
    from hopefoam_gb300.ins import pearson_mesh

    c = _oracle(pearson_mesh(4))
    U = np.stack([np.full_like(c.x, 0.7), np.full_like(c.x, -0.3)])
    ub = np.zeros((c.K, 3, 2, c.Nfp))
    ub[:, :, 0], ub[:, :, 1] = 0.7, -0.3
    Nn = c.O.convection(U, ub)
    assert np.abs(Nn).max() < 1e-12


@pytest.mark.parametrize("fixture", ["pearson_h", "pearson_0.5h", "pearson_0.25h"])
def test_pearson_fixture_patches(fixture):
    m = golden_mesh(fixture)
    assert m.patch_names == ("outlet", "inlet")
    assert np.array_equal(m.patch >= 0, m.EToE < 0)


def test_pearson_vortex_converges():
    """100 steps of dt = 1e-3 (the tutorial's controlDict), N = 2 (its
    dgSolution baseOrder), nu = 0.01, on the tutorial's three meshes."""
    errs = []
    for name in ("pearson_h", "pearson_0.5h", "pearson_0.25h"):
        c = _oracle(golden_mesh(name), nu=0.01, dt=1e-3)
        for _ in range(100):
            c.step()
        errs.append(c.pressure_error()[0])
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert errs[-1] < 5e-3
    assert np.all(rates > 2.0), (errs, rates)


def test_generated_pearson_mesh_matches_tutorial_pattern():
    from hopefoam_gb300.ins import pearson_mesh

    m = pearson_mesh(8)
    mid = 0.5 * (m.VXY + np.roll(m.VXY, -1, axis=1))
    k, f = np.nonzero(m.patch == 1)  # outlet
    xy = mid[k, f]
    on_bottom = np.isclose(xy[:, 1], -0.5)
    assert np.all(xy[on_bottom, 0] < 0)  # outflow on the left half of the bottom side, as in vortexh.msh
    errs = []
    for n in (8, 16):
        c = _oracle(pearson_mesh(n), nu=0.01, dt=1e-3)
        for _ in range(20):
            c.step()
        errs.append(c.pressure_error()[0])
    assert errs[1] < 2e-3 and np.log2(errs[0] / errs[1]) > 2.0, errs
