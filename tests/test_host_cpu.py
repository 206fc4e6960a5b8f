"""Host logic without a GPU: the product library loads and exports every
entry point of include/dgcu.h, its host operator builder agrees with the
oracle, and the mesh tools build consistent connectivity."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden_mesh


@pytest.fixture(scope="module")
def lib():
    from hopefoam_gb300 import build

    build.build()
    from hopefoam_gb300 import _lib

    return _lib.lib()


def header_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*(?:int|const char\*)\s+(dg_\w+)\s*\(", txt, re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol(lib):
    from hopefoam_gb300 import _lib

    names = header_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, "python binding missing for " + n


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 6, 7])
def test_host_operators_match_oracle(lib, N):
    from hopefoam_gb300 import euler
    from hopefoam_gb300.mesh import load_cubature, periodic_square
    from oracle import oracle

    ops = euler.reference_operators(N)
    o = oracle.Oracle(periodic_square(3, 3, 1.0, 1.0), N, load_cubature(3 * (N + 1)))
    ref = o.operators()
    scale = 1 + np.abs(ref["Dr"]).max()
    assert np.abs(ops["r"] - ref["r"]).max() < 1e-14
    assert np.abs(ops["s"] - ref["s"]).max() < 1e-14
    assert np.abs(ops["Dr"] - ref["Dr"]).max() < 1e-13 * scale
    assert np.abs(ops["Ds"] - ref["Ds"]).max() < 1e-13 * scale
    assert np.abs(ops["Vg"] - ref["cellV"]).max() < 1e-13
    assert np.abs(ops["If"] - ref["faceInterp"]).max() < 1e-13
    fn = euler.face_nodes(N)
    assert (fn == ref["fci"][:, 0, :]).all()


def test_operator_errors(lib):
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300 import euler

    with pytest.raises(L.DGError) as e:
        euler.reference_operators(9, cubature=np.zeros((5, 3)))
    assert e.value.code in (L.DG_ERR_UNSUPPORTED, L.DG_ERR_ARG)
    with pytest.raises(L.DGError) as e:
        euler.reference_operators(3, cubature=np.zeros((5, 3)))
    assert e.value.code == L.DG_ERR_ARG


def test_periodic_mesh_connectivity():
    from hopefoam_gb300.mesh import periodic_square

    m = periodic_square(9, 7, 10.0, 5.0, perturb=0.1, seed=4)
    K = m.K
    assert K == 2 * 9 * 7
    assert (m.EToE >= 0).all()
    k = np.repeat(np.arange(K), 3)
    f = np.tile(np.arange(3), K)
    n, fn = m.EToE.reshape(-1), m.EToF.reshape(-1)
    assert (m.EToE[n, fn] == k).all() and (m.EToF[n, fn] == f).all()
    v = m.VXY
    a, b = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
    assert ((a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]) > 0).all()
    # the two sides of each face are the same segment up to a period shift
    p0 = v[k, f]
    p1 = v[k, (f + 1) % 3]
    q0 = v[n, fn]
    q1 = v[n, (fn + 1) % 3]
    d = (p0 - q1)
    d2 = (p1 - q0)
    assert np.allclose(d, d2)
    assert np.allclose(np.mod(d[:, 0] + 1e-9, 10.0), 1e-9) and np.allclose(np.mod(d[:, 1] + 1e-9, 5.0), 1e-9)


def test_delaunay_and_fluent_meshes():
    from hopefoam_gb300.mesh import delaunay_square

    m = delaunay_square(400, seed=1)
    assert m.K > 700 and (m.EToE < 0).sum() > 0
    g = golden_mesh("vortex0256")
    assert g.K == 256 and (g.EToE < 0).sum() == 32


def test_batch_case_list_is_seeded():
    from hopefoam_gb300.batch import batch_cases, concat_meshes
    from hopefoam_gb300.mesh import periodic_square

    a = batch_cases(n=64, seed=0)
    b = batch_cases(n=64, seed=0)
    assert a == b
    assert {c["order"] for c in a} <= {2, 3, 4, 5, 6}
    ks = [2 * c["m"] ** 2 for c in a]
    assert min(ks) >= 2 * 20 ** 2 * 0.9 and max(ks) <= 20000 * 1.1
    m1 = periodic_square(3, 3, seed=1)
    m2 = periodic_square(4, 4, seed=2)
    big = concat_meshes([m1, m2])
    assert big.K == m1.K + m2.K
    # the cases stay disconnected: every neighbour lies in the same case
    own = np.repeat([0, 1], [m1.K, m2.K])
    nb = big.EToE
    assert np.all(own[nb] == own[:, None])


def test_oracle_limiter_properties():
    """The restated limiter keeps a uniform state, keeps each element's
    average of rho (when no density correction triggers) and leaves every
    element linear."""
    from hopefoam_gb300 import euler
    from hopefoam_gb300.mesh import box_square, load_cubature
    from oracle.oracle import Oracle

    N = 3
    m = box_square(5, 4, 1.0, 1.0)
    orc = Oracle(m, N, load_cubature(12))
    x, y = orc.nodes()
    kk, ff = euler.boundary_faces(m)
    nb = len(kk)
    fn = euler.face_nodes(N)
    const = np.stack([np.full_like(x, 1.2), np.full_like(x, 0.3), np.full_like(x, -0.1), np.full_like(x, 3.0)])
    bnd = np.stack([const[:, k, fn[f]] for k, f in zip(kk, ff)])
    out = orc.limiter(const, bnd, np.zeros(nb, np.int32))
    assert np.allclose(out, const, rtol=0, atol=1e-13)
    rho = 1 + 0.2 * np.sin(3 * x) * np.cos(2 * y)
    q = np.stack([rho, rho * 0.4, rho * 0.1, 2.5 + 0.1 * x])
    bnd = np.stack([q[:, k, fn[f]] for k, f in zip(kk, ff)])
    out = orc.limiter(q, bnd, np.full(nb, 2, np.int32))
    M = orc.mass()
    w = M.sum(1)  # integral weights of each node
    assert np.allclose((w * out[0]).sum(1), (w * q[0]).sum(1), rtol=1e-12)
    ops = orc.operators()
    r, s = ops["r"], ops["s"]
    A = np.stack([np.ones_like(r), r, s], 1)  # linear fit per element is exact
    for v in range(4):
        coef, res, *_ = np.linalg.lstsq(A, out[v].T, rcond=None)
        assert np.abs(A @ coef - out[v].T).max() < 1e-11


def test_oracle_boundary_kinds_in_limited_step():
    """Zero-gradient slots take the interior trace, walls the trace with the
    normal momentum reversed, fixed-value and other slots keep their values
    (the limited step's boundary bookkeeping, oracle/limited_oracle.py)."""
    from hopefoam_gb300 import euler
    from hopefoam_gb300.mesh import box_square, load_cubature
    from oracle.limited_oracle import LimitedSSPOracle

    N = 2
    m = box_square(4, 3, 1.0, 0.8)
    kk, ff = euler.boundary_faces(m)
    kinds = (np.arange(len(kk)) % 4).astype(np.int32)
    lo = LimitedSSPOracle(m, N, load_cubature(9), kinds)
    x, y = lo.O.nodes()
    rho = 1 + 0.2 * np.sin(3 * x)
    q = np.stack([rho, 0.3 * rho + 0.1 * y, -0.2 * rho, 2.5 + 0.1 * x])
    B0 = np.random.default_rng(1).standard_normal((len(kk), 4, N + 1))
    B = lo.reflect(q, B0)
    t = lo.traces(q)
    assert np.array_equal(B[kinds == 3], t[kinds == 3])
    assert np.array_equal(B[kinds == 0], B0[kinds == 0]) and np.array_equal(B[kinds == 2], B0[kinds == 2])
    w = kinds == 1
    nx, ny = lo.nx[w][:, None], lo.ny[w][:, None]
    # the wall value's normal momentum is the trace's, negated; tangential and scalars kept
    assert np.allclose(nx * B[w, 1] + ny * B[w, 2], -(nx * t[w, 1] + ny * t[w, 2]), atol=1e-14)
    assert np.allclose(-ny * B[w, 1] + nx * B[w, 2], -ny * t[w, 1] + nx * t[w, 2], atol=1e-14)
    assert np.array_equal(B[w, 0], t[w, 0]) and np.array_equal(B[w, 3], t[w, 3])
