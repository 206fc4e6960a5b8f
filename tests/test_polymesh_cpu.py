"""Mesh and field file I/O: OpenFOAM polyMesh (one-layer prism 2D cases),
Fluent face zones as patches, DG field files.

The reference's own tutorial meshes are read from the reference checkout
named by the environment variable HOPEFOAM_REFERENCE_ROOT (the directory that
holds HopeFOAM-0.1/; they are not copied into this repository), and skipped
without it; the round trips run on generated meshes."""
import os

import numpy as np
import pytest

from hopefoam_gb300.mesh import box_square, delaunay_square
from hopefoam_gb300.polymesh import read_dg_field, read_polymesh, write_dg_field, write_polymesh

REF = os.path.join(os.environ.get("HOPEFOAM_REFERENCE_ROOT", "/nonexistent"), "HopeFOAM-0.1", "tutorials", "DG", "2D")


def _areas(m):
    a = m.VXY[:, 1] - m.VXY[:, 0]
    b = m.VXY[:, 2] - m.VXY[:, 0]
    return 0.5 * (a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0])


def _same(m1, m2):
    for f in ("EToV", "EToE", "EToF", "ROT", "BC"):
        assert np.array_equal(getattr(m1, f), getattr(m2, f)), f
    assert np.array_equal(m1.VXY, m2.VXY)


def test_polymesh_round_trip_box(tmp_path):
    m = box_square(7, 5, 2.0, 1.0)
    # patches by side: left/right/bottom/top from the face midpoints
    mid = 0.5 * (m.VXY + np.roll(m.VXY, -1, axis=1))
    patch = -np.ones((m.K, 3), np.int32)
    bk, bf = np.nonzero(m.EToE < 0)
    x, y = mid[bk, bf, 0], mid[bk, bf, 1]
    patch[bk, bf] = np.select([np.isclose(x, 0), np.isclose(x, 2.0), np.isclose(y, 0)], [0, 1, 2], 3)
    write_polymesh(m, str(tmp_path), patch=patch, patch_names=("left", "right", "bottom", "top"))
    r = read_polymesh(str(tmp_path))
    _same(m, r)
    assert r.patch_names == ("left", "right", "bottom", "top")
    assert np.array_equal(r.patch, patch)
    assert (_areas(r) > 0).all()


def test_polymesh_round_trip_delaunay(tmp_path):
    m = delaunay_square(300, seed=4)
    write_polymesh(m, str(tmp_path))
    r = read_polymesh(os.path.join(str(tmp_path), "constant", "polyMesh"))
    _same(m, r)
    assert r.patch_names == ("boundary",)
    assert np.array_equal(r.patch >= 0, m.EToE < 0)


def test_dg_field_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    s = rng.standard_normal((40, 10))
    v = rng.standard_normal((40, 10, 2))
    write_dg_field(str(tmp_path / "p"), "p", s, dimensions="[0 2 -2 0 0 0 0]", boundary={"inlet": {"type": "zeroGradient"}})
    write_dg_field(str(tmp_path / "U"), "U", v)
    assert np.array_equal(read_dg_field(str(tmp_path / "p"), K=40), s)
    r = read_dg_field(str(tmp_path / "U"), K=40)
    assert np.array_equal(r[..., :2], v) and np.all(r[..., 2] == 0)


@pytest.mark.skipif(not os.path.isdir(REF), reason="HOPEFOAM_REFERENCE_ROOT not set")
def test_reference_cylinder_polymesh():
    m = read_polymesh(os.path.join(REF, "cylinder"))
    assert m.K == 1840
    counts = {n: int((m.patch == i).sum()) for i, n in enumerate(m.patch_names)}
    assert counts == {"channel": 128, "outlet": 12, "inlet": 16, "upcylinder": 16, "downcylinder": 16}
    assert (_areas(m) > 0).all()
    kk, ff = np.nonzero(m.EToE >= 0)
    n, fn = m.EToE[kk, ff], m.EToF[kk, ff]
    assert np.array_equal(m.EToE[n, fn], kk) and np.array_equal(m.EToF[n, fn], ff)


@pytest.mark.skipif(not os.path.isdir(REF), reason="HOPEFOAM_REFERENCE_ROOT not set")
def test_reference_fluent_zones_and_fields():
    from hopefoam_gb300.meshio import read_fluent_msh

    for f, K, nb in (("vortexh.msh", 14, 4), ("vortex0.5h.msh", 56, 8), ("vortex0.25h.msh", 224, 16)):
        m = read_fluent_msh(os.path.join(REF, "pearsonVortex", f))
        assert m.K == K and m.patch_names == ("outlet", "inlet")
        assert [int((m.patch == i).sum()) for i in range(2)] == [nb, nb]
    assert read_dg_field(os.path.join(REF, "pearsonVortex", "0", "p")) == 0.0
    assert np.array_equal(read_dg_field(os.path.join(REF, "pearsonVortex", "0", "U")), [0.0, 0.0, 0.0])


@pytest.mark.parametrize("order", [1, 3, 5])
def test_vtk_output(tmp_path, order):
    """Every element split into N^2 counter-clockwise sub-triangles over its own
    nodes (dgToVTK's vtkTopo.C); the sub-triangles tile the domain."""
    from hopefoam_gb300.vtk import read_vtk, write_vtk

    m = delaunay_square(60, seed=2)
    Np = (order + 1) * (order + 2) // 2
    rng = np.random.default_rng(0)
    p = rng.standard_normal((m.K, Np))
    U = rng.standard_normal((m.K, Np, 2))
    path = str(tmp_path / "out.vtk")
    write_vtk(path, m, order, {"p": p, "U": U})
    r = read_vtk(path)
    assert r["points"].shape == (m.K * Np, 3) and r["cells"].shape == (m.K * order * order, 3)
    P = r["points"][:, :2]
    a = P[r["cells"][:, 1]] - P[r["cells"][:, 0]]
    b = P[r["cells"][:, 2]] - P[r["cells"][:, 0]]
    area = 0.5 * (a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0])
    assert np.all(area > 0)
    assert np.isclose(area.sum(), (2 * np.pi) ** 2)
    assert np.array_equal(r["data"]["p"], p.reshape(-1)) and np.array_equal(r["data"]["U"][:, :2], U.reshape(-1, 2))
