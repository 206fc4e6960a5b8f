"""Curved arc patches on the host: the patch code, the closest points, the
mesh-point snapping of applyCurveBoundary and the node relocation next to the
curve (hopefoam_gb300/curved.py) against known answers and the oracle's
restatement (oracle.oracle.curved_nodes).

Known answer: the cylinder tutorial's arcs are halves of the circle of radius
0.05 about the origin, whose closest point to p is 0.05 p / |p|.  Tolerance
1e-14 absolute on coordinates of size 0.2 (rounding of the same formulas in
a different order)."""
import os

import numpy as np
import pytest

from conftest import golden_mesh

R = 0.05


def _radial(x, y):
    x, y = np.asarray(x, np.float64), np.asarray(y, np.float64)
    rr = np.hypot(x, y)
    return R * x / rr, R * y / rr


def test_arc_code_parsing():
    from hopefoam_gb300.curved import ArcCurve, read_arc_patches

    m = golden_mesh("cylinder")
    up, down = m.curves["upcylinder"], m.curves["downcylinder"]
    x, y = up.point(np.array([-0.5, 0.0, 0.25]))
    assert np.allclose(x, [-R, 0.0, R * np.sin(np.pi / 4)], atol=1e-17)
    assert np.allclose(y, [0.0, R, R * np.cos(np.pi / 4)], atol=1e-17)
    assert np.allclose(down.point(0.0)[1], -R)
    text = """
    3
    (
        wall { type wall; nFaces 4; startFace 10; }
        bump
        {
            type            arc;
            nFaces          8;
            startFace       14;
            u_Range         (0 2);
            v_Range         (0 0);
            code
            #{
                2.0*u - 1.0,
                0.1*Foam::pow(Foam::sin(Foam::constant::mathematical::pi*u/2.0), 2) + std::sqrt(4.0),
                v
            #};
        }
        out { type patch; nFaces 2; startFace 22; }
    )"""
    c = read_arc_patches(text)
    assert list(c) == ["bump"]
    x, y = c["bump"].point(np.array([0.0, 1.0, 2.0]))
    assert np.allclose(x, [-1, 1, 3]) and np.allclose(y, [2.0, 2.1, 2.0])
    for bad in ("__import__('os').getcwd(), u, v", "u.real, u, v", "open, u, v", "[u], u, v", "u, v"):
        with pytest.raises((ValueError, SyntaxError)):
            ArcCurve.from_code(bad, (0, 1))


def test_closest_points_on_circle():
    m = golden_mesh("cylinder")
    up = m.curves["upcylinder"]
    rng = np.random.default_rng(0)
    th = rng.uniform(0.05, np.pi - 0.05, 200)
    rad = R * (1 + rng.uniform(-0.2, 0.2, 200))
    px, py = rad * np.cos(th), rad * np.sin(th)
    x, y = up.project(px, py)
    ex, ey = _radial(px, py)
    assert max(np.abs(x - ex).max(), np.abs(y - ey).max()) < 1e-15


@pytest.mark.parametrize("N", [2, 4, 7])
def test_face_nodes_on_curve(N):
    from hopefoam_gb300 import curved
    from hopefoam_gb300.euler import face_nodes, node_coords, reference_operators

    m = golden_mesh("cylinder")
    ops = reference_operators(N)
    x, y = node_coords(m, ops["r"], ops["s"])
    curves, m.curves = m.curves, None
    x0, y0 = node_coords(m, ops["r"], ops["s"])
    m.curves = curves
    fn = face_nodes(N)
    faces = curved._curved_faces(m)
    assert len(faces) == 32
    moved = np.zeros(m.K, bool)
    for k, f, _ in faces:
        ids = fn[f]
        ex, ey = _radial(x0[k, ids[1:-1]], y0[k, ids[1:-1]])
        assert np.abs(x[k, ids[1:-1]] - ex).max() < 1e-14 and np.abs(y[k, ids[1:-1]] - ey).max() < 1e-14
        assert np.abs(x[k, ids[[0, -1]]] - x0[k, ids[[0, -1]]]).max() < 1e-16  # the end nodes stay
        # the element's other faces keep their nodes
        for g in range(3):
            if g != f:
                assert np.abs(x[k, fn[g]] - x0[k, fn[g]]).max() < 1e-15
        moved[k] = True
    assert np.array_equal(x[~moved], x0[~moved]) and np.array_equal(y[~moved], y0[~moved])
    assert np.hypot(x - x0, y - y0).max() > 1e-4  # the sagitta of a 1/32 circle arc


@pytest.mark.parametrize("N", [2, 3, 5])
def test_blend_against_oracle(N):
    from hopefoam_gb300.euler import node_coords, reference_operators
    from hopefoam_gb300.mesh import load_cubature
    from oracle.oracle import Oracle, curved_nodes

    m = golden_mesh("cylinder")
    ops = reference_operators(N)
    x, y = node_coords(m, ops["r"], ops["s"])
    O = Oracle(m, N, load_cubature(3 * (N + 1)))
    xo, yo = curved_nodes(O, m, ("upcylinder", "downcylinder"), _radial)
    assert np.abs(x - xo).max() < 1e-15 and np.abs(y - yo).max() < 1e-15


def test_blend_of_a_parabola_on_a_box():
    """A non-circular curve on another mesh: the bottom side of a box bent to
    y = a x (1 - x); the oracle takes the curve's closest points by bisection
    on the foot-point condition."""
    from hopefoam_gb300.curved import ArcCurve
    from hopefoam_gb300.euler import face_nodes, node_coords, reference_operators
    from hopefoam_gb300.mesh import box_square, load_cubature
    from oracle.oracle import Oracle, curved_nodes

    a = 0.15
    m = box_square(5, 4, 1.0, 1.0)
    m.patch = np.where(m.EToE < 0, 1, -1).astype(np.int32)
    bottom = (m.EToE < 0) & (np.abs(m.VXY[:, :, 1] + np.roll(m.VXY[:, :, 1], -1, axis=1)) < 1e-12)
    m.patch[bottom] = 0
    m.patch_names = ("curve", "rest")
    m.curves = {"curve": ArcCurve(lambda u: (u, a * u * (1 - u)), (0.0, 1.0), "curve")}

    def project(px, py):
        out = []
        for x0, y0 in zip(np.ravel(px), np.ravel(py)):
            g = lambda u: (u - x0) + (a * u * (1 - u) - y0) * a * (1 - 2 * u)
            lo, hi = x0 - 0.3, x0 + 0.3
            for _ in range(200):
                mid = 0.5 * (lo + hi)
                lo, hi = (mid, hi) if g(mid) < 0 else (lo, mid)
            u = 0.5 * (lo + hi)
            out.append((u, a * u * (1 - u)))
        out = np.array(out)
        return out[:, 0], out[:, 1]

    from hopefoam_gb300.curved import apply_curve_boundary

    m = apply_curve_boundary(m)  # the side's vertices onto the parabola first
    N = 4
    ops = reference_operators(N)
    x, y = node_coords(m, ops["r"], ops["s"])
    O = Oracle(m, N, load_cubature(15))
    xo, yo = curved_nodes(O, m, ("curve",), project)
    assert np.abs(x - xo).max() < 1e-14 and np.abs(y - yo).max() < 1e-14
    fn = face_nodes(N)
    k, f = np.nonzero(m.patch == 0)
    yy = y[k[:, None], fn[f]]
    xx = x[k[:, None], fn[f]]
    # face nodes are the closest points of the parabola: on it to rounding
    assert np.abs(yy - a * xx * (1 - xx)).max() < 1e-15


def test_apply_curve_boundary():
    from hopefoam_gb300 import curved

    m = golden_mesh("cylinder")
    rng = np.random.default_rng(3)
    nv = int(m.EToV.max()) + 1
    P = np.zeros((nv, 2))
    P[m.EToV.ravel()] = m.VXY.reshape(-1, 2)
    on_arc = set()
    for k, f, _ in curved._curved_faces(m):
        on_arc |= {int(m.EToV[k, f]), int(m.EToV[k, (f + 1) % 3])}
    on_arc = np.array(sorted(on_arc))
    Q = P.copy()
    Q[on_arc] *= (1 + rng.uniform(-0.05, 0.05, len(on_arc)))[:, None]  # off the circle, same angle
    m.VXY = Q[m.EToV]
    s = curved.apply_curve_boundary(m)
    S = np.zeros((nv, 2))
    S[s.EToV.ravel()] = s.VXY.reshape(-1, 2)
    assert np.abs(np.hypot(S[on_arc, 0], S[on_arc, 1]) - R).max() < 1e-15
    ex, ey = _radial(Q[on_arc, 0], Q[on_arc, 1])
    assert np.abs(S[on_arc, 0] - ex).max() < 1e-15 and np.abs(S[on_arc, 1] - ey).max() < 1e-15
    rest = np.setdiff1d(np.arange(nv), on_arc)
    assert np.array_equal(S[rest], Q[rest])
    # every element sees the same moved vertex
    assert np.array_equal(s.VXY, S[s.EToV])


@pytest.mark.skipif(not os.environ.get("HOPEFOAM_REFERENCE_ROOT"),
                    reason="HOPEFOAM_REFERENCE_ROOT (the reference tree) not set")
def test_tutorial_polymesh_arcs():
    from hopefoam_gb300.polymesh import read_polymesh

    root = os.environ["HOPEFOAM_REFERENCE_ROOT"]
    m = read_polymesh(os.path.join(root, "HopeFOAM-0.1", "tutorials", "DG", "2D", "cylinder", "constant",
                                   "polyMesh"))
    g = golden_mesh("cylinder")
    assert sorted(m.curves) == ["downcylinder", "upcylinder"]
    assert np.array_equal(m.EToV, g.EToV) and np.array_equal(m.VXY, g.VXY)
    for n in m.curves:
        u = np.linspace(*m.curves[n].u_range, 7)
        assert np.allclose(np.array(m.curves[n].point(u)), np.array(g.curves[n].point(u)), atol=0, rtol=0)
