"""Host checks of the facts the two-pass FP32 SIPG apply builds on (no GPU).

The first pass writes, per element face, the trace and the outward normal
derivative at the face's Gauss points in the element's own traversal order;
the second pass reads the neighbour's record of the shared face at Gauss
point Nfq-1-g when the neighbour traverses the face the other way (ROT = 1)
and takes minus its normal derivative.  That needs: (1) the face
interpolation to Gauss points is symmetric under reversing both the face
nodes and the Gauss points; (2) on a conforming counter-clockwise mesh the
two sides traverse every interior face in opposite directions, node for node;
(3) the metric-based outward normals of the two sides are negatives of each
other."""
import numpy as np
import pytest

from conftest import golden_mesh


@pytest.fixture(scope="module")
def lib():
    from hopefoam_gb300 import build

    build.build()
    from hopefoam_gb300 import _lib

    return _lib.lib()


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5])
def test_face_interpolation_is_reversal_symmetric(lib, N):
    from hopefoam_gb300 import euler

    If = euler.reference_operators(N)["If"]  # (Nfq, Nfp): face nodes in face direction -> Gauss points
    assert If.shape == (N + 2, N + 1)
    assert np.abs(If - If[::-1, ::-1]).max() < 1e-14


def _normals(mesh):
    """Outward unit normals per (element, face) from the element metrics, the
    formula of the device code (face 0: -grad s, face 1: grad r + grad s,
    face 2: -grad r)."""
    V = mesh.VXY  # (K, 3, 2): each element's vertex coordinates
    xr, yr = 0.5 * (V[:, 1, 0] - V[:, 0, 0]), 0.5 * (V[:, 1, 1] - V[:, 0, 1])
    xs, ys = 0.5 * (V[:, 2, 0] - V[:, 0, 0]), 0.5 * (V[:, 2, 1] - V[:, 0, 1])
    J = xr * ys - xs * yr
    rx, sx, ry, sy = ys / J, -yr / J, -xs / J, xr / J
    g = np.stack([np.stack([-sx, -sy], -1), np.stack([rx + sx, ry + sy], -1), np.stack([-rx, -ry], -1)], 1)
    return g / np.linalg.norm(g, axis=-1, keepdims=True)


@pytest.mark.parametrize("which", ["delaunay", "periodic", "doublemach"])
def test_shared_faces_run_opposite_with_opposite_normals(lib, which):
    from hopefoam_gb300 import euler
    from hopefoam_gb300.mesh import delaunay_square, periodic_square

    N = 4
    if which == "delaunay":
        mesh = delaunay_square(300, seed=3)
    elif which == "periodic":
        mesh = periodic_square(6, 5, 2.0, 1.5, perturb=0.15, seed=2)
    else:
        mesh = golden_mesh("doublemach")
    ops = euler.reference_operators(N)
    x, y = euler.node_coords(mesh, ops["r"], ops["s"])
    fn_nodes = euler.face_nodes(N)
    kk, ff = np.nonzero(mesh.EToE >= 0)
    nb, fb = mesh.EToE[kk, ff], mesh.EToF[kk, ff]
    # (2) every interior face is traversed the other way by the neighbour
    assert (mesh.ROT[kk, ff] == 1).all()
    if which != "periodic":  # periodic images sit a period apart: compare geometry only within the box
        own = np.stack([x[kk[:, None], fn_nodes[ff]], y[kk[:, None], fn_nodes[ff]]], -1)
        oth = np.stack([x[nb[:, None], fn_nodes[fb]], y[nb[:, None], fn_nodes[fb]]], -1)
        assert np.abs(own - oth[:, ::-1]).max() < 1e-12
    # (3) the two outward normals of a shared face are negatives of each other
    n = _normals(mesh)
    assert np.abs(n[kk, ff] + n[nb, fb]).max() < 1e-12
