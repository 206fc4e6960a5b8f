"""Triangle meshes for the DG hot path: descriptors plus the synthetic generators.

A mesh descriptor carries, per element k and local face f (faces are the edges
(v0,v1), (v1,v2), (v2,v0) of a counter-clockwise triangle, as in HopeFOAM's
dgPolyMesh.C:601-613):

* ``EToV[k]``   global vertex ids.  Periodic images share one id, so periodic
  faces are ordinary interior faces (HopeFOAM compiles no cyclic dgPatch;
  periodicity here is connectivity).
* ``VXY[k]``    the element's own vertex coordinates (unwrapped across the
  periodic boundary), shape (K, 3, 2).
* ``EToE[k,f]`` neighbour element (-1 on a boundary), ``EToF[k,f]`` the
  neighbour's local face, ``ROT[k,f]`` 1 when the neighbour traverses the edge
  in the opposite direction (the reference's ``firstPointIndex``,
  dgPolyMesh.C:866-893; always 1 for conforming counter-clockwise meshes).
* ``BC[k,f]``   0 interior, 1 Dirichlet / fixed-value boundary.
"""
from dataclasses import dataclass

import numpy as np


@dataclass
class Mesh:
    EToV: np.ndarray
    VXY: np.ndarray
    EToE: np.ndarray
    EToF: np.ndarray
    ROT: np.ndarray
    BC: np.ndarray
    name: str = ""
    # boundary patches (from mesh files): patch[k, f] = index into patch_names
    # for a boundary face, -1 for an interior face; None when not read from a file
    patch: np.ndarray = None
    patch_names: tuple = ()
    patch_first_face: np.ndarray = None  # per patch (k, f) of its first face in the file's order
    # curved patches: patch name -> curved.ArcCurve; their faces' nodes lie on the curve
    curves: dict = None

    @property
    def K(self):
        return int(self.EToV.shape[0])

    def min_h(self):
        """Smallest element length scale 2*area/longest edge."""
        v = self.VXY
        a = v[:, 1] - v[:, 0]
        b = v[:, 2] - v[:, 0]
        area = 0.5 * np.abs(a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0])
        e = np.stack([np.linalg.norm(v[:, (i + 1) % 3] - v[:, i], axis=1) for i in range(3)], 1)
        return float(np.min(2 * area / e.max(1)))


def make_ccw(EToV, VXY):
    """Reorder vertices counter-clockwise (dgPolyMesh.C:486-506)."""
    EToV = EToV.copy()
    VXY = VXY.copy()
    a = VXY[:, 1] - VXY[:, 0]
    b = VXY[:, 2] - VXY[:, 0]
    cw = (a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]) < 0
    EToV[cw, 1], EToV[cw, 2] = EToV[cw, 2].copy(), EToV[cw, 1].copy()
    VXY[cw, 1], VXY[cw, 2] = VXY[cw, 2].copy(), VXY[cw, 1].copy()
    return EToV, VXY


def connect(EToV):
    """Face-to-face connectivity by matching edges on their vertex-id pairs."""
    K = EToV.shape[0]
    a = EToV
    b = np.roll(EToV, -1, axis=1)
    lo = np.minimum(a, b).reshape(-1).astype(np.int64)
    hi = np.maximum(a, b).reshape(-1).astype(np.int64)
    key = lo * (int(EToV.max()) + 1) + hi
    order = np.argsort(key, kind="stable")
    ks = key[order]
    EToE = -np.ones(3 * K, np.int32)
    EToF = -np.ones(3 * K, np.int32)
    same = np.nonzero(ks[1:] == ks[:-1])[0]
    if np.any(np.diff(same) == 1):
        raise ValueError("an edge is shared by more than two triangles")
    i1 = order[same]
    i2 = order[same + 1]
    EToE[i1] = i2 // 3
    EToF[i1] = i2 % 3
    EToE[i2] = i1 // 3
    EToF[i2] = i1 % 3
    EToE = EToE.reshape(K, 3)
    EToF = EToF.reshape(K, 3)
    ROT = np.zeros((K, 3), np.int32)
    kk, ff = np.nonzero(EToE >= 0)
    n = EToE[kk, ff]
    fn = EToF[kk, ff]
    first = EToV[kk, ff]
    ROT[kk, ff] = np.where(first == EToV[n, (fn + 1) % 3], 1, 0)
    BC = (EToE < 0).astype(np.int32)
    return EToE, EToF, ROT, BC


def periodic_square(nx, ny, Lx=10.0, Ly=10.0, x0=0.0, y0=0.0, perturb=0.0, seed=0, name=""):
    """Periodic [x0,x0+Lx]x[y0,y0+Ly] grid of nx*ny squares, each cut into two
    counter-clockwise triangles on the (0,0)-(1,1) diagonal.  Vertices move by
    a seeded uniform U(-perturb*h, perturb*h) per coordinate; periodic images
    move together.  Element order: k = 2*(j*nx + i) + t."""
    hx, hy = Lx / nx, Ly / ny
    rng = np.random.default_rng(seed)
    d = np.zeros((ny, nx, 2))
    if perturb > 0:
        d[..., 0] = rng.uniform(-perturb * hx, perturb * hx, size=(ny, nx))
        d[..., 1] = rng.uniform(-perturb * hy, perturb * hy, size=(ny, nx))
    j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    i = i.reshape(-1)
    j = j.reshape(-1)

    def vid(ii, jj):
        return (jj % ny) * nx + (ii % nx)

    def pos(ii, jj):
        p = np.stack([x0 + ii * hx, y0 + jj * hy], -1).astype(np.float64)
        return p + d[jj % ny, ii % nx]

    v00, v10, v11, v01 = vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)
    p00, p10, p11, p01 = pos(i, j), pos(i + 1, j), pos(i + 1, j + 1), pos(i, j + 1)
    EToV = np.empty((2 * nx * ny, 3), np.int32)
    VXY = np.empty((2 * nx * ny, 3, 2))
    EToV[0::2] = np.stack([v00, v10, v11], 1)
    EToV[1::2] = np.stack([v00, v11, v01], 1)
    VXY[0::2] = np.stack([p00, p10, p11], 1)
    VXY[1::2] = np.stack([p00, p11, p01], 1)
    EToV, VXY = make_ccw(EToV, VXY)
    EToE, EToF, ROT, BC = connect(EToV)
    return Mesh(EToV, VXY, EToE, EToF, ROT, BC, name or "periodic_%dx%dx2" % (nx, ny))


def box_square(nx, ny, Lx, Ly, x0=0.0, y0=0.0, name=""):
    """Non-periodic structured box (boundary faces tagged Dirichlet)."""
    hx, hy = Lx / nx, Ly / ny
    j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    i = i.reshape(-1)
    j = j.reshape(-1)

    def vid(ii, jj):
        return jj * (nx + 1) + ii

    def pos(ii, jj):
        return np.stack([x0 + ii * hx, y0 + jj * hy], -1).astype(np.float64)

    EToV = np.empty((2 * nx * ny, 3), np.int32)
    VXY = np.empty((2 * nx * ny, 3, 2))
    EToV[0::2] = np.stack([vid(i, j), vid(i + 1, j), vid(i + 1, j + 1)], 1)
    EToV[1::2] = np.stack([vid(i, j), vid(i + 1, j + 1), vid(i, j + 1)], 1)
    VXY[0::2] = np.stack([pos(i, j), pos(i + 1, j), pos(i + 1, j + 1)], 1)
    VXY[1::2] = np.stack([pos(i, j), pos(i + 1, j + 1), pos(i, j + 1)], 1)
    EToE, EToF, ROT, BC = connect(EToV)
    return Mesh(EToV, VXY, EToE, EToF, ROT, BC, name or "box_%dx%dx2" % (nx, ny))


def delaunay_square(n_interior, L=2 * np.pi, n_edge=None, seed=0, jitter=0.35, uniform=False, name=""):
    """Unstructured Delaunay triangulation of [0,L]^2 from a seeded point set
    plus evenly spaced boundary points; boundary faces are Dirichlet.  About
    2*n_interior triangles.  The interior points are a jittered lattice
    (each point moved by U(-jitter*h, jitter*h) per coordinate), which keeps
    the triangles well shaped; uniform=True draws them i.i.d. uniform instead
    (slivers, much worse conditioning)."""
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    if n_edge is None:
        n_edge = max(4, int(round(np.sqrt(n_interior))))
    t = np.linspace(0, L, n_edge + 1)[:-1]
    bnd = np.concatenate([
        np.stack([t, np.zeros_like(t)], 1),
        np.stack([np.full_like(t, L), t], 1),
        np.stack([L - t, np.full_like(t, L)], 1),
        np.stack([np.zeros_like(t), L - t], 1),
    ])
    margin = 0.25 * L / n_edge
    if uniform:
        pts = rng.uniform(margin, L - margin, size=(n_interior, 2))
    else:
        m = max(2, int(round(np.sqrt(n_interior))))
        h = L / (m + 1)
        g = (np.arange(m) + 1) * h
        X, Y = np.meshgrid(g, g, indexing="ij")
        pts = np.stack([X.reshape(-1), Y.reshape(-1)], 1)
        pts = pts + rng.uniform(-jitter * h, jitter * h, size=pts.shape)
    P = np.concatenate([bnd, pts])
    tri = Delaunay(P)
    EToV = tri.simplices.astype(np.int32)
    VXY = P[EToV]
    # drop degenerate slivers (zero area) if any
    a = VXY[:, 1] - VXY[:, 0]
    b = VXY[:, 2] - VXY[:, 0]
    area = 0.5 * (a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0])
    keep = np.abs(area) > 1e-14 * L * L
    EToV, VXY = make_ccw(EToV[keep], VXY[keep])
    EToE, EToF, ROT, BC = connect(EToV)
    return Mesh(EToV, VXY, EToE, EToF, ROT, BC, name or "delaunay_%d" % EToV.shape[0])


def load_cubature(strength):
    """Triangle cubature rule (r, s, w) of the given strength from the package
    data file (the reference's table, see data/make_tri_cubature.py)."""
    import os

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "tri_cubature.txt")
    with open(path) as f:
        lines = [l for l in f.read().split("\n") if l and not l.startswith("#")]
    i = 0
    while i < len(lines):
        _, q, n = lines[i].split()
        q, n = int(q), int(n)
        if q == strength:
            return np.array([[float(x) for x in l.split()] for l in lines[i + 1:i + 1 + n]])
        i += n + 1
    raise KeyError("no cubature rule of strength %d" % strength)
