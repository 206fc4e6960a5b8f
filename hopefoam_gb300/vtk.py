"""Legacy-VTK output of DG fields (the role of the reference's dgToVTK utility,
applications/utilities/DG/dgToVTK: each order-N triangle is split into N^2
linear triangles over its nodal lattice, vtkTopo.C; points are the element's
own nodes, so the file shows the discontinuous solution as it is).

write_vtk(path, mesh, order, fields): fields maps a name to a (K, Np) scalar
or (K, Np, 2|3) vector array in the reference node order.
"""
import numpy as np

from .euler import node_coords, reference_operators


def lattice_triangles(order):
    """Sub-triangles of the reference node lattice, counter-clockwise: nodes are
    numbered row by row from s = -1 (row i has N + 1 - i nodes)."""
    N = order
    idx = {}
    c = 0
    for i in range(N + 1):
        for j in range(N + 1 - i):
            idx[(i, j)] = c
            c += 1
    tris = []
    for i in range(N):
        for j in range(N - i):
            tris.append((idx[(i, j)], idx[(i, j + 1)], idx[(i + 1, j)]))
            if j < N - i - 1:
                tris.append((idx[(i, j + 1)], idx[(i + 1, j + 1)], idx[(i + 1, j)]))
    return np.array(tris, np.int64)


def write_vtk(path, mesh, order, fields, title="hopefoam_gb300"):
    ops = reference_operators(order)
    x, y = node_coords(mesh, ops["r"], ops["s"])
    K, Np = x.shape
    tri = lattice_triangles(order)
    cells = (tri[None, :, :] + (np.arange(K) * Np)[:, None, None]).reshape(-1, 3)
    with open(path, "w") as f:
        f.write("# vtk DataFile Version 3.0\n%s\nASCII\nDATASET UNSTRUCTURED_GRID\n" % title)
        f.write("POINTS %d double\n" % (K * Np))
        np.savetxt(f, np.c_[x.reshape(-1), y.reshape(-1), np.zeros(K * Np)], fmt="%.17g")
        f.write("CELLS %d %d\n" % (len(cells), 4 * len(cells)))
        np.savetxt(f, np.c_[np.full(len(cells), 3), cells], fmt="%d")
        f.write("CELL_TYPES %d\n" % len(cells))
        np.savetxt(f, np.full(len(cells), 5), fmt="%d")  # VTK_TRIANGLE
        if fields:
            f.write("POINT_DATA %d\n" % (K * Np))
        for name, v in fields.items():
            v = np.asarray(v, np.float64)
            if v.ndim == 2:
                f.write("SCALARS %s double 1\nLOOKUP_TABLE default\n" % name)
                np.savetxt(f, v.reshape(-1), fmt="%.17g")
            else:
                w = v.reshape(K * Np, -1)
                if w.shape[1] == 2:
                    w = np.c_[w, np.zeros(len(w))]
                f.write("VECTORS %s double\n" % name)
                np.savetxt(f, w, fmt="%.17g")


def read_vtk(path):
    """Points, triangles and point data of a file written by write_vtk."""
    toks = open(path).read().split("\n")
    out = {"data": {}}
    i = 0
    while i < len(toks):
        t = toks[i].split()
        if not t:
            i += 1
            continue
        if t[0] == "POINTS":
            n = int(t[1])
            out["points"] = np.loadtxt(toks[i + 1:i + 1 + n]).reshape(n, 3)
            i += 1 + n
        elif t[0] == "CELLS":
            n = int(t[1])
            out["cells"] = np.loadtxt(toks[i + 1:i + 1 + n], dtype=np.int64).reshape(n, 4)[:, 1:]
            i += 1 + n
        elif t[0] == "SCALARS":
            n = len(out["points"])
            out["data"][t[1]] = np.loadtxt(toks[i + 2:i + 2 + n]).reshape(n)
            i += 2 + n
        elif t[0] == "VECTORS":
            n = len(out["points"])
            out["data"][t[1]] = np.loadtxt(toks[i + 1:i + 1 + n]).reshape(n, 3)
            i += 1 + n
        else:
            i += 1
    return out
