"""OpenFOAM polyMesh I/O for 2D DG cases, and DG field files.

read_polymesh: a 2D case is one layer of prisms between two planes; HopeFOAM
takes each cell's face that lies in the z = 0 plane as the triangle, in the
face's own point order, and swaps its last two points when they run clockwise
seen from +z (dgPolyMesh.C:154-183 picks the face, :489-506 reorders).  The
other boundary patches (side faces, two points in the z = 0 plane) become the
triangles' boundary edges, tagged with their patch (``Mesh.patch``); patches
of type ``empty`` (the two planes) are not edges.  Patches of type ``arc``
carry their curve (``Mesh.curves``, curved.read_arc_patches).  Only triangles
(prism cells) are read; quads (hex cells) are outside this triangle-only path.

write_polymesh writes a Mesh as such a one-layer prism mesh (points at z = 0
and z = dz, the z = 0 triangles as the cells' first face), so that cases can
be exported to the reference's tools and read back.

read_dg_field / write_dg_field: the ``internalField nonuniform List<scalar>``
(or ``List<vector>``) form of a DG field, one entry per node in element order
(the layout of the reference's dof fields, GeometricDofField.H).
"""
import os
import re

import numpy as np

from .mesh import Mesh, connect, make_ccw

_HEADER = """/*--------------------------------*- C++ -*----------------------------------*\\
  written by hopefoam_gb300
\\*---------------------------------------------------------------------------*/
FoamFile
{
    version     2.0;
    format      ascii;
    class       %s;
    location    "%s";
    object      %s;
}
// * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * //

"""


def _strip(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    # drop the FoamFile header dictionary
    m = re.search(r"FoamFile\s*\{.*?\}", text, flags=re.S)
    if m:
        text = text[:m.start()] + text[m.end():]
    return text


def _list_body(text):
    """The body of the first top-level 'N ( ... )' list."""
    m = re.search(r"(\d+)\s*\(", text)
    if not m:
        raise ValueError("no list found")
    n = int(m.group(1))
    depth, i = 1, m.end()
    start = i
    while depth:
        c = text[i]
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
        i += 1
    return n, text[start:i - 1]


def _read(path):
    with open(path) as f:
        return _strip(f.read())


def _points(path):
    n, body = _list_body(_read(path))
    vals = np.array(body.replace("(", " ").replace(")", " ").split(), dtype=np.float64)
    return vals.reshape(n, 3)


def _faces(path):
    n, body = _list_body(_read(path))
    faces = [tuple(int(v) for v in g.split()) for g in re.findall(r"\d+\s*\(([^)]*)\)", body)]
    if len(faces) != n:
        raise ValueError("%s: %d faces declared, %d read" % (path, n, len(faces)))
    return faces


def _labels(path):
    n, body = _list_body(_read(path))
    vals = np.array(body.split(), dtype=np.int64)
    if vals.size != n:
        raise ValueError("%s: %d labels declared, %d read" % (path, n, vals.size))
    return vals


def _boundary(path):
    n, body = _list_body(_read(path))
    out = []
    for name, entries in re.findall(r"(\w+)\s*\{([^}]*)\}", body):
        d = dict(re.findall(r"(\w+)\s+([^;]+);", entries))
        out.append((name, d.get("type", "patch").strip(), int(d["nFaces"]), int(d["startFace"])))
    if len(out) != n:
        raise ValueError("%s: %d patches declared, %d read" % (path, n, len(out)))
    return out


def _polymesh_dir(path):
    for cand in (path, os.path.join(path, "constant", "polyMesh"), os.path.join(path, "polyMesh")):
        if os.path.exists(os.path.join(cand, "points")):
            return cand
    raise FileNotFoundError("no polyMesh under %s" % path)


def read_polymesh(path):
    """Mesh of the triangles of a one-layer prism polyMesh (case directory or
    constant/polyMesh directory)."""
    d = _polymesh_dir(path)
    P = _points(os.path.join(d, "points"))
    faces = _faces(os.path.join(d, "faces"))
    owner = _labels(os.path.join(d, "owner"))
    neighbour = _labels(os.path.join(d, "neighbour"))
    patches = _boundary(os.path.join(d, "boundary"))
    ncell = int(max(owner.max(), neighbour.max() if neighbour.size else -1)) + 1
    on_plane = P[:, 2] == 0.0
    tri = -np.ones((ncell, 3), np.int64)
    for fi, f in enumerate(faces):
        if len(f) == 3 and all(on_plane[v] for v in f):
            c = owner[fi]
            if fi < neighbour.size:
                raise ValueError("a face in the z = 0 plane is internal")
            tri[c] = f
        elif all(on_plane[v] for v in f):
            raise ValueError("cell %d: only triangles are supported" % owner[fi])
    if (tri < 0).any():
        raise ValueError("%d cells have no triangle face in the z = 0 plane" % int((tri[:, 0] < 0).sum()))
    used = np.unique(tri)
    remap = -np.ones(P.shape[0], np.int64)
    remap[used] = np.arange(used.size)
    EToV = remap[tri].astype(np.int32)
    VXY = P[used][:, :2][EToV]
    EToV, VXY = make_ccw(EToV, VXY)
    EToE, EToF, ROT, BC = connect(EToV)
    names, edge_patch = [], {}
    for name, ptype, nf, start in patches:
        if ptype == "empty" or nf == 0:
            continue
        pid = len(names)
        names.append(name)
        for fi in range(start, start + nf):
            v = [remap[x] for x in faces[fi] if on_plane[x]]
            if len(v) != 2:
                raise ValueError("patch %s face %d does not cross the z = 0 plane in an edge" % (name, fi))
            edge_patch[(min(v), max(v))] = pid
    patch = -np.ones(EToV.shape, np.int32)
    for k, f in zip(*np.nonzero(EToE < 0)):
        a, b = int(EToV[k, f]), int(EToV[k, (f + 1) % 3])
        key = (min(a, b), max(a, b))
        if key not in edge_patch:
            raise ValueError("boundary edge %s of cell %d belongs to no patch" % (key, k))
        patch[k, f] = edge_patch[key]
    from .curved import read_arc_patches

    curves = {n: c for n, c in read_arc_patches(_read(os.path.join(d, "boundary"))).items() if n in names}
    return Mesh(EToV, VXY, EToE, EToF, ROT, BC, name=os.path.basename(os.path.dirname(os.path.dirname(d))) or d,
                patch=patch, patch_names=tuple(names), curves=curves or None)


def _write(path, cls, location, obj, body):
    with open(path, "w") as f:
        f.write(_HEADER % (cls, location, obj))
        f.write(body)
        f.write("\n// ************************************************************************* //\n")


def write_polymesh(mesh, path, dz=0.1, patch_names=None, patch=None):
    """Write `mesh` as a one-layer prism polyMesh under `path` (a case directory:
    files go to path/constant/polyMesh).  Boundary edges are grouped by
    `patch` (K x 3, default mesh.patch, else one patch "boundary"); the two
    planes form the patch "frontAndBack" of type empty."""
    K = mesh.K
    EToV = mesh.EToV
    nv = int(EToV.max()) + 1
    xy = np.zeros((nv, 2))
    xy[EToV.reshape(-1)] = mesh.VXY.reshape(-1, 2)
    pts = np.concatenate([np.c_[xy, np.zeros(nv)], np.c_[xy, np.full(nv, dz)]])
    if patch is None:
        patch = mesh.patch if mesh.patch is not None else np.where(mesh.EToE < 0, 0, -1)
    if patch_names is None:
        patch_names = mesh.patch_names if mesh.patch_names else ("boundary",)
    internal, bnd = [], [[] for _ in patch_names]
    for k in range(K):
        for f in range(3):
            a, b = int(EToV[k, f]), int(EToV[k, (f + 1) % 3])
            quad = (a, b, b + nv, a + nv)  # outward normal for a counter-clockwise triangle
            n = int(mesh.EToE[k, f])
            if n < 0:
                bnd[int(patch[k, f])].append((k, quad))
            elif k < n:
                internal.append((k, n, quad))
    faces, owner, neighbour = [], [], []
    for k, n, quad in sorted(internal, key=lambda t: (t[0], t[1])):
        faces.append(quad)
        owner.append(k)
        neighbour.append(n)
    starts = []
    for lst in bnd:
        starts.append(len(faces))
        for k, quad in lst:
            faces.append(quad)
            owner.append(k)
    start_fb = len(faces)
    for k in range(K):
        a, b, c = (int(v) for v in EToV[k])
        faces.append((a, c, b))  # z = 0: normal -z
        owner.append(k)
    for k in range(K):
        a, b, c = (int(v) for v in EToV[k])
        faces.append((a + nv, b + nv, c + nv))  # z = dz: normal +z
        owner.append(k)
    d = os.path.join(path, "constant", "polyMesh")
    os.makedirs(d, exist_ok=True)
    loc = "constant/polyMesh"
    _write(os.path.join(d, "points"), "vectorField", loc, "points",
           "%d\n(\n%s\n)\n" % (len(pts), "\n".join("(%.17g %.17g %.17g)" % tuple(p) for p in pts)))
    _write(os.path.join(d, "faces"), "faceList", loc, "faces",
           "%d\n(\n%s\n)\n" % (len(faces), "\n".join("%d(%s)" % (len(f), " ".join(map(str, f))) for f in faces)))
    _write(os.path.join(d, "owner"), "labelList", loc, "owner",
           "%d\n(\n%s\n)\n" % (len(owner), "\n".join(map(str, owner))))
    _write(os.path.join(d, "neighbour"), "labelList", loc, "neighbour",
           "%d\n(\n%s\n)\n" % (len(neighbour), "\n".join(map(str, neighbour))))
    entries = []
    for name, lst, st in zip(patch_names, bnd, starts):
        entries.append("    %s\n    {\n        type            patch;\n        nFaces          %d;\n"
                       "        startFace       %d;\n    }" % (name, len(lst), st))
    entries.append("    frontAndBack\n    {\n        type            empty;\n        nFaces          %d;\n"
                   "        startFace       %d;\n    }" % (2 * K, start_fb))
    _write(os.path.join(d, "boundary"), "polyBoundaryMesh", loc, "boundary",
           "%d\n(\n%s\n)\n" % (len(entries), "\n".join(entries)))


def write_dg_field(path, name, values, dimensions="[0 0 0 0 0 0 0]", boundary=None, time="0"):
    """Write a DG field: values (K, Np) scalar or (K, Np, 2|3) vector, node order
    within each element as the element's nodes (z = 0 appended for 2-vectors)."""
    v = np.asarray(values, dtype=np.float64)
    if v.ndim == 2:
        cls, typ = "dgScalarField", "scalar"
        items = "\n".join("%.17g" % x for x in v.reshape(-1))
        n = v.size
    else:
        cls, typ = "dgVectorField", "vector"
        flat = v.reshape(-1, v.shape[-1])
        if flat.shape[1] == 2:
            flat = np.c_[flat, np.zeros(len(flat))]
        items = "\n".join("(%.17g %.17g %.17g)" % tuple(r) for r in flat)
        n = len(flat)
    bnd = boundary or {}
    bbody = "\n".join("    %s\n    {\n%s    }" % (k, "".join("        %s %s;\n" % kv for kv in b.items()))
                      for k, b in bnd.items())
    body = ("dimensions      %s;\n\ninternalField   nonuniform List<%s>\n%d\n(\n%s\n)\n;\n\nboundaryField\n{\n%s\n}\n"
            % (dimensions, typ, n, items, bbody))
    _write(path, cls, time, name, body)


def read_dg_field(path, K=None):
    """internalField of a DG field file: (n,) for scalars, (n, 3) for vectors;
    reshaped to (K, -1[, 3]) when K is given.  A uniform field returns its value."""
    text = _read(path)
    m = re.search(r"internalField\s+uniform\s+([^;]+);", text)
    if m:
        val = m.group(1).strip()
        return np.array(val.strip("()").split(), dtype=np.float64) if val.startswith("(") else float(val)
    m = re.search(r"internalField\s+nonuniform\s+List<(\w+)>", text)
    if not m:
        raise ValueError("%s: no internalField" % path)
    n, body = _list_body(text[m.end():])
    vals = np.array(body.replace("(", " ").replace(")", " ").split(), dtype=np.float64)
    out = vals.reshape(n, 3) if m.group(1) == "vector" else vals
    if out.shape[0] != n:
        raise ValueError("%s: %d values declared, %d read" % (path, n, out.shape[0]))
    if K is not None:
        out = out.reshape((K, -1) + out.shape[1:])
    return out
