"""Reader for 2D Fluent/GAMBIT ASCII ``.msh`` triangle meshes (the format of
HopeFOAM's isentropic-vortex and Pearson-vortex tutorial meshes, e.g.
tutorials/DG/2D/isentropicVortex/vortex0256.msh).

Sections used: ``(10 ...)`` nodes (x y per line), ``(13 (zone first last
bc type)( ... ))`` faces (``[2] n0 n1 c0 c1`` in hex, c1 = 0 on a boundary),
``(12 ...)`` cell count, ``(45 (zone type name)())`` zone names.  Triangles are
rebuilt from their three edges and made counter-clockwise; boundary faces are
tagged Dirichlet (the tutorial's exact fixed-value boundary) and carry the name
of their face zone as their patch (``Mesh.patch`` / ``Mesh.patch_names``).
"""
import re

import numpy as np

from .mesh import Mesh, connect, make_ccw


def read_fluent_msh(path):
    text = open(path).read()
    nodes = []
    faces = []
    pos = 0
    pat = re.compile(r"\((10|13|12)\s*\(([0-9a-fA-F\s]+)\)\s*(\()?")
    while True:
        m = pat.search(text, pos)
        if not m:
            break
        sec = m.group(1)
        hdr = m.group(2).split()
        pos = m.end()
        if m.group(3) is None:
            continue
        end = text.index(")", pos)
        body = text[pos:end]
        pos = end + 1
        if sec == "10":
            vals = np.array(body.split(), dtype=np.float64).reshape(-1, 2)
            nodes.append((int(hdr[1], 16), vals))
        elif sec == "13":
            ftype = int(hdr[4], 16) if len(hdr) > 4 else 0
            toks = body.split()
            i = 0
            while i < len(toks):
                if ftype == 0 or ftype == 5:
                    n = int(toks[i], 16)
                    i += 1
                else:
                    n = 2
                ids = [int(t, 16) for t in toks[i:i + n + 2]]
                i += n + 2
                faces.append(ids + [int(hdr[0], 16)])
    zone_names = {int(z): name for z, name in re.findall(r"\(45\s*\(\s*(\d+)\s+\S+\s+(\S+?)\)", text)}
    nodes.sort()
    P = np.concatenate([v for _, v in nodes])
    faces = np.array(faces, dtype=np.int64)  # n0 n1 c0 c1 zone (1-based, c=0 none)
    ncell = int(max(faces[:, 2].max(), faces[:, 3].max()))
    edges = [[] for _ in range(ncell)]
    for n0, n1, c0, c1, _ in faces:
        for c in (c0, c1):
            if c > 0:
                edges[c - 1].append((n0 - 1, n1 - 1))
    EToV = np.empty((ncell, 3), np.int32)
    for c, es in enumerate(edges):
        if len(es) != 3:
            raise ValueError("cell %d has %d edges (only triangles supported)" % (c, len(es)))
        a, b = es[0]
        rest = es[1:]
        third = [v for e in rest for v in e if v not in (a, b)][0]
        EToV[c] = (a, b, third)
    VXY = P[EToV]
    EToV, VXY = make_ccw(EToV, VXY)
    EToE, EToF, ROT, BC = connect(EToV)
    # patches: the zone of each boundary face, matched on its vertex pair
    bzones = sorted({int(z) for n0, n1, c0, c1, z in faces if c0 == 0 or c1 == 0})
    names = tuple(zone_names.get(z, "zone%d" % z) for z in bzones)
    edge_zone = {(min(n0, n1) - 1, max(n0, n1) - 1): bzones.index(int(z)) for n0, n1, c0, c1, z in faces if c0 == 0 or c1 == 0}
    patch = -np.ones((ncell, 3), np.int32)
    kf_of_edge = {}
    for k, f in zip(*np.nonzero(EToE < 0)):
        a, b = int(EToV[k, f]), int(EToV[k, (f + 1) % 3])
        patch[k, f] = edge_zone[(min(a, b), max(a, b))]
        kf_of_edge[(min(a, b), max(a, b))] = (int(k), int(f))
    m = Mesh(EToV, VXY, EToE, EToF, ROT, BC, name=path.split("/")[-1], patch=patch, patch_names=names)
    # each patch's first face in file order (the reference's patch face order)
    first = {}
    for n0, n1, c0, c1, z in faces:
        if c0 == 0 or c1 == 0:
            pid = bzones.index(int(z))
            if pid not in first:
                first[pid] = kf_of_edge[(min(n0, n1) - 1, max(n0, n1) - 1)]
    m.patch_first_face = np.array([first[i] for i in range(len(names))], np.int32)
    return m
