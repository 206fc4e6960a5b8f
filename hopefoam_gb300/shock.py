"""The double-Mach-reflection case of the reference's tutorial
(tutorials/DG/2D/doubleMach): a Mach-10 shock at 60 degrees to a reflecting
wall, advanced with the limited SSP-RK2 step (include/dgcu.h:
dg_limited_ssprk2_step).

DoubleMach restates setNonUniformInlet.H (the initial state) and
setBoundaryValues.H (the moving shock's values on the far / inlet / outlet
patches at time t; the wall patch is reflective), and gives the boundary kinds
and the slot whose first value each fixed-value ghost cell takes (the first
face of its patch in the mesh file, Trianglelimite.C:182-185).
"""
import numpy as np

from .euler import boundary_faces, face_nodes, node_coords, reference_operators

GAMMA = 1.4
POST = (8.0, 8.25 * np.cos(np.pi / 6.0) * 8.0, -8.25 * np.sin(np.pi / 6.0) * 8.0, 116.5)  # rho, rhou, rhov, p
PRE = (1.4, 0.0, 0.0, 1.0)


def _state(x, y, t, gamma=GAMMA):
    g = (1 + 20 * t) / np.sqrt(3.0)
    behind = (1.0 / g * (x - 1.0 / 6.0) - y) < 0
    out = []
    for post, pre in zip(POST[:3], PRE[:3]):
        out.append(np.where(behind, post, pre))
    rho, ru, rv = out
    p = np.where(behind, POST[3], PRE[3])
    E = p / (gamma - 1.0) + (ru * ru + rv * rv) / (2 * rho)
    return np.stack([rho, ru, rv, E])


class DoubleMach:
    def __init__(self, mesh, order):
        self.mesh, self.order = mesh, order
        ops = reference_operators(order)
        self.x, self.y = node_coords(mesh, ops["r"], ops["s"])
        kk, ff = boundary_faces(mesh)
        fn = face_nodes(order)[ff]
        self.bx, self.by = self.x[kk[:, None], fn], self.y[kk[:, None], fn]
        names = list(mesh.patch_names)
        pid = mesh.patch[kk, ff]
        self.kinds = np.where(pid == names.index("wall"), 1, 0).astype(np.int32)
        slot_of = {(int(k), int(f)): s for s, (k, f) in enumerate(zip(kk, ff))}
        if mesh.patch_first_face is not None:
            first = [slot_of[(int(k), int(f))] for k, f in mesh.patch_first_face]
            self.gref = np.array([first[p] for p in pid], np.int32)
        else:
            self.gref = np.arange(len(kk), dtype=np.int32)

    def initial_state(self):
        return _state(self.x, self.y, 0.0)

    def bdata(self, t):
        """(n_bfaces, 4, Nfp) values of the fixed-value slots at time t."""
        return np.ascontiguousarray(_state(self.bx, self.by, t).transpose(1, 0, 2))
