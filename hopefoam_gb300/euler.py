"""Host-side Python mirror of the reference's Euler solver interface over the
C ABI (a thin layer: all arithmetic runs in libdgcu on the GPU).

``EulerContext`` stands for the reference's dgMesh + the three conserved
dgFields of dgEulerFoam (rho, rhoU, Ener; tutorials/DG/2D/isentropicVortex/
dgEulerFoam/createFields.H) and the per-stage ``dg::solveEquation`` calls
(dgEulerFoam.C:86-90).  States are numpy arrays of shape (4, K, Np) in the
reference node order: rho, rhoU.x, rhoU.y, Ener.
"""
import ctypes

import numpy as np

from . import _lib as L
from .mesh import load_cubature


def isentropic_vortex(x, y, t=0.0, beta=5.0, x0=5.0, y0=0.0, uinf=1.0, vinf=0.0, rho_inf=1.0, p_inf=1.0,
                      gamma=1.4):
    """Isentropic vortex at time t (form of setNonUniformInlet.H:20-26 /
    setBoundaryValues.H, generalised to a free stream (uinf, vinf) with
    rho_inf = p_inf = 1 giving the reference's case)."""
    dx = x - x0 - uinf * t
    dy = y - y0 - vinf * t
    r2 = dx * dx + dy * dy
    pi = np.pi
    rho = (1.0 - (gamma - 1.0) * beta ** 2 * np.exp(2.0 * (1.0 - r2)) / (16.0 * gamma * pi * pi)) ** (1.0 / (gamma - 1.0))
    u = uinf - beta * np.exp(1.0 - r2) * dy / (2.0 * pi)
    v = vinf + beta * np.exp(1.0 - r2) * dx / (2.0 * pi)
    rho = rho * rho_inf
    p = p_inf * (rho / rho_inf) ** gamma
    E = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    return np.stack([rho, rho * u, rho * v, E])


def kelvin_helmholtz(x, y, seed=0, gamma=1.4, noise=1e-3):
    """Periodic shear layer on [0,1]^2: rho = 2, u = 0.5 in |y - 0.5| < 0.25,
    rho = 1, u = -0.5 outside; p = 2.5; v = 0.01 sin(4 pi x) plus seeded
    uniform white noise of amplitude `noise` per node."""
    inside = np.abs(y - 0.5) < 0.25
    rho = np.where(inside, 2.0, 1.0)
    u = np.where(inside, 0.5, -0.5)
    rng = np.random.default_rng(seed)
    v = 0.01 * np.sin(4.0 * np.pi * x) + noise * rng.uniform(-1.0, 1.0, size=np.shape(x))
    p = np.full(np.shape(x), 2.5)
    E = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    return np.stack([rho, rho * u, rho * v, E])


def _check(ctx_handle, rc):
    if rc != L.DG_OK:
        msg = ""
        if ctx_handle:
            m = L.lib().dg_last_error(ctx_handle)
            msg = m.decode() if m else ""
        raise L.DGError(rc, msg)


class EulerContext:
    """One mesh + order on the GPU (C-ABI context)."""

    def __init__(self, mesh, order, gamma=1.4, cubature=None, stream=None):
        self.lib = L.lib()
        self.mesh = mesh
        self.order = order
        self.gamma = gamma
        self._keep = []
        cub = np.ascontiguousarray(load_cubature(3 * (order + 1)) if cubature is None else cubature, np.float64)
        arrays = dict(EToV=np.ascontiguousarray(mesh.EToV, np.int32), VXY=np.ascontiguousarray(mesh.VXY, np.float64),
                      EToE=np.ascontiguousarray(mesh.EToE, np.int32), EToF=np.ascontiguousarray(mesh.EToF, np.int32),
                      ROT=np.ascontiguousarray(mesh.ROT, np.int32), BC=np.ascontiguousarray(mesh.BC, np.int32))
        self._keep += list(arrays.values()) + [cub]
        md = L.MeshDesc(mesh.K, L.iptr(arrays["EToV"]), L.dptr(arrays["VXY"]), L.iptr(arrays["EToE"]),
                        L.iptr(arrays["EToF"]), L.iptr(arrays["ROT"]), L.iptr(arrays["BC"]))
        op = L.Opts(order, L.dptr(cub), cub.shape[0], gamma, ctypes.c_void_p(stream) if stream else None)
        h = ctypes.c_void_p()
        _check(None, self.lib.dg_ctx_create(ctypes.byref(md), ctypes.byref(op), ctypes.byref(h)))
        self.h = h
        info = L.Info()
        _check(self.h, self.lib.dg_get_info(self.h, ctypes.byref(info)))
        self.K, self.Np, self.Ng, self.Nfp, self.Nfq = info.K, info.Np, info.Ng, info.Nfp, info.Nfq
        self.n_bfaces = info.n_bfaces
        self.stream = info.stream
        self.device_bytes = info.device_bytes
        if getattr(mesh, "curves", None):  # nodes next to curved patches sit on their curves
            ops = reference_operators(order)
            self.set_node_locations(*node_coords(mesh, ops["r"], ops["s"]))

    def close(self):
        if getattr(self, "h", None):
            self.lib.dg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- state ---------------------------------------------------------
    def upload(self, q):
        q = np.ascontiguousarray(q, np.float64).reshape(-1)
        assert q.size == 4 * self.K * self.Np
        _check(self.h, self.lib.dg_upload_state(self.h, L.dptr(q)))

    def download(self):
        q = np.empty(4 * self.K * self.Np)
        _check(self.h, self.lib.dg_download_state(self.h, L.dptr(q)))
        return q.reshape(4, self.K, self.Np)

    def upload_device(self, ptr):
        _check(self.h, self.lib.dg_upload_state_device(self.h, ctypes.c_void_p(ptr)))

    def download_device(self, ptr):
        _check(self.h, self.lib.dg_download_state_device(self.h, ctypes.c_void_p(ptr)))

    def set_boundary_traces(self, traces):
        t = np.ascontiguousarray(traces, np.float64).reshape(-1)
        assert t.size == self.n_bfaces * 4 * self.Nfp
        _check(self.h, self.lib.dg_set_boundary_traces(self.h, L.dptr(t)))

    # --- hot path ------------------------------------------------------
    def rhs(self, flux=L.DG_FLUX_LF, precision=L.DG_PREC_FP64):
        out = np.empty(4 * self.K * self.Np)
        _check(self.h, self.lib.dg_euler_rhs(self.h, flux, precision, L.dptr(out)))
        return out.reshape(4, self.K, self.Np)

    def lserk4(self, dt, nsteps, flux=L.DG_FLUX_LF, precision=L.DG_PREC_FP64):
        _check(self.h, self.lib.dg_lserk4_step(self.h, float(dt), int(nsteps), flux, precision))

    def ssprk2(self, dt, nsteps, flux=L.DG_FLUX_ROE, precision=L.DG_PREC_FP64):
        _check(self.h, self.lib.dg_ssprk2_step(self.h, float(dt), int(nsteps), flux, precision))

    # --- limiter (shock cases) -------------------------------------------
    def set_node_locations(self, x, y):
        """Node locations (K, Np) read by the limiter (curved patches move them;
        the operators keep the straight element's metrics)."""
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        y = np.ascontiguousarray(y, np.float64).reshape(-1)
        assert x.size == self.K * self.Np and y.size == x.size
        _check(self.h, self.lib.dg_set_node_locations(self.h, L.dptr(x), L.dptr(y)))

    def set_boundary_kinds(self, kinds, gref=None):
        """Per boundary slot: 0 fixed value, 1 reflective wall, 2 other (value as
        set), 3 zero gradient (the interior trace)."""
        k = np.ascontiguousarray(kinds, np.int32)
        g = None if gref is None else np.ascontiguousarray(gref, np.int32)
        self._keep += [k] + ([g] if g is not None else [])
        _check(self.h, self.lib.dg_set_boundary_kinds(self.h, L.iptr(k), L.iptr(g) if g is not None else None))

    def limit(self):
        _check(self.h, self.lib.dg_limit(self.h))

    def reflect_boundary_traces(self):
        _check(self.h, self.lib.dg_reflect_boundary_traces(self.h))

    def limited_ssprk2(self, dt, bdata, flux=L.DG_FLUX_ROE, precision=L.DG_PREC_FP64):
        """One limited SSP-RK2 step; bdata (n_bfaces, 4, Nfp): this step's
        values of the fixed-value slots."""
        b = np.ascontiguousarray(bdata, np.float64).reshape(-1)
        _check(self.h, self.lib.dg_limited_ssprk2_step(self.h, float(dt), L.dptr(b), flux, precision))

    def cfl_dt(self, cfl):
        dt = np.zeros(1)
        _check(self.h, self.lib.dg_cfl_dt(self.h, float(cfl), L.dptr(dt)))
        return float(dt[0])


def reference_operators(order, cubature=None):
    """Host-only operator set of the library (reference node order)."""
    cub = np.ascontiguousarray(load_cubature(3 * (order + 1)) if cubature is None else cubature, np.float64)
    Np = (order + 1) * (order + 2) // 2
    Ng = cub.shape[0]
    Nfp, Nfq = order + 1, order + 2
    out = dict(r=np.zeros(Np), s=np.zeros(Np), Dr=np.zeros((Np, Np)), Ds=np.zeros((Np, Np)),
               Vg=np.zeros((Ng, Np)), If=np.zeros((Nfq, Nfp)), Mref=np.zeros((Np, Np)))
    rc = L.lib().dg_reference_operators(order, L.dptr(cub), Ng, *[L.dptr(out[k]) for k in
                                                                   ["r", "s", "Dr", "Ds", "Vg", "If", "Mref"]])
    _check(None, rc)
    return out


def face_nodes(order):
    """Reference node ids of each face's nodes in face direction,
    faceToCellIndex[f][0] of triangleBaseFunction.C:75-94; shape (3, N+1)."""
    N = order
    Np = (N + 1) * (N + 2) // 2
    f = np.zeros((3, N + 1), np.int64)
    f[0] = np.arange(N + 1)
    f[1, 0] = N
    f[2, 0] = Np - 1
    for i in range(1, N + 1):
        f[1, i] = f[1, i - 1] + (N + 1 - i)
        f[2, i] = f[2, i - 1] - i - 1
    return f


def boundary_faces(mesh):
    """(k, f) of the boundary faces in the order the C ABI indexes them."""
    kk, ff = np.nonzero(mesh.EToE < 0)
    return kk, ff


def boundary_traces_from_nodes(mesh, order, qnode_fn, x, y):
    """Fixed-value traces (n_bfaces, 4, Nfp): qnode_fn(x, y) -> (4, n) evaluated
    at each boundary face's nodes in face direction."""
    kk, ff = boundary_faces(mesh)
    fn = face_nodes(order)
    ids = fn[ff]  # (nb, Nfp)
    xs = x[kk[:, None], ids]
    ys = y[kk[:, None], ids]
    q = qnode_fn(xs.reshape(-1), ys.reshape(-1)).reshape(4, len(kk), -1)
    return np.ascontiguousarray(q.transpose(1, 0, 2))


def node_coords(mesh, r, s):
    """Physical node coordinates x(r,s) of every element (triangleBaseFunction.C:303-313),
    with the nodes next to curved patches moved onto their curves when the mesh
    carries curves (curved.curve_node_shift)."""
    v = mesh.VXY
    x = (-(r + s)[None, :] * 0.5 * v[:, 0, 0:1] + (r + 1)[None, :] * 0.5 * v[:, 1, 0:1]
         + (s + 1)[None, :] * 0.5 * v[:, 2, 0:1])
    y = (-(r + s)[None, :] * 0.5 * v[:, 0, 1:2] + (r + 1)[None, :] * 0.5 * v[:, 1, 1:2]
         + (s + 1)[None, :] * 0.5 * v[:, 2, 1:2])
    if getattr(mesh, "curves", None):
        from .curved import curve_node_shift

        order = int(round((np.sqrt(8 * len(r) + 1) - 3) / 2))
        x, y = curve_node_shift(mesh, order, x, y)
    return x, y
