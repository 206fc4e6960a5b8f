"""Incompressible Navier-Stokes on the GPU: the velocity-correction (Chorin)
step of the reference's dgChorinFoam (include/dgcu.h: dg_ins_*), and the
Pearson-vortex case of its tutorial (tutorials/DG/2D/pearsonVortex).

ChorinSolver mirrors the solver's time loop (dgChorinFoam.C:63-109): one
``step`` is convection, pressure Poisson solve, velocity correction and a
Helmholtz solve per velocity component, with BDF1/EXT1 on the first step and
BDF2/EXT2 after.  The boundary data of each step come from the caller
(``PearsonVortex.bdata`` restates setBoundaryValues.H, setparaT.H and the
exact-solution terms of pCorrectEquation.H for that case; ``CylinderFlow``
does the same for the cylinder tutorial, tutorials/DG/2D/cylinder, whose
curved patches move the boundary nodes the inflow is evaluated at).
"""
import ctypes

import numpy as np

from . import _lib as L
from .euler import boundary_faces, face_nodes, node_coords, reference_operators
from .mesh import load_cubature

PI = np.pi


class ChorinSolver:
    """u_kind / p_kind per boundary slot (boundary faces in element, face
    order): U 0 fixedValue / 1 fixedGradient, p 0 fixedValue / 2
    zeroGradient.  Default from the mesh patches: "inlet" -> U fixedValue, p
    zeroGradient; "outlet" -> U fixedGradient, p fixedValue (the tutorial's
    0/U and 0/p)."""

    def __init__(self, mesh, order, nu=0.01, dt=1e-3, tau_coef=20.0, u_kind=None, p_kind=None, precision=None):
        self.lib = L.lib()
        self.mesh, self.order, self.nu, self.dt = mesh, order, nu, dt
        kk, ff = boundary_faces(mesh)
        self.bk, self.bf = kk, ff
        if u_kind is None or p_kind is None:
            names = list(mesh.patch_names)
            pid = mesh.patch[kk, ff]
            inlet = pid == names.index("inlet")
            outlet = pid == names.index("outlet")
            if not np.all(inlet | outlet):
                raise ValueError("boundary faces outside the inlet and outlet patches need u_kind / p_kind")
            u_kind = np.where(inlet, 0, 1)
            p_kind = np.where(inlet, 2, 0)
        self.u_kind = np.ascontiguousarray(u_kind, np.int32)
        self.p_kind = np.ascontiguousarray(p_kind, np.int32)
        cub = np.ascontiguousarray(load_cubature(3 * (order + 1)), np.float64)
        arrays = dict(EToV=np.ascontiguousarray(mesh.EToV, np.int32), VXY=np.ascontiguousarray(mesh.VXY, np.float64),
                      EToE=np.ascontiguousarray(mesh.EToE, np.int32), EToF=np.ascontiguousarray(mesh.EToF, np.int32),
                      ROT=np.ascontiguousarray(mesh.ROT, np.int32), BC=np.ascontiguousarray(mesh.BC, np.int32))
        self._keep = list(arrays.values()) + [cub]
        md = L.MeshDesc(mesh.K, L.iptr(arrays["EToV"]), L.dptr(arrays["VXY"]), L.iptr(arrays["EToE"]),
                        L.iptr(arrays["EToF"]), L.iptr(arrays["ROT"]), L.iptr(arrays["BC"]))
        op = L.Opts(order, L.dptr(cub), cub.shape[0], 1.4, None)
        h = ctypes.c_void_p()
        rc = self.lib.dg_ins_create(ctypes.byref(md), ctypes.byref(op), L.iptr(self.u_kind), L.iptr(self.p_kind),
                                    float(nu), float(dt), float(tau_coef), ctypes.byref(h))
        if rc != L.DG_OK:
            raise L.DGError(rc, "dg_ins_create")
        self.h = h
        if precision is not None:  # arithmetic of the linear solves (FP64 by default)
            rc = self.lib.dg_ins_set_precision(self.h, int(precision))
            if rc != L.DG_OK:
                raise L.DGError(rc, "dg_ins_set_precision")
        self.K = mesh.K
        self.Np = (order + 1) * (order + 2) // 2
        self.Nfp = order + 1
        self.nb = len(kk)
        ops = reference_operators(order)
        self.x, self.y = node_coords(mesh, ops["r"], ops["s"])
        fn = face_nodes(order)[ff]  # (nb, Nfp) reference node ids in face-node order
        self.bx = self.x[kk[:, None], fn]
        self.by = self.y[kk[:, None], fn]
        v = mesh.VXY
        d = v[kk, (ff + 1) % 3] - v[kk, ff]
        ln = np.hypot(d[:, 0], d[:, 1])
        self.bnx, self.bny = d[:, 1] / ln, -d[:, 0] / ln  # outward normals of counter-clockwise triangles

    def _check(self, rc):
        if rc != L.DG_OK:
            m = self.lib.dg_ins_last_error(self.h)
            raise L.DGError(rc, m.decode() if m else "")

    def close(self):
        if getattr(self, "h", None):
            self.lib.dg_ins_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, U, p):
        U = np.ascontiguousarray(U, np.float64).reshape(-1)
        p = np.ascontiguousarray(p, np.float64).reshape(-1)
        self._check(self.lib.dg_ins_set_state(self.h, L.dptr(U), L.dptr(p)))

    def get_state(self):
        U = np.empty(2 * self.K * self.Np)
        p = np.empty(self.K * self.Np)
        self._check(self.lib.dg_ins_get_state(self.h, L.dptr(U), L.dptr(p)))
        return U.reshape(2, self.K, self.Np), p.reshape(self.K, self.Np)

    def _bdata(self, bd):
        arrs = [np.ascontiguousarray(bd.get(k, np.zeros(s)), np.float64).reshape(-1) for k, s in
                (("u_value", (self.nb, 2, self.Nfp)), ("u_gradient", (self.nb, 2, self.Nfp)),
                 ("p_value", (self.nb, self.Nfp)), ("p_neumann_extra", (self.nb, self.Nfp)))]
        b = L.InsBdata(L.dptr(arrs[0]), L.dptr(arrs[1]), L.dptr(arrs[2]), L.dptr(arrs[3]),
                       float(bd.get("p_data_scale", 1.0)), float(bd.get("u_data_scale", 1.0)))
        return b, arrs

    def step(self, bd, rtol=1e-13, maxit=20000):
        """One time step with this step's boundary data `bd` (dict of per-slot
        arrays and scales, include/dgcu.h: dg_ins_bdata).  Returns the solve
        statistics."""
        b, keep = self._bdata(bd)
        st = L.InsStats()
        self._check(self.lib.dg_ins_step(self.h, ctypes.byref(b), float(rtol), int(maxit), ctypes.byref(st)))
        return dict(iterations_p=st.iterations_p, iterations_u=(st.iterations_u[0], st.iterations_u[1]),
                    rel_residual_p=st.rel_residual_p, rel_residual_u=st.rel_residual_u, ms=st.ms)

    def operator(self, op, field, bd=None):
        """One operator of the step (0 convection, 1 div, 2 grad, 3 curl curl)."""
        b, keep = self._bdata(bd or {})
        nout = 1 if op == 1 else 2
        x = np.ascontiguousarray(field, np.float64).reshape(-1)
        out = np.empty(nout * self.K * self.Np)
        self._check(self.lib.dg_ins_operator(self.h, int(op), ctypes.byref(b), L.dptr(x), L.dptr(out)))
        return out.reshape((self.K, self.Np) if nout == 1 else (2, self.K, self.Np))


class PearsonVortex:
    """The tutorial's exact solution and per-step boundary data
    (setNonUniformInlet.H, setBoundaryValues.H, setparaT.H, pCorrectEquation.H)."""

    def __init__(self, solver):
        self.s = solver
        self.nu, self.dt = solver.nu, solver.dt

    def exact(self, x, y, t):
        e1 = np.exp(-4 * PI * PI * self.nu * t)
        e2 = np.exp(-8 * PI * PI * self.nu * t)
        return (-np.sin(2 * PI * y) * e1, np.sin(2 * PI * x) * e1, -np.cos(2 * PI * x) * np.cos(2 * PI * y) * e2)

    def initial_state(self, t=0.0):
        u, v, p = self.exact(self.s.x, self.s.y, t)
        return np.stack([u, v]), p

    def bdata(self, t):
        """Boundary data at the start of a step at time t (the reference sets
        them at the end of the previous step for its time)."""
        s, nu = self.s, self.nu
        x, y = s.bx, s.by
        nx, ny = s.bnx[:, None], s.bny[:, None]
        u, v, p = self.exact(x, y, t)
        e1 = np.exp(-4 * PI * PI * nu * t)
        grad = np.stack([2 * PI * ny * (-np.cos(2 * PI * y)) * e1, 2 * PI * nx * np.cos(2 * PI * x) * e1], 1)
        extra = (-nx * np.sin(2 * PI * y) + ny * np.sin(2 * PI * x)) * (-nu * 4 * PI * PI * e1)
        return dict(u_value=np.stack([u, v], 1), u_gradient=grad, p_value=p, p_neumann_extra=extra,
                    p_data_scale=np.exp(-8 * PI * PI * nu * self.dt), u_data_scale=np.exp(-4 * PI * PI * nu * self.dt))

    def pressure_error(self, p, t):
        """average and max |p - p_exact| over the nodes (chorinerror.H)."""
        d = np.abs(p - self.exact(self.s.x, self.s.y, t)[2])
        return float(d.mean()), float(d.max())


class CylinderFlow:
    """The cylinder tutorial (tutorials/DG/2D/cylinder: channel flow past a
    cylinder of radius 0.05 whose two halves are arc patches; nu = 0.001,
    dt = 2e-4, order 3): boundary kinds of its 0/U and 0/p, the inflow profile
    and the per-step boundary data of its solver (setNonUniformInlet.H,
    setBoundaryValues.H, setparaT.H, the inlet term of pCorrectEquation.H).

    U fixedValue on inlet, channel and the cylinder (zero there), zeroGradient
    on the outlet; p zeroGradient except on the outlet (fixedValue 0).  Inflow
    u = 6 (y + 0.2)(0.21 - y) / 0.41^2 * sin(pi t / 8)."""

    U_FIXED = ("inlet", "channel", "upcylinder", "downcylinder")
    NU, DT, ORDER = 0.001, 2e-4, 3

    @classmethod
    def kinds(cls, mesh):
        """(u_kind, p_kind) per boundary slot for ChorinSolver."""
        kk, ff = boundary_faces(mesh)
        names = [mesh.patch_names[i] for i in mesh.patch[kk, ff]]
        fixed = np.array([n in cls.U_FIXED for n in names])
        if not all(n in cls.U_FIXED or n == "outlet" for n in names):
            raise ValueError("cylinder case: unexpected patch among %s" % sorted(set(names)))
        return np.where(fixed, 0, 1).astype(np.int32), np.where(fixed, 2, 0).astype(np.int32)

    def __init__(self, solver):
        self.s = solver
        kk, ff = solver.bk, solver.bf
        names = list(solver.mesh.patch_names)
        self.inlet = solver.mesh.patch[kk, ff] == names.index("inlet")

    @staticmethod
    def profile(y):
        return (1.0 / 0.41) ** 2 * 6.0 * (y + 0.2) * (0.21 - y)

    def initial_state(self):
        z = np.zeros((self.s.K, self.s.Np))
        return np.stack([z, z]), z.copy()

    def bdata(self, t, first=None):
        """Boundary data of the step that starts at time t.  The solver holds
        the inflow of t (of t = 0 without the time factor before the first
        step, setNonUniformInlet.H) and scales it by sin(pi (t+dt)/8) / its
        factor at t (paraT4); the inlet's pressure Neumann term is
        -n_x du/dt = -profile * pi/8 cos(pi t/8) (paraT1)."""
        s = self.s
        first = (t == 0.0) if first is None else first
        fac = 1.0 if first else np.sin(PI * t / 8.0)
        prof = self.profile(s.by)
        inl = self.inlet[:, None]
        u = np.where(inl, prof * fac, 0.0)
        ub = np.stack([u, np.zeros_like(u)], 1)
        para_t1 = PI / 8.0 * np.cos(PI * t / 8.0)
        extra = np.where(inl, -prof * para_t1, 0.0)
        return dict(u_value=ub, p_neumann_extra=extra, p_data_scale=para_t1,
                    u_data_scale=np.sin(PI * (t + s.dt) / 8.0) / fac)


def pearson_mesh(n, name=""):
    """[-0.5, 0.5]^2 as n x n squares cut into triangles, boundary faces split
    into "inlet" (the exact flow enters: u.n < 0 at the face midpoint at t = 0)
    and "outlet" (it leaves), the pattern of the tutorial's meshes."""
    from .mesh import box_square

    m = box_square(n, n, 1.0, 1.0, x0=-0.5, y0=-0.5, name=name or "pearson_%dx%dx2" % (n, n))
    mid = 0.5 * (m.VXY + np.roll(m.VXY, -1, axis=1))
    d = np.roll(m.VXY, -1, axis=1) - m.VXY
    nx, ny = d[..., 1], -d[..., 0]
    un = -np.sin(2 * PI * mid[..., 1]) * nx + np.sin(2 * PI * mid[..., 0]) * ny
    patch = np.where(m.EToE < 0, np.where(un < 0, 0, 1), -1).astype(np.int32)
    m.patch = patch
    m.patch_names = ("inlet", "outlet")
    return m
