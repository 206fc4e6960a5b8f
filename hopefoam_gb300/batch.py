"""Many independent isentropic-vortex cases advanced together.

Cases of the same order share one context over their disjoint (concatenated)
periodic meshes; each element carries its case's CFL time step as a
per-element factor, so every case keeps its own step.  The groups run as one
batch (include/dgcu.h: dg_batch_*): all LSERK4 stages of all groups in one
CUDA-graph launch, launch shapes chosen by the library's autotuner.

The reference runs one case per process (dgEulerFoam); this module has no
counterpart there.
"""
import ctypes

import numpy as np

from . import _lib as L
from .euler import EulerContext, isentropic_vortex, node_coords, reference_operators
from .mesh import Mesh, connect, periodic_square


def batch_cases(n=512, seed=0, orders=(2, 3, 4, 5, 6), kmin=800, kmax=20000, beta=(1.0, 6.0), mach=(0.1, 0.8)):
    """Seeded case list: vortex strength ~ U(beta), free-stream Mach ~ U(mach),
    order uniform over `orders`, element count K* log-uniform in [kmin, kmax]
    realised as an m x m x 2 periodic grid with m = round(sqrt(K*/2))."""
    rng = np.random.default_rng(seed)
    cases = []
    for i in range(n):
        b = float(rng.uniform(*beta))
        M = float(rng.uniform(*mach))
        N = int(rng.choice(orders))
        kstar = float(np.exp(rng.uniform(np.log(kmin), np.log(kmax))))
        m = max(2, int(round(np.sqrt(kstar / 2.0))))
        cases.append(dict(beta=b, mach=M, order=N, m=m, seed=seed * 100003 + i))
    return cases


def concat_meshes(meshes, name=""):
    """One mesh holding the given meshes side by side (no shared vertices)."""
    EToV, VXY, off = [], [], 0
    for m in meshes:
        EToV.append(m.EToV + off)
        VXY.append(m.VXY)
        off += int(m.EToV.max()) + 1
    EToV = np.concatenate(EToV).astype(np.int32)
    VXY = np.concatenate(VXY)
    EToE, EToF, ROT, BC = connect(EToV)
    return Mesh(EToV, VXY, EToE, EToF, ROT, BC, name=name)


def _cfl_dt(mesh, q, order, cfl, gamma):
    """The library's CFL rule (dg_cfl_dt) for one case:
    dt = cfl min_k h_k / ((N+1)^2 max(|u| + c)), h_k = 2 area / longest edge."""
    rho, ru, rv, E = q
    u, v = ru / rho, rv / rho
    p = (gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v))
    smax = float(np.max(np.sqrt(u * u + v * v) + np.sqrt(gamma * p / rho)))
    return cfl * mesh.min_h() / ((order + 1) ** 2 * smax)


class EulerBatch:
    """The cases grouped by order; `run` advances all of them."""

    def __init__(self, cases, L_box=10.0, perturb=0.1, gamma=1.4, cfl=0.5):
        self.lib = L.lib()
        self.gamma = gamma
        self.groups = []  # (order, ctx, [case indices], element offsets)
        orders = sorted({c["order"] for c in cases})
        for N in orders:
            idx = [i for i, c in enumerate(cases) if c["order"] == N]
            ops = reference_operators(N)
            meshes, states, dts = [], [], []
            for i in idx:
                c = cases[i]
                m = periodic_square(c["m"], c["m"], L_box, L_box, perturb=perturb, seed=c["seed"])
                x, y = node_coords(m, ops["r"], ops["s"])
                uinf = c["mach"] * np.sqrt(gamma)  # rho_inf = p_inf = 1: c_inf = sqrt(gamma)
                q = isentropic_vortex(x, y, 0.0, beta=c["beta"], x0=L_box / 2, y0=L_box / 2, uinf=uinf,
                                      gamma=gamma)
                meshes.append(m)
                states.append(q)
                dts.append(np.full(m.K, _cfl_dt(m, q, N, cfl, gamma)))
            big = concat_meshes(meshes, name="batch_N%d" % N)
            ctx = EulerContext(big, N, gamma=gamma)
            ctx.upload(np.concatenate(states, axis=1))
            dtk = np.ascontiguousarray(np.concatenate(dts))
            _ck(ctx.h, self.lib.dg_set_element_dt(ctx.h, L.dptr(dtk)))
            offs = np.cumsum([0] + [m.K for m in meshes])
            self.groups.append(dict(order=N, ctx=ctx, cases=idx, offsets=offs, dtk=dtk))
        arr = (ctypes.c_void_p * len(self.groups))(*[g["ctx"].h for g in self.groups])
        h = ctypes.c_void_p()
        _ck(None, self.lib.dg_batch_create(arr, len(self.groups), ctypes.byref(h)))
        self.h = h
        self.elements = sum(g["ctx"].K for g in self.groups)
        self.dofs = sum(4 * g["ctx"].K * g["ctx"].Np for g in self.groups)

    def _check(self, rc):
        if rc != L.DG_OK:
            m = self.lib.dg_batch_last_error(self.h)
            raise L.DGError(rc, m.decode() if m else "")

    def tune(self, flux=L.DG_FLUX_LF, precision=L.DG_PREC_SPLIT, steps_per_trial=2):
        t = L.BatchTuning()
        self._check(self.lib.dg_batch_tune(self.h, 1.0, flux, precision, steps_per_trial, ctypes.byref(t)))
        shapes = []
        for g in range(len(self.groups)):
            cps, smb, conc = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
            self._check(self.lib.dg_batch_get_shape(self.h, g, ctypes.byref(cps), ctypes.byref(smb),
                                                    ctypes.byref(conc)))
            shapes.append(dict(order=self.groups[g]["order"], ctas_per_sm=cps.value, sm_budget=smb.value))
        return dict(concurrent=t.concurrent, ms_sequential=t.ms_sequential, ms_concurrent=t.ms_concurrent,
                    ms_fused=t.ms_fused, groups=shapes)

    def set_schedule(self, schedule, precision=L.DG_PREC_SPLIT):
        """0: groups one after another, 1: side by side on streams, 2: one
        mixed-order launch per stage."""
        self._check(self.lib.dg_batch_set_schedule(self.h, int(schedule), int(precision)))

    def run(self, nsteps, flux=L.DG_FLUX_LF, precision=L.DG_PREC_SPLIT):
        """Advances every case nsteps LSERK4 steps (one graph launch);
        returns the device milliseconds."""
        ms = ctypes.c_double()
        self._check(self.lib.dg_batch_run(self.h, 1.0, int(nsteps), flux, precision, ctypes.byref(ms)))
        return ms.value

    def states(self):
        """Per case (4, K_case, Np) states, in the order of the case list."""
        out = {}
        for g in self.groups:
            q = g["ctx"].download()
            for j, i in enumerate(g["cases"]):
                out[i] = q[:, g["offsets"][j]:g["offsets"][j + 1]]
        return [out[i] for i in sorted(out)]

    def close(self):
        if getattr(self, "h", None):
            self.lib.dg_batch_destroy(self.h)
            self.h = None
        for g in self.groups:
            g["ctx"].close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ck(h, rc):
    if rc != L.DG_OK:
        msg = ""
        if h:
            m = L.lib().dg_last_error(h)
            msg = m.decode() if m else ""
        raise L.DGError(rc, msg)
