"""CPU restatement of the reference's limited SSP-RK2 Euler step (test
infrastructure only): tutorials/DG/2D/doubleMach/dgEulerFoam/dgEulerFoam.C:50-101
with the slope limiter of Trianglelimite.C (dg_oracle.cpp: limiter) and the
reflective wall of reflectiveDgPatchField.C:79-111.

Boundary fields are kept per boundary slot (boundary faces in element, face
order) as [slot][4][Nfp] at the owner's face nodes, for the state (Bq) and for
the stage state (Bs), with the reference's update points: ``rho1 = rho``
copies the field and its boundary values, setBoundaryValues overwrites the
fixed-value slots, every equation solve re-evaluates the walls from the new
interior (dgMatrixSolve.C:209), the limiter does not, and ``rho = 0.5 rho +
0.5 rho1`` combines the boundary values as well."""
import numpy as np

from .oracle import FLUX_ROE, Oracle


class LimitedSSPOracle:
    def __init__(self, mesh, order, cub, kinds, gref=None, flux=FLUX_ROE, gamma=1.4):
        self.O = Oracle(mesh, order, cub)
        self.flux, self.gamma = flux, gamma
        self.kinds = np.asarray(kinds, np.int32)
        self.gref = np.arange(len(kinds)) if gref is None else np.asarray(gref)
        self.fci = self.O.operators()["fci"][:, 0, :]
        g = self.O.face_geom()
        kk, ff = np.nonzero(mesh.EToE < 0)
        self.kk, self.ff = kk, ff
        self.nx, self.ny = g[kk, ff, 0], g[kk, ff, 1]
        self.walls = self.kinds == 1
        self.Bq = None

    def traces(self, q):
        idx = self.fci[self.ff]  # (nb, Nfp)
        return np.stack([q[v][self.kk[:, None], idx] for v in range(4)], 1)  # (nb, 4, Nfp)

    def reflect(self, q, B):
        t = self.traces(q)
        nx, ny = self.nx[:, None], self.ny[:, None]
        m = nx * t[:, 1] + ny * t[:, 2]
        r = t.copy()
        r[:, 1] = t[:, 1] - 2 * nx * m
        r[:, 2] = t[:, 2] - 2 * ny * m
        B = B.copy()
        B[self.walls] = r[self.walls]
        zg = self.kinds == 3  # zero gradient: the interior trace
        B[zg] = t[zg]
        return B

    def rhs(self, q, B):
        return self.O.euler_rhs_traces(q, B, flux=self.flux, gamma=self.gamma).reshape(q.shape)

    def limit(self, q, B):
        return self.O.limiter(q, B, self.kinds, self.gref)

    def step(self, q, dt, bdata):
        if self.Bq is None:
            self.Bq = self.reflect(q, bdata)
        Bs = self.Bq.copy()
        Bs[self.kinds == 0] = bdata[self.kinds == 0]
        q1 = q + dt * self.rhs(q, Bs)
        Bs = self.reflect(q1, Bs)
        q1 = self.limit(q1, Bs)
        q2 = q1 + dt * self.rhs(q1, Bs)
        Bs = self.reflect(q2, Bs)
        q = 0.5 * q + 0.5 * q2
        self.Bq = 0.5 * self.Bq + 0.5 * Bs
        q = self.limit(q, self.Bq)
        self.Bq = self.reflect(q, self.Bq)
        return q

    def step_unlimited(self, q, dt, B):
        """The reference's unlimited SSP-RK2 step (dgEulerFoam.C:69-117) with
        wall and zero-gradient traces taken from each stage's input state;
        B holds the traces of the other slots (kept)."""
        B = self.reflect(q, B)
        q1 = q + dt * self.rhs(q, B)
        B = self.reflect(q1, B)
        q2 = q1 + dt * self.rhs(q1, B)
        return 0.5 * q + 0.5 * q2, B

    def lserk4_unlimited(self, q, dt, B, res=None):
        """One LSERK4 step with the same boundary rule (coefficients of
        oracle.lserk4_coeffs)."""
        from .oracle import lserk4_coeffs

        a, b, _ = lserk4_coeffs()
        res = np.zeros_like(q) if res is None else res
        for s in range(5):
            B = self.reflect(q, B)
            res = a[s] * res + dt * self.rhs(q, B)
            q = q + b[s] * res
        return q, B, res
