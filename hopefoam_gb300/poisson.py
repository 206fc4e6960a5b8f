"""Pressure Poisson solve (SIPG + PCG) over the C ABI -- the host-side mirror
of the reference's ``dg::solveEquation(dgm::laplacian(p) == rhs)`` with a KSP
``cg`` solver (tutorials/DG/2D/pearsonVortex/dgChorinFoam/dgChorinFoam.C:82-85,
DG/dgMatrices/dgMatrix/dgMatrix.C:162-283).

Sign convention: the reference assembles A = laplacian (negative
semi-definite); this interface solves S x = b with S = -A (SPD), so a
reference right-hand side b_ref maps to b = -b_ref.  Vectors are K*Np in
the reference node order.
"""
import ctypes

import numpy as np

from . import _lib as L
from .euler import EulerContext, _check


class PressureSolver:
    def __init__(self, mesh, order, tau_coef=20.0, ctx=None):
        self.ctx = ctx if ctx is not None else EulerContext(mesh, order)
        self.K, self.Np = self.ctx.K, self.ctx.Np
        self.tau_coef = tau_coef
        _check(self.ctx.h, self.ctx.lib.dg_ipdg_setup(self.ctx.h, float(tau_coef)))

    def apply(self, x):
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        y = np.empty_like(x)
        _check(self.ctx.h, self.ctx.lib.dg_ipdg_apply(self.ctx.h, L.dptr(x), L.dptr(y)))
        return y

    def solve(self, b, x0=None, rtol=1e-10, maxit=20000, pc=L.DG_PC_BLOCK_JACOBI, precision=L.DG_PREC_SPLIT,
              raise_on_fail=True):
        b = np.ascontiguousarray(b, np.float64).reshape(-1)
        x = np.zeros_like(b) if x0 is None else np.array(x0, np.float64, copy=True).reshape(-1)
        st = L.SolveStats()
        rc = self.ctx.lib.dg_pcg_solve(self.ctx.h, L.dptr(b), L.dptr(x), float(rtol), int(maxit), int(pc),
                                       int(precision), ctypes.byref(st))
        if rc != L.DG_OK and raise_on_fail:
            _check(self.ctx.h, rc)
        return x, {"iterations": st.iterations, "rel_residual": st.rel_residual, "ms": st.ms, "status": rc}
