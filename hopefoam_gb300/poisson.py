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


def poisson_rhs(mesh, order, seed=0, kmax=16, tg_weight=1.0, t=0.0, nu=0.01):
    """Right-hand side of the pressure benchmark on [0, 2pi]^2: the pressure
    source of the Taylor-Green vortex, cos 2x + cos 2y (the divergence of
    u.grad u for u = (sin x cos y, -cos x sin y) e^{-2 nu t}, Re = 1/nu = 100),
    plus seeded Gaussian random Fourier modes with |k| <= kmax, amplitudes
    ~ N(0, 1/|k|^2); projected with the element mass matrices (b = M f)."""
    from .euler import node_coords, reference_operators

    ops = reference_operators(order)
    x, y = node_coords(mesh, ops["r"], ops["s"])
    f = tg_weight * np.exp(-4 * nu * t) * (np.cos(2 * x) + np.cos(2 * y))
    rng = np.random.default_rng(seed)
    kxs = np.arange(-kmax, kmax + 1)
    kys = np.arange(0, kmax + 1)
    C = np.zeros((kxs.size, kys.size), np.complex128)
    for i, kx in enumerate(kxs):
        for j, ky in enumerate(kys):
            k2 = kx * kx + ky * ky
            if k2 == 0 or k2 > kmax * kmax or (ky == 0 and kx < 0):
                continue
            a, b = rng.standard_normal(2) / np.sqrt(k2)
            C[i, j] = a - 1j * b  # a cos(phase) + b sin(phase) = Re((a - i b) e^{i phase})
    xf, yf = x.reshape(-1), y.reshape(-1)
    Ex = np.exp(1j * np.outer(xf, kxs))
    Ey = np.exp(1j * np.outer(yf, kys))
    f += np.sum((Ex @ C) * Ey, axis=1).real.reshape(x.shape)
    v = mesh.VXY
    J = 0.25 * ((v[:, 1, 0] - v[:, 0, 0]) * (v[:, 2, 1] - v[:, 0, 1]) - (v[:, 2, 0] - v[:, 0, 0]) * (v[:, 1, 1] - v[:, 0, 1]))
    b = J[:, None] * (f @ ops["Mref"].T)
    return b.reshape(-1), f


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

    # ------------------------------------------------------------------
    # learned element-block preconditioner (DG_PC_LEARNED)

    FORMS = {"relu": L.DG_LPC_RELU, "linear": L.DG_LPC_LINEAR, "schwarz": L.DG_LPC_SCHWARZ,
             "mlp": L.DG_LPC_SCHWARZ_MLP}
    SCHWARZ_FORMS = ("schwarz", "mlp")

    def lpc_setup(self, hidden=None, seed=0, capacity=0, form="schwarz", linear=False):
        """Allocates the learned preconditioner and room for `capacity`
        training residual vectors on the device.  form "schwarz" (default):
        M = P + sum_m G_m^T W^T W G_m, SPD by construction, W hidden x 4 Np
        (hidden 32 or 64); "mlp": M = P + sum_m G_m^T W^T relu(W G_m), the
        two-layer network with tied weights, hidden 128, BF16 tensor-core
        kernels, flexible PCG; "relu" / "linear": the two-layer correction of
        the block-Jacobi output (hidden default 128).  linear=True selects
        "linear"."""
        if linear:
            form = "linear"
        self.lpc_form = form
        self.lpc_hidden = int(hidden if hidden is not None else (32 if form == "schwarz" else 128))
        self.lpc_F = 4 * self.Np + (0 if form in self.SCHWARZ_FORMS else 4)
        self.lpc_linear = form == "linear"
        _check(self.ctx.h, self.ctx.lib.dg_lpc_setup(self.ctx.h, self.lpc_hidden, int(seed), int(capacity),
                                                     self.FORMS[form]))

    def lpc_set_slope(self, slope):
        """Activation max(h, slope h) of the "mlp" form (0: relu, 1: linear)."""
        _check(self.ctx.h, self.ctx.lib.dg_lpc_set_slope(self.ctx.h, float(slope)))

    def lpc_set_coarse(self, on=True):
        """Train the learned local stage for DG_PC_LEARNED_MULTILEVEL (its loss
        takes the coarse-space correction into account)."""
        _check(self.ctx.h, self.ctx.lib.dg_lpc_set_coarse(self.ctx.h, 1 if on else 0))

    def lpc_add_residual(self, r):
        r = np.ascontiguousarray(r, np.float64).reshape(-1)
        _check(self.ctx.h, self.ctx.lib.dg_lpc_add_residual(self.ctx.h, L.dptr(r)))

    def lpc_collect(self, rhs_list, snapshots=(1, 2, 3, 5, 8, 13, 21, 34, 55, 89, 144, 233), rtol=1e-10,
                    precision=L.DG_PREC_SPLIT, pc=L.DG_PC_BLOCK_JACOBI):
        """Training residuals from this solver's own PCG (block Jacobi by
        default; DG_PC_LEARNED_ONLY: the learned iteration's own iterates): for
        each right-hand side b, the residuals b - S x_j of the iterates after
        j iterations (j in `snapshots`).  Returns the number added."""
        n = 0
        for b in rhs_list:
            for j in snapshots:
                xj, st = self.solve(b, rtol=rtol, maxit=int(j), pc=pc, precision=precision, raise_on_fail=False)
                if st["status"] not in (L.DG_OK, L.DG_ERR_NOT_CONVERGED):
                    _check(self.ctx.h, st["status"])
                self.lpc_add_residual(b - self.apply(xj))
                n += 1
        return n

    def lpc_train(self, epochs=20, lr=1e-3, seed=0):
        """Adam epochs over the stored residuals on the GPU; returns the mean
        energy loss with the network and with block Jacobi alone."""
        loss, loss_bj = ctypes.c_double(0.0), ctypes.c_double(0.0)
        _check(self.ctx.h, self.ctx.lib.dg_lpc_train(self.ctx.h, int(epochs), float(lr), int(seed),
                                                     ctypes.byref(loss), ctypes.byref(loss_bj)))
        return loss.value, loss_bj.value

    def lpc_loss(self, r):
        r = np.ascontiguousarray(r, np.float64).reshape(-1)
        loss, loss_bj = ctypes.c_double(0.0), ctypes.c_double(0.0)
        _check(self.ctx.h, self.ctx.lib.dg_lpc_loss(self.ctx.h, L.dptr(r), ctypes.byref(loss), ctypes.byref(loss_bj)))
        return loss.value, loss_bj.value

    def lpc_energy_gradients(self, r):
        r = np.ascontiguousarray(r, np.float64).reshape(-1)
        gW1 = np.zeros((self.lpc_hidden, self.lpc_F), np.float32)
        gW2 = None if self.lpc_form in self.SCHWARZ_FORMS else np.zeros((self.Np, self.lpc_hidden), np.float32)
        loss = ctypes.c_double(0.0)
        fp = ctypes.POINTER(ctypes.c_float)
        _check(self.ctx.h, self.ctx.lib.dg_lpc_energy_gradients(
            self.ctx.h, L.dptr(r), gW1.ctypes.data_as(fp), None if gW2 is None else gW2.ctypes.data_as(fp),
            ctypes.byref(loss)))
        return gW1, gW2, loss.value

    def lpc_weights(self):
        """(W1, W2); W2 is None for the Schwarz forms (one tied weight matrix)."""
        fp = ctypes.POINTER(ctypes.c_float)
        W1 = np.zeros((self.lpc_hidden, self.lpc_F), np.float32)
        if self.lpc_form in self.SCHWARZ_FORMS:
            _check(self.ctx.h, self.ctx.lib.dg_lpc_get_weights(self.ctx.h, W1.ctypes.data_as(fp), None))
            return W1, None
        W2 = np.zeros((self.Np, self.lpc_hidden), np.float32)
        _check(self.ctx.h, self.ctx.lib.dg_lpc_get_weights(self.ctx.h, W1.ctypes.data_as(fp), W2.ctypes.data_as(fp)))
        return W1, W2

    def lpc_set_weights(self, W1, W2=None):
        fp = ctypes.POINTER(ctypes.c_float)
        W1 = np.ascontiguousarray(W1, np.float32)
        if W1.shape != (self.lpc_hidden, self.lpc_F):
            raise ValueError("weight shapes do not match the network")
        if self.lpc_form in self.SCHWARZ_FORMS:
            _check(self.ctx.h, self.ctx.lib.dg_lpc_set_weights(self.ctx.h, W1.ctypes.data_as(fp), None))
            return
        W2 = np.ascontiguousarray(W2, np.float32)
        if W2.shape != (self.Np, self.lpc_hidden):
            raise ValueError("weight shapes do not match the network")
        _check(self.ctx.h, self.ctx.lib.dg_lpc_set_weights(self.ctx.h, W1.ctypes.data_as(fp), W2.ctypes.data_as(fp)))

    def lpc_gradients(self, X, T):
        """One forward/backward of the training kernels on a host batch:
        (dL/dW1, dL/dW2, loss)."""
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        B = X.shape[0]
        gW1 = np.zeros((self.lpc_hidden, self.lpc_F), np.float32)
        gW2 = np.zeros((self.Np, self.lpc_hidden), np.float32)
        loss = ctypes.c_double(0.0)
        fp = ctypes.POINTER(ctypes.c_float)
        _check(self.ctx.h, self.ctx.lib.dg_lpc_gradients(self.ctx.h, X.ctypes.data_as(fp), T.ctypes.data_as(fp), B,
                                                         gW1.ctypes.data_as(fp), gW2.ctypes.data_as(fp),
                                                         ctypes.byref(loss)))
        return gW1, gW2, loss.value

    def lpc_apply(self, r):
        """The learned preconditioner applied once: z = M(r)."""
        r = np.ascontiguousarray(r, np.float64).reshape(-1)
        z = np.empty_like(r)
        _check(self.ctx.h, self.ctx.lib.dg_lpc_apply(self.ctx.h, L.dptr(r), L.dptr(z)))
        return z


def train_learned_preconditioner(order, tau_coef=1.0, n_interior=2000, n_rhs=16, epochs=(10, 10), lr=(1e-3, 3e-4),
                                 snapshots=(1, 2, 3, 5, 8, 13, 21, 34, 55, 89, 144, 233, 377, 610, 987), form="schwarz",
                                 hidden=None, seed=11, slope=None, coarse=False):
    """Trains the learned preconditioner on a small seeded Delaunay mesh from
    residuals of this solver's own block-Jacobi PCG (the network is local,
    so the weights transfer to larger meshes).  Returns (W1, W2, info); W2 is
    None for the Schwarz forms."""
    import time

    from .mesh import delaunay_square

    t0 = time.perf_counter()
    mesh = delaunay_square(n_interior, seed=seed)
    ps = PressureSolver(mesh, order, tau_coef=tau_coef)
    ps.lpc_setup(hidden=hidden, seed=0, capacity=n_rhs * len(snapshots), form=form)
    if slope is not None:
        ps.lpc_set_slope(slope)
    if coarse:
        ps.lpc_set_coarse(True)
    rhs = [poisson_rhs(mesh, order, seed=100 + i)[0] for i in range(n_rhs)]
    n = ps.lpc_collect(rhs, snapshots=snapshots)
    losses = []
    for i, (ep, rate) in enumerate(zip(epochs, lr)):
        losses.append(ps.lpc_train(epochs=ep, lr=rate, seed=i))
    W1, W2 = ps.lpc_weights()
    info = {"train_K": ps.K, "residuals": n, "loss": losses[-1][0], "loss_block_jacobi": losses[-1][1],
            "seconds": time.perf_counter() - t0, "form": form, "hidden": ps.lpc_hidden}
    if slope is not None:
        info["slope"] = slope
    if coarse:
        info["coarse"] = True
    ps.ctx.close()
    return W1, W2, info
