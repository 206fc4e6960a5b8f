"""CPU restatement of the reference's Chorin step (test infrastructure only).

Follows tutorials/DG/2D/pearsonVortex/dgChorinFoam (dgChorinFoam.C:63-109,
pEqnCorrect.H, pCorrectEquation.H, bCorrectEquation.H, setBoundaryValues.H,
setparaT.H, chorinerror.H) on the operators of the C++ oracle (dg_oracle.cpp:
ins_convection, ins_div_nodal, ins_grad_nodal, ins_curlcurl, face_mass_lift,
ipdg_assemble with boundary types).  Each equation is restated in the sign
convention of the reference's Equation algebra (Equation.C:39-60,
EquationEqual.H, dgLduMatrix.C:316-321: explicit terms hold minus their
mass-weighted value, ``A == B`` solves (A - B) x = b_A - b_B):

  1. N^n = div(U^n (x) U^n)                           (Sp(convecU) == div(U, U))
  2. UT = (a0 U^n + a1 U^{n-1} - dt (b0 N^n + b1 N^{n-1})) / g0
  3. L_p p = q3 b_Lp + F^T W F (b0 nbp^n + b1 nbp^{n-1}) + (g0/dt) M div(UT)
     nbp = n . (N^n + nu curl curl U^n) + (n . U_shape) d/dt(exp term) on the
     inlet (U fixesValue) faces
  4. UT <- UT - (dt/g0) grad p
  5. (g0/(dt nu) M - L_U) U^{n+1} = g0/(dt nu) M UT - q4 b_LU
with q3 = exp(-8 pi^2 nu dt), q4 = exp(-4 pi^2 nu dt) (the reference's
paraT3/paraT4 factors on the Laplacians' boundary data, which is set at the
old time), BDF1/EXT1 on the first step and BDF2/EXT2 after.  The linear
systems are solved directly (the reference's PETSc preonly + LU).

Boundary conditions of the Pearson tutorial: U fixedValue (exact) on "inlet"
and fixedGradient (exact n.grad U) on "outlet"; p zeroGradient on "inlet"
and fixedValue (exact) on "outlet" (PearsonCase).  CylinderCase restates the
cylinder tutorial's (tutorials/DG/2D/cylinder/dgChorinFoam), whose solver
differs only in its boundary data and the factors paraT1 / paraT4.  Exact solution (Pearson vortex):
u = -sin(2 pi y) e^{-4 pi^2 nu t}, v = sin(2 pi x) e^{-4 pi^2 nu t},
p = -cos(2 pi x) cos(2 pi y) e^{-8 pi^2 nu t}.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl

from .oracle import Oracle

PI = np.pi


def pearson_exact(x, y, t, nu):
    e1 = np.exp(-4 * PI * PI * nu * t)
    e2 = np.exp(-8 * PI * PI * nu * t)
    return (-np.sin(2 * PI * y) * e1, np.sin(2 * PI * x) * e1, -np.cos(2 * PI * x) * np.cos(2 * PI * y) * e2)


def assemble(diag, off, EToE):
    """CSR matrix of element blocks (diag[k], off[k][f] coupling to EToE[k][f])."""
    K, Np, _ = diag.shape
    rows, cols, vals = [], [], []
    ii, jj = np.meshgrid(np.arange(Np), np.arange(Np), indexing="ij")
    for k in range(K):
        rows.append(k * Np + ii.ravel())
        cols.append(k * Np + jj.ravel())
        vals.append(diag[k].ravel())
        for f in range(3):
            n = EToE[k, f]
            if n >= 0:
                rows.append(k * Np + ii.ravel())
                cols.append(n * Np + jj.ravel())
                vals.append(off[k, f].ravel())
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(K * Np, K * Np))


def mass_matrix(M):
    return sp.block_diag([sp.csr_matrix(m) for m in M], format="csr")


class PearsonCase:
    """tutorials/DG/2D/pearsonVortex: U fixedValue (exact) on "inlet", fixedGradient
    (exact n.grad U) on "outlet"; p zeroGradient on "inlet", fixedValue (exact)
    on "outlet"; the exact-solution Neumann term of pCorrectEquation.H:78-90."""

    def __init__(self, nu, dt):
        self.nu, self.dt = nu, dt

    def masks(self, names, patch, E):
        inlet = (patch == names.index("inlet")) & (E < 0)
        outlet = (patch == names.index("outlet")) & (E < 0)
        if not np.all((E >= 0) | inlet | outlet):
            raise ValueError("boundary faces outside inlet/outlet")
        return inlet, outlet  # U fixedValue faces, the rest of the boundary

    def initial(self, x, y, t0):
        u, v, p = pearson_exact(x, y, t0, self.nu)
        return np.stack([u, v]), p

    def u_bnd(self, xb, yb, nstep, t):
        u, v, _ = pearson_exact(xb, yb, t, self.nu)
        return np.stack([u, v], 2)  # (K, 3, 2, Nfp)

    def grad_bnd(self, xb, yb, nx, ny, t):
        e1 = np.exp(-4 * PI * PI * self.nu * t)
        gx = 2 * PI * ny * (-np.cos(2 * PI * yb)) * e1
        gy = 2 * PI * nx * np.cos(2 * PI * xb) * e1
        return np.stack([gx, gy], 2)

    def p_bnd(self, xb, yb, t):
        return pearson_exact(xb, yb, t, self.nu)[2]

    def nbp_extra(self, xb, yb, nx, ny, ufix, nstep, t):
        para_t = -self.nu * 4 * PI * PI * np.exp(-4 * PI * PI * self.nu * t)
        return (-nx * np.sin(2 * PI * yb) + ny * np.sin(2 * PI * xb)) * para_t

    def scales(self, nstep, t):
        """(q3, q4): the factors of the p and U Laplacians' boundary data."""
        return np.exp(-8 * PI * PI * self.nu * self.dt), np.exp(-4 * PI * PI * self.nu * self.dt)


class CylinderCase:
    """tutorials/DG/2D/cylinder (0/U, 0/p, setNonUniformInlet.H,
    setBoundaryValues.H, setparaT.H, pCorrectEquation.H:78-85): U fixedValue
    on inlet / channel / upcylinder / downcylinder (the inflow profile on the
    inlet, zero elsewhere), zeroGradient on outlet; p zeroGradient except the
    outlet's fixedValue 0.  The inlet values held before step n+1 are
    profile(y) * sin(pi t_n / 8), and profile(y) alone before the first step;
    paraT1 = pi/8 cos(pi t_n / 8) scales the inlet Neumann term and the p
    Laplacian's data, paraT4 = sin(pi t_{n+1}/8) / paraT3 the U Laplacian's
    (paraT3 = 1 before the first step, then sin(pi t_n / 8))."""

    def __init__(self, nu, dt):
        self.nu, self.dt = nu, dt

    @staticmethod
    def _profile(y):
        return 6.0 * (y + 0.2) * (0.21 - y) / (0.41 * 0.41)

    def masks(self, names, patch, E):
        bnd = E < 0
        fixed = np.zeros_like(bnd)
        for n in ("inlet", "channel", "upcylinder", "downcylinder"):
            fixed |= bnd & (patch == names.index(n))
        self.inlet = bnd & (patch == names.index("inlet"))
        outlet = bnd & (patch == names.index("outlet"))
        if not np.all(~bnd | fixed | outlet):
            raise ValueError("unexpected boundary patch")
        return fixed, outlet

    def initial(self, x, y, t0):
        return np.zeros((2,) + x.shape), np.zeros_like(x)

    def u_bnd(self, xb, yb, nstep, t):
        fac = 1.0 if nstep == 0 else np.sin(PI * t / 8)
        u = np.where(self.inlet[:, :, None], self._profile(yb) * fac, 0.0)
        return np.stack([u, np.zeros_like(u)], 2)

    def grad_bnd(self, xb, yb, nx, ny, t):
        return np.zeros(xb.shape[:2] + (2,) + xb.shape[2:])

    def p_bnd(self, xb, yb, t):
        return np.zeros_like(xb)

    def nbp_extra(self, xb, yb, nx, ny, ufix, nstep, t):
        return np.where(self.inlet[:, :, None], -self._profile(yb) * (PI / 8 * np.cos(PI * t / 8)), 0.0)

    def scales(self, nstep, t):
        para_t3 = 1.0 if nstep == 0 else np.sin(PI * t / 8)
        return PI / 8 * np.cos(PI * t / 8), np.sin(PI * (t + self.dt) / 8) / para_t3


class ChorinOracle:
    """The Chorin solver of dgChorinFoam on a mesh with boundary patches
    (Mesh.patch / patch_names) for one case (default: the Pearson vortex,
    patches "inlet" and "outlet")."""

    def __init__(self, mesh, order, cub, nu=0.01, dt=1e-3, tau_coef=20.0, t0=0.0, case=None):
        O = Oracle(mesh, order, cub)
        self.O, self.N, self.nu, self.dt, self.tau = O, order, nu, dt, tau_coef
        self.case = PearsonCase(nu, dt) if case is None else case
        self.K, self.Np, self.Nfp = O.K, O.Np, O.Nfp
        ops = O.operators()
        self.fci = ops["fci"][:, 0, :]  # (3, Nfp) owner face-node order
        self.x, self.y = O.nodes()
        g = O.face_geom()
        self.nx, self.ny = g[:, :, 0], g[:, :, 1]
        E, _, _ = O.connectivity()
        self.EToE = E
        # U fixedValue faces (p natural there) and the other boundary faces
        self.inlet, self.outlet = self.case.masks(list(mesh.patch_names), mesh.patch, E)
        # face-node coordinates per element face (K, 3, Nfp)
        self.xb = np.stack([self.x[:, self.fci[f]] for f in range(3)], 1)
        self.yb = np.stack([self.y[:, self.fci[f]] for f in range(3)], 1)
        # boundary types: U Dirichlet / Neumann, p natural / Dirichlet
        self.btU = np.where(self.outlet, 1, 0).astype(np.int32)
        self.btP = np.where(self.inlet, 2, 0).astype(np.int32)
        self.M = O.mass()
        self.Msp = mass_matrix(self.M)
        dP, oP, _ = O.ipdg_blocks_bc(self.btP, tau_coef=tau_coef)
        dU, oU, _ = O.ipdg_blocks_bc(self.btU, tau_coef=tau_coef)
        self.Lp = assemble(dP, oP, E)
        self.LU = assemble(dU, oU, E)
        self.lu_p = spl.splu(self.Lp.tocsc())
        self._lu_h = {}
        # state (dgChorinFoam createFields.H / setNonUniformInlet.H)
        self.U, self.p = self.case.initial(self.x, self.y, t0)
        self.Uold = self.U.copy()
        self.Nc = np.zeros_like(self.U)
        self.Nold = np.zeros_like(self.U)
        self.nbp = np.zeros((self.K, 3, self.Nfp))
        self.t = t0
        self.nstep = 0

    def _helmholtz(self, g0):
        if g0 not in self._lu_h:
            tmp = g0 / (self.dt * self.nu)
            self._lu_h[g0] = spl.splu((tmp * self.Msp - self.LU).tocsc())
        return self._lu_h[g0]

    def _mass(self, v):
        return np.einsum("kij,kj->ki", self.M, v)

    def step(self):
        nu, dt, t, c = self.nu, self.dt, self.t, self.case
        if self.nstep == 0:
            g0, a0, a1, b0, b1 = 1.0, 1.0, 0.0, 1.0, 0.0
        else:
            g0, a0, a1, b0, b1 = 1.5, 2.0, -0.5, 2.0, -1.0
        ub = c.u_bnd(self.xb, self.yb, self.nstep, t)
        # fixedGradient and interior faces: the boundary value is the interior trace
        trace = np.stack([self.U[:, :, self.fci[f]] for f in range(3)], 1).transpose(2, 1, 0, 3)  # (K,3,2,Nfp)
        ubnd = np.where(self.inlet[:, :, None, None], ub, trace)
        Nn = self.O.convection(self.U, ubnd)
        UT = (a0 * self.U + a1 * self.Uold - dt * (b0 * Nn + b1 * self.Nold)) / g0
        # pressure Neumann data on the U fixedValue faces (pEqnCorrect.H, pCorrectEquation.H:78-110)
        cu = Nn + nu * self.O.curlcurl(self.U)
        cub = np.stack([cu[:, :, self.fci[f]] for f in range(3)], 2)  # (2, K, 3, Nfp)
        nx, ny = self.nx[:, :, None], self.ny[:, :, None]
        nbp_new = nx * cub[0] + ny * cub[1] + c.nbp_extra(self.xb, self.yb, nx, ny, self.inlet, self.nstep, t)
        nbp_new = np.where(self.inlet[:, :, None], nbp_new, 0.0)
        nbp_old = b0 * nbp_new + b1 * self.nbp
        self.nbp = nbp_new
        bN = self.O.face_mass_lift(self.inlet, nbp_old)
        _, _, bLp = self.O.ipdg_blocks_bc(self.btP, gD=c.p_bnd(self.xb, self.yb, t), tau_coef=self.tau)
        q3, q4 = c.scales(self.nstep, t)
        rhs = q3 * bLp + bN.ravel() + (g0 / dt) * self._mass(self.O.div_nodal(UT)).ravel()
        p = self.lu_p.solve(rhs).reshape(self.K, self.Np)
        # velocity correction
        UT = UT - (dt / g0) * self.O.grad_nodal(p)
        # viscous step
        tmp = g0 / (dt * nu)
        lu = self._helmholtz(g0)
        gU = c.grad_bnd(self.xb, self.yb, self.nx[:, :, None], self.ny[:, :, None], t)
        Unew = np.empty_like(self.U)
        for k in range(2):
            _, _, bLU = self.O.ipdg_blocks_bc(self.btU, gD=ub[:, :, k], gN=gU[:, :, k], tau_coef=self.tau)
            rhs = tmp * self._mass(UT[k]).ravel() - q4 * bLU
            Unew[k] = lu.solve(rhs).reshape(self.K, self.Np)
        self.Uold, self.U = self.U, Unew
        self.Nold = Nn
        self.p = p
        self.t = t + dt
        self.nstep += 1

    def pressure_error(self):
        """average and max |p - p_exact| over the nodes (chorinerror.H)."""
        pe = pearson_exact(self.x, self.y, self.t, self.nu)[2]
        d = np.abs(self.p - pe)
        return float(d.mean()), float(d.max())

    def velocity_error(self):
        u, v, _ = pearson_exact(self.x, self.y, self.t, self.nu)
        return float(max(np.abs(self.U[0] - u).max(), np.abs(self.U[1] - v).max()))
