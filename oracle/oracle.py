"""ctypes wrapper of the CPU oracle (test infrastructure: only tests/,
__graft_entry__.smoke() and bench.py's CPU baseline use it)."""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libdgoracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build():
    subprocess.check_call(["make", "-s", "-C", _HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        L = ctypes.CDLL(_LIB)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int, ctypes.c_int, _ip, _dp, _dp, ctypes.c_int]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_sizes.argtypes = [ctypes.c_void_p, _ip]
        L.orc_ref_operators.argtypes = [ctypes.c_void_p] + [_dp] * 11 + [_ip]
        L.orc_nodes.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_set_nodes.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_connectivity.argtypes = [ctypes.c_void_p, _ip, _ip, _ip]
        L.orc_mass.argtypes = [ctypes.c_void_p, _dp]
        L.orc_euler_rhs.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_int, ctypes.c_double, _dp]
        L.orc_euler_weak.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_int, ctypes.c_double, _dp]
        L.orc_ssprk2.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_double, _dp, ctypes.c_double]
        L.orc_lserk4.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_double]
        L.orc_lserk4_coeffs.argtypes = [_dp, _dp, _dp]
        L.orc_face_geom.argtypes = [ctypes.c_void_p, _dp]
        L.orc_ipdg_blocks.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp, _dp, _dp, _dp]
        L.orc_blk_apply.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp]
        L.orc_pcg_bj.restype = ctypes.c_int
        L.orc_pcg_bj.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, ctypes.c_double, ctypes.c_int, _dp]
        L.orc_ipdg_blocks_bc.argtypes = [ctypes.c_void_p, ctypes.c_double, _ip, _dp, _dp, _dp, _dp, _dp]
        L.orc_ins_div_nodal.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_ins_grad_nodal.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_ins_curlcurl.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_ins_convection.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc_face_mass_lift.argtypes = [ctypes.c_void_p, _ip, _dp, _dp]
        L.orc_limiter.argtypes = [ctypes.c_void_p, _dp, _dp, _ip, _ip]
        L.orc_euler_rhs_traces.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_int, ctypes.c_double, _dp]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


FLUX_LF, FLUX_ROE = 0, 1


class Oracle:
    """FP64 CPU restatement of the reference's DG discretisation on one mesh."""

    def __init__(self, mesh, order, cub):
        self.L = lib()
        self.mesh = mesh
        self.N = order
        EToV = np.ascontiguousarray(mesh.EToV, np.int32)
        VXY = np.ascontiguousarray(mesh.VXY, np.float64)
        self.cub = np.ascontiguousarray(cub, np.float64)
        self.h = self.L.orc_create(order, mesh.K, _i(EToV), _d(VXY), _d(self.cub), self.cub.shape[0])
        s = np.zeros(6, np.int32)
        self.L.orc_sizes(self.h, _i(s))
        self.Np, self.Ng, self.Nfp, self.Nfq, self.nfaces, self.nfacegauss = [int(v) for v in s]
        self.K = mesh.K

    def __del__(self):
        try:
            self.L.orc_destroy(self.h)
        except Exception:
            pass

    def operators(self):
        Np, Ng, Nfq, Nfp = self.Np, self.Ng, self.Nfq, self.Nfp
        out = dict(r=np.zeros(Np), s=np.zeros(Np), V=np.zeros((Np, Np)), Dr=np.zeros((Np, Np)),
                   Ds=np.zeros((Np, Np)), cellV=np.zeros((Ng, Np)), cellDr=np.zeros((Ng, Np)),
                   cellDs=np.zeros((Ng, Np)), fq=np.zeros(Nfq), fw=np.zeros(Nfq),
                   faceInterp=np.zeros((Nfq, Nfp)))
        fci = np.zeros((3, 2, Nfp), np.int32)
        self.L.orc_ref_operators(self.h, *[_d(out[k]) for k in ["r", "s", "V", "Dr", "Ds", "cellV", "cellDr",
                                                                  "cellDs", "fq", "fw", "faceInterp"]], _i(fci))
        out["fci"] = fci
        return out

    def nodes(self):
        x = np.zeros(self.K * self.Np)
        y = np.zeros(self.K * self.Np)
        self.L.orc_nodes(self.h, _d(x), _d(y))
        return x.reshape(self.K, self.Np), y.reshape(self.K, self.Np)

    def set_nodes(self, x, y):
        """Replace the node locations (not the metrics), as arc patches do."""
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        y = np.ascontiguousarray(y, np.float64).reshape(-1)
        assert x.size == self.K * self.Np and y.size == x.size
        self.L.orc_set_nodes(self.h, _d(x), _d(y))

    def connectivity(self):
        E = np.zeros((self.K, 3), np.int32)
        F = np.zeros((self.K, 3), np.int32)
        R = np.zeros((self.K, 3), np.int32)
        self.L.orc_connectivity(self.h, _i(E), _i(F), _i(R))
        return E, F, R

    def mass(self):
        M = np.zeros((self.K, self.Np, self.Np))
        self.L.orc_mass(self.h, _d(M))
        return M

    def face_geom(self):
        g = np.zeros((self.K, 3, 3))
        self.L.orc_face_geom(self.h, _d(g))
        return g

    @staticmethod
    def _bc(bc):
        if bc is None:
            return None
        return np.ascontiguousarray(bc, np.float64)

    def euler_rhs(self, q, flux=FLUX_LF, gamma=1.4, bc=None):
        q = np.ascontiguousarray(q, np.float64)
        out = np.zeros_like(q)
        b = self._bc(bc)
        self.L.orc_euler_rhs(self.h, _d(q), _d(out), flux, gamma, _d(b) if b is not None else None)
        return out

    def euler_weak(self, q, flux=FLUX_LF, gamma=1.4, bc=None):
        q = np.ascontiguousarray(q, np.float64)
        out = np.zeros_like(q)
        b = self._bc(bc)
        self.L.orc_euler_weak(self.h, _d(q), _d(out), flux, gamma, _d(b) if b is not None else None)
        return out

    def ssprk2(self, q, dt, nsteps, flux=FLUX_ROE, gamma=1.4, bc=None, t0=0.0):
        q = np.array(q, np.float64, copy=True)
        b = self._bc(bc)
        self.L.orc_ssprk2(self.h, _d(q), dt, nsteps, flux, gamma, _d(b) if b is not None else None, t0)
        return q

    def lserk4(self, q, dt, nsteps, flux=FLUX_LF, gamma=1.4, res=None):
        q = np.array(q, np.float64, copy=True)
        res = np.zeros_like(q) if res is None else np.array(res, np.float64, copy=True)
        self.L.orc_lserk4(self.h, _d(q), _d(res), dt, nsteps, flux, gamma)
        return q, res

    def ipdg_blocks(self, tau_coef=20.0, gD=None):
        Np = self.Np
        diag = np.zeros((self.K, Np, Np))
        off = np.zeros((self.K, 3, Np, Np))
        b = np.zeros(self.K * Np)
        g = None if gD is None else np.ascontiguousarray(gD, np.float64)
        self.L.orc_ipdg_blocks(self.h, tau_coef, _d(g) if g is not None else None, _d(diag), _d(off), _d(b))
        return diag, off, b

    def ipdg_blocks_bc(self, btype, gD=None, gN=None, tau_coef=20.0):
        """SIPG blocks with a boundary type per element face (0 Dirichlet with
        data gD, 1 Neumann with data gN, 2 natural), data per element face in
        the element's face-node order: arrays (K, 3, Nfp)."""
        Np, K, Nfp = self.Np, self.K, self.Nfp
        diag = np.zeros((K, Np, Np))
        off = np.zeros((K, 3, Np, Np))
        b = np.zeros(K * Np)
        bt = np.ascontiguousarray(btype, np.int32).reshape(K * 3)
        gd = None if gD is None else np.ascontiguousarray(gD, np.float64).reshape(K * 3 * Nfp)
        gn = None if gN is None else np.ascontiguousarray(gN, np.float64).reshape(K * 3 * Nfp)
        self.L.orc_ipdg_blocks_bc(self.h, tau_coef, _i(bt), _d(gd) if gd is not None else None,
                                  _d(gn) if gn is not None else None, _d(diag), _d(off), _d(b))
        return diag, off, b

    def _vec_op(self, fn, x, ncomp_out):
        x = np.ascontiguousarray(x, np.float64)
        out = np.zeros(ncomp_out * self.K * self.Np)
        fn(self.h, _d(x), _d(out))
        return out

    def div_nodal(self, u):
        """Strong nodal divergence of u (2, K, Np) -> (K, Np)."""
        return self._vec_op(self.L.orc_ins_div_nodal, u, 1).reshape(self.K, self.Np)

    def grad_nodal(self, p):
        return self._vec_op(self.L.orc_ins_grad_nodal, p, 2).reshape(2, self.K, self.Np)

    def curlcurl(self, u):
        return self._vec_op(self.L.orc_ins_curlcurl, u, 2).reshape(2, self.K, self.Np)

    def convection(self, u, ubnd):
        """div(U (x) U) of the LF-flux DG convection operator; ubnd (K, 3, 2, Nfp)
        boundary values (read on boundary faces)."""
        u = np.ascontiguousarray(u, np.float64)
        g = np.ascontiguousarray(ubnd, np.float64)
        out = np.zeros(2 * self.K * self.Np)
        self.L.orc_ins_convection(self.h, _d(u), _d(g), _d(out))
        return out.reshape(2, self.K, self.Np)

    def face_mass_lift(self, mask, g):
        """b[k, face nodes of f] += (I^T W I) g[k, f] where mask[k, f]."""
        m = np.ascontiguousarray(mask, np.int32).reshape(-1)
        g = np.ascontiguousarray(g, np.float64)
        b = np.zeros(self.K * self.Np)
        self.L.orc_face_mass_lift(self.h, _i(m), _d(g), _d(b))
        return b.reshape(self.K, self.Np)

    def euler_rhs_traces(self, q, traces, flux=FLUX_ROE, gamma=1.4):
        """R(q) with fixed boundary values per boundary slot [nb][4][Nfp]."""
        q = np.ascontiguousarray(q, np.float64).reshape(-1)
        t = np.ascontiguousarray(traces, np.float64)
        out = np.zeros_like(q)
        self.L.orc_euler_rhs_traces(self.h, _d(q), _d(out), flux, gamma, _d(t))
        return out

    def limiter(self, q, bnd, kind, gref=None):
        """The reference's slope limiter applied to q ([4][K][Np]); bnd per
        boundary slot [nb][4][Nfp], kind per slot (0 fixed value, 1
        reflective, 2 other, 3 zero gradient: ghost cells as 2), gref per slot
        (default: itself)."""
        q = np.array(q, np.float64, copy=True).reshape(-1)
        bnd = np.ascontiguousarray(bnd, np.float64)
        kind = np.ascontiguousarray(kind, np.int32)
        gref = np.ascontiguousarray(np.arange(len(kind)) if gref is None else gref, np.int32)
        self.L.orc_limiter(self.h, _d(q), _d(bnd), _i(kind), _i(gref))
        return q.reshape(4, self.K, self.Np)

    def blk_apply(self, diag, off, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self.L.orc_blk_apply(self.h, _d(diag), _d(off), _d(x), _d(y))
        return y

    def pcg_bj(self, diag, off, rhs, x0=None, rtol=1e-10, maxit=10000):
        rhs = np.ascontiguousarray(rhs, np.float64)
        x = np.zeros_like(rhs) if x0 is None else np.array(x0, np.float64, copy=True)
        rr = np.zeros(1)
        it = self.L.orc_pcg_bj(self.h, _d(diag), _d(off), _d(rhs), _d(x), rtol, maxit, _d(rr))
        return x, int(it), float(rr[0])


def curved_nodes(O, mesh, curved_patches, project):
    """Node locations after the relocation of the nodes next to curved patches
    (physicalElementData.C:186-224 and triangleBaseFunction.C:421-466).

    For each boundary face (k, f) on a patch named in ``curved_patches``: the
    face's interior nodes go to ``project(x, y)`` (closest curve points; the
    end nodes stay), and the shift d of the face nodes is carried into the
    element as  x_i += blend_i * sum_j d_j l_j(vr_i)  with l_j the Lagrange
    polynomials of the face's 1D nodes and
      f = 0: vr = r, blend = -(r + s) / (1 - vr)
      f = 1: vr = s, blend = (r + 1) / (1 - vr)
      f = 2: vr = s, blend = -(r + s) / (1 - vr), d reversed,
    nodes with |1 - vr| < 1e-7 untouched."""
    ops = O.operators()
    r, s, fci = ops["r"], ops["s"], ops["fci"][:, 0, :]
    x, y = O.nodes()
    x, y = x.copy(), y.copy()
    E, _, _ = O.connectivity()
    Nfp = fci.shape[1]
    t = r[fci[0]]  # the 1D nodes: face 0 runs along r

    def lagrange(z):
        Lm = np.ones((z.size, Nfp))
        for j in range(Nfp):
            for m in range(Nfp):
                if m != j:
                    Lm[:, j] *= (z - t[m]) / (t[j] - t[m])
        return Lm

    names = list(mesh.patch_names)
    for k in range(O.K):
        for f in range(3):
            if E[k, f] >= 0 or names[mesh.patch[k, f]] not in curved_patches:
                continue
            ids = fci[f]
            sx, sy = x[k, ids].copy(), y[k, ids].copy()
            px, py = project(sx[1:-1], sy[1:-1])
            d = np.zeros((Nfp, 2))
            d[1:-1, 0] = np.asarray(px) - sx[1:-1]
            d[1:-1, 1] = np.asarray(py) - sy[1:-1]
            if f == 2:
                d = d[::-1]
            vr = r if f == 0 else s
            move = lagrange(vr) @ d
            for i in range(O.Np):
                if abs(1.0 - vr[i]) < 1e-7:
                    continue
                b = (r[i] + 1) / (1 - vr[i]) if f == 1 else -(r[i] + s[i]) / (1 - vr[i])
                x[k, i] += b * move[i, 0]
                y[k, i] += b * move[i, 1]
    return x, y


def lserk4_coeffs():
    a, b, c = np.zeros(5), np.zeros(5), np.zeros(5)
    lib().orc_lserk4_coeffs(_d(a), _d(b), _d(c))
    return a, b, c


def set_threads(n):
    lib().orc_set_threads(int(n))


def max_threads():
    return int(lib().orc_max_threads())
