"""Curved ``arc`` boundary patches: the reference's arcDgPatch (a patch that
follows a parametric curve x(u, v) given as code in the mesh's boundary file,
src/DG/dgMesh/dgPatches/constraint/arc/arcDgPatch.C), its applyCurveBoundary
utility (mesh points of the patch moved onto the curve,
applications/utilities/DG/applyCurveBoundary/applyCurveBoundary.C:112-140) and
the relocation of the element nodes next to the curve
(physicalElementData.C:186-224 with triangleBaseFunction.C:421-466).

What curvature changes in the reference: the node locations only.  dgMesh
builds every element's metric terms (dx/dr, Jacobians, mass matrix, face
normals and face Jacobians; physicalElementData.C:60-136) from the straight
triangle first and moves the nodes afterwards (dgMesh.C:110-113), so the
operators stay those of the straight-sided element and the moved nodes reach
only the code that reads node locations: boundary values and initial fields
evaluated at nodes, the slope limiter's cell geometry, and field output.  This
module computes those locations; ``euler.node_coords`` applies them when a
mesh carries curves (``Mesh.curves``), and ``EulerContext`` hands them to the
limiter.

Relocation of one element with a face on a curved patch (per face):
  * the face's interior nodes move to the closest point of the curve, the two
    end nodes stay (arcDgPatch::positions, isEnd);
  * the shift d_j of the face nodes is interpolated along the face and blended
    into the element: node i moves by  b_i * p(v_i), where p is the degree-N
    interpolant of d on the face's 1D nodes and, with the element's reference
    coordinates (r, s),
      face 0 (s = -1):  v = r,  b = -(r + s) / (1 - v)
      face 1 (r + s = 0): v = s, b = (r + 1) / (1 - v)
      face 2 (r = -1):  v = s,  b = -(r + s) / (1 - v), d taken in reverse order
    and nodes with |1 - v| < 1e-7 left in place (triangleBaseFunction.C:
    433-460).  The blend follows the element's vertex order (it is not
    symmetric under relabelling), which is the mesh file's order made
    counter-clockwise, as dgPolyMesh reads it.

Closest points: the reference iterates a secant scheme on finite-difference
tangents until |(P(u) - S) x n| < 1e-12 (arcDgPatch.C:293-392).  Here the
foot point is found by Newton's method on g(u) = (P(u) - S) . P'(u) = 0 from
the nearest of a dense sample of the curve over u_range, with P' by the
complex-step derivative (exact to rounding for the analytic expressions of the
patch code); it is the same point up to the reference's tolerance.  Neither
iteration is confined to u_range: a point shared with the next patch (the end
of a half circle) goes to its foot point on the continued curve.
"""
import ast
import re

import numpy as np

# names the patch code may use (the C++ math of the reference's code blocks)
_FUNCS = {"sin": np.sin, "cos": np.cos, "tan": np.tan, "exp": np.exp, "log": np.log, "sqrt": np.sqrt,
          "pow": np.power, "atan": np.arctan, "asin": np.arcsin, "acos": np.arccos, "atan2": np.arctan2,
          "sinh": np.sinh, "cosh": np.cosh, "tanh": np.tanh, "fabs": np.abs, "abs": np.abs, "sqr": np.square}
_CONSTS = {"pi": np.pi}
_ALLOWED = (ast.Expression, ast.BinOp, ast.UnaryOp, ast.Call, ast.Name, ast.Load, ast.Constant, ast.Add, ast.Sub,
            ast.Mult, ast.Div, ast.USub, ast.UAdd)


def _split_top(code):
    out, depth, cur = [], 0, []
    for ch in code:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            out.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    out.append("".join(cur))
    return [s.strip() for s in out]


def _compile_expr(src):
    tree = ast.parse(src, mode="eval")
    for node in ast.walk(tree):
        if not isinstance(node, _ALLOWED):
            raise ValueError("arc patch code: %s not allowed in %r" % (type(node).__name__, src))
        if isinstance(node, ast.Call) and not (isinstance(node.func, ast.Name) and node.func.id in _FUNCS):
            raise ValueError("arc patch code: unknown function in %r" % src)
        if isinstance(node, ast.Name) and node.id not in _FUNCS and node.id not in _CONSTS and node.id not in ("u", "v"):
            raise ValueError("arc patch code: unknown name %r" % node.id)
        if isinstance(node, ast.Constant) and not isinstance(node.value, (int, float)):
            raise ValueError("arc patch code: constant %r" % node.value)
    code = compile(tree, "<arc patch>", "eval")
    return lambda u, v: eval(code, {"__builtins__": {}}, dict(_FUNCS, **_CONSTS, u=u, v=v))


class ArcCurve:
    """The curve of one arc patch: ``fn(u) -> (x, y)`` for u in ``u_range``
    (2D cases: v = 0).  ``fn`` should accept complex u (numpy math does) for
    the exact tangent; other callables fall back to central differences."""

    def __init__(self, fn, u_range, name=""):
        self.fn, self.name = fn, name
        self.u_range = (float(u_range[0]), float(u_range[1]))

    @classmethod
    def from_code(cls, code, u_range, v_range=(0.0, 0.0), name=""):
        """The boundary file's ``code #{ x, y, z #}`` block of C++ expressions
        in u and v (Foam::sin, Foam::constant::mathematical::pi, ...)."""
        src = re.sub(r"(Foam|std)::constant::mathematical::pi", "pi", code)
        src = re.sub(r"\b(Foam|std)::", "", src).replace("\n", " ")
        parts = _split_top(src)
        if len(parts) != 3:
            raise ValueError("arc patch code needs three components, got %d" % len(parts))
        fx, fy = _compile_expr(parts[0]), _compile_expr(parts[1])
        v0 = float(v_range[0])
        return cls(lambda u: (fx(u, v0) + 0 * u, fy(u, v0) + 0 * u), u_range, name)

    def point(self, u):
        x, y = self.fn(np.asarray(u))
        return np.asarray(x), np.asarray(y)

    def tangent(self, u):
        u = np.asarray(u, np.float64)
        span = self.u_range[1] - self.u_range[0]
        try:
            h = 1e-30 * span
            x, y = self.fn(u + 1j * h)
            return np.imag(x) / h, np.imag(y) / h
        except TypeError:
            h = 1e-6 * span
            xp, yp = self.point(u + h)
            xm, ym = self.point(u - h)
            return (xp - xm) / (2 * h), (yp - ym) / (2 * h)

    def project(self, px, py, samples=4096, iters=60):
        """Closest points of the curve to the points (px, py)."""
        px, py = np.asarray(px, np.float64).ravel(), np.asarray(py, np.float64).ravel()
        if px.size == 0:
            return px.copy(), py.copy()
        u0, u1 = self.u_range
        us = np.linspace(u0, u1, samples + 1)
        X, Y = self.point(us)
        u = np.empty(px.size)
        for a in range(0, px.size, 256):  # nearest sample, in chunks
            d2 = (X[None, :] - px[a:a + 256, None]) ** 2 + (Y[None, :] - py[a:a + 256, None]) ** 2
            u[a:a + 256] = us[np.argmin(d2, axis=1)]
        span = u1 - u0
        hd = 1e-5 * span
        for _ in range(iters):
            x, y = self.point(u)
            tx, ty = self.tangent(u)
            g = (x - px) * tx + (y - py) * ty
            # g'(u) = |P'|^2 + (P - S) . P'' (P'' by central differences of the exact tangent)
            txp, typ = self.tangent(u + hd)
            txm, tym = self.tangent(u - hd)
            gp = tx * tx + ty * ty + (x - px) * (txp - txm) / (2 * hd) + (y - py) * (typ - tym) / (2 * hd)
            du = -g / np.where(gp > 0, gp, tx * tx + ty * ty)
            u = u + du  # not clipped to u_range: the curve's expression continues past it, as in the reference
            if np.max(np.abs(du)) <= 1e-15 * span:
                break
        return self.point(u)


def read_arc_patches(boundary_text):
    """ArcCurve per ``arc`` patch of a polyMesh boundary file's text."""
    out = {}
    for m in re.finditer(r"(\w+)\s*\{((?:[^{}]|#\{.*?#\})*)\}", boundary_text, re.S):
        name, body = m.group(1), m.group(2)
        if not re.search(r"\btype\s+arc\s*;", body):
            continue
        code = re.search(r"\bcode\s*#\{(.*?)#\}", body, re.S)
        ur = re.search(r"\bu_Range\s*\(\s*([-+\d.eE]+)\s+([-+\d.eE]+)\s*\)", body)
        vr = re.search(r"\bv_Range\s*\(\s*([-+\d.eE]+)\s+([-+\d.eE]+)\s*\)", body)
        if not code or not ur:
            raise ValueError("arc patch %s: code and u_Range are required" % name)
        out[name] = ArcCurve.from_code(code.group(1), (float(ur.group(1)), float(ur.group(2))),
                                       (float(vr.group(1)), float(vr.group(2))) if vr else (0.0, 0.0), name=name)
    return out


def _curved_faces(mesh):
    """(k, f, curve) of the boundary faces on curved patches, in slot order."""
    curves = getattr(mesh, "curves", None) or {}
    if not curves:
        return []
    names = list(mesh.patch_names)
    out = []
    for k, f in zip(*np.nonzero(mesh.EToE < 0)):
        pid = int(mesh.patch[k, f])
        if pid >= 0 and names[pid] in curves:
            out.append((int(k), int(f), curves[names[pid]]))
    return out


def apply_curve_boundary(mesh):
    """The applyCurveBoundary utility: a copy of the mesh whose vertices on
    curved patches lie on their curves (each shared vertex moved once)."""
    import copy

    m = copy.copy(mesh)
    VXY = np.array(mesh.VXY, np.float64, copy=True)
    nv = int(mesh.EToV.max()) + 1
    P = np.zeros((nv, 2))
    P[mesh.EToV.ravel()] = VXY.reshape(-1, 2)
    for k, f, curve in _curved_faces(mesh):
        for v in (mesh.EToV[k, f], mesh.EToV[k, (f + 1) % 3]):
            x, y = curve.project(P[v, 0], P[v, 1])
            P[v] = (x[0], y[0])
    m.VXY = P[mesh.EToV]
    return m


def _face_interp(order):
    """(vander of the face's 1D nodes, the 1D nodes) for the face-shift interpolant."""
    from .euler import face_nodes, reference_operators

    ops = reference_operators(order)
    t = ops["r"][face_nodes(order)[0]]  # face 0 runs along r at s = -1
    return np.polynomial.legendre.legvander(t, order), ops["r"], ops["s"]


def curve_node_shift(mesh, order, x, y):
    """Node coordinates (K, Np) with the shifts of the curved faces added
    (physicalElementData.C:186-224, triangleBaseFunction.C:421-466)."""
    from .euler import face_nodes

    faces = _curved_faces(mesh)
    if not faces or order < 2:  # order 1: a face has no interior nodes to move
        return x, y
    x, y = np.array(x, copy=True), np.array(y, copy=True)
    V1, r, s = _face_interp(order)
    fn = face_nodes(order)
    N = order
    # straight face-node positions of every curved face, projected at once per curve
    by_curve = {}
    for i, (k, f, c) in enumerate(faces):
        by_curve.setdefault(id(c), (c, []))[1].append(i)
    shift = np.zeros((len(faces), N + 1, 2))
    for c, idx in by_curve.values():
        ks = np.array([faces[i][0] for i in idx])
        ids = fn[np.array([faces[i][1] for i in idx])]
        sx, sy = x[ks[:, None], ids], y[ks[:, None], ids]
        px, py = c.project(sx[:, 1:N], sy[:, 1:N])
        shift[idx, 1:N, 0] = px.reshape(len(idx), N - 1) - sx[:, 1:N]
        shift[idx, 1:N, 1] = py.reshape(len(idx), N - 1) - sy[:, 1:N]
    for i, (k, f, c) in enumerate(faces):
        d = shift[i][::-1] if f == 2 else shift[i]
        vr = r if f == 0 else s
        coef = np.linalg.solve(V1, d)  # Legendre coefficients of the face shift
        dv = np.polynomial.legendre.legvander(vr, N) @ coef  # (Np, 2)
        keep = np.abs(1.0 - vr) >= 1e-7
        b = np.zeros_like(vr)
        den = np.where(keep, 1.0 - vr, 1.0)
        b[keep] = ((r + 1) / den if f == 1 else -(r + s) / den)[keep]
        x[k] += b * dv[:, 0]
        y[k] += b * dv[:, 1]
    return x, y
