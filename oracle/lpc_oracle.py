"""CPU restatement of the learned element-block preconditioner (numpy).

TEST INFRASTRUCTURE ONLY: the checker for the library's BF16 training and
inference kernels (hopefoam_gb300/csrc/lpc.cu, schwarz_tc.cu,
schwarz_mlp.cu).  Nothing in the product path imports this module.

The learned preconditioner has no counterpart in the reference (its pressure
solve hands the assembled matrix to PETSc KSP with a jacobi / LU
preconditioner, DG/dgMatrices/dgMatrix/dgMatrix.C:199-222), so the parity
anchor is this restatement of the network the kernels implement, written
from its definition:

    x_k = [z_k, Rot(z_n0), Rot(z_n1), Rot(z_n2)] / s_k ++ sqrt(J_k) (rx, sx, ry, sy)
    M(r)_k = z_k + s_k W2 relu(W1 x_k),         z = P r (block Jacobi)

with element vectors in the library's ring node order (the 3N boundary nodes
face by face, then the interior nodes), Rot the node permutation that turns
the neighbour's shared face into its face 0, s_k the RMS of the element's
four z blocks.  Kernel arithmetic rules restated here: BF16 operands (inputs,
weights, hidden activations and the hidden-layer gradient rounded to BF16,
round to nearest even), sums accumulated in FP32 or wider, block Jacobi with
FP32 blocks and FP32 accumulation.

Loss of a batch of B samples: L = sum_b 0.5 ||W2 h_b - t_b||^2 / B; the
library reports L / Np.
"""
import numpy as np


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def face_nodes(order):
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


def ring_order(order):
    """Reference node id at each ring position."""
    N = order
    Np = (N + 1) * (N + 2) // 2
    fn = face_nodes(order)
    ring = [int(fn[f, j]) for f in range(3) for j in range(N)]
    onb = set(ring)
    ring += [i for i in range(Np) if i not in onb]
    return np.array(ring, np.int64)


def rotation_perms(r, s, ring):
    """perm[fn, i]: ring position of the node that the rotation taking face fn
    to face 0 maps onto ring position i (barycentric coordinates cycled)."""
    rr, ss = r[ring], s[ring]
    lam = np.stack([-(rr + ss) / 2, (1 + rr) / 2, (1 + ss) / 2], axis=1)
    Np = ring.size
    perm = np.full((3, Np), -1, np.int64)
    for fn in range(3):
        for i in range(Np):
            want = np.empty(3)
            for m in range(3):
                want[(fn + m) % 3] = lam[i, m]
            d = np.abs(lam - want).sum(axis=1)
            j = int(np.argmin(d))
            assert d[j] < 1e-9
            perm[fn, i] = j
    return perm


def block_jacobi32(S_blocks, r):
    """z = P r per element with P = inv(S_kk) rounded to FP32 and FP32
    accumulation (reference node order)."""
    P = np.linalg.inv(S_blocks).astype(np.float32)
    rk = r.reshape(S_blocks.shape[0], -1).astype(np.float32)
    return np.einsum("kij,kj->ki", P, rk).astype(np.float64)


def features(zb_ring, EToE, EToF, geo, perm, linear=False):
    """X (K x F, float32, before BF16 rounding) and s (K) from the block
    Jacobi output in ring order; geo = K x 4 (rx, sx, ry, sy); boundary faces
    (EToE[k, f] < 0) give zero blocks."""
    K, Np = zb_ring.shape
    blocks = [zb_ring]
    for f in range(3):
        nb = EToE[:, f]
        bnd = nb < 0
        nbc = np.where(bnd, 0, nb)
        fn = np.where(bnd, 0, EToF[:, f])
        zn = zb_ring[nbc][np.arange(K)[:, None], perm[fn]]
        zn[bnd] = 0.0
        blocks.append(zn)
    Z = np.concatenate(blocks, axis=1)
    s = (np.sqrt((Z * Z).sum(axis=1) / (4.0 * Np))).astype(np.float32) + np.float32(1e-30)
    X = (Z.astype(np.float32) * (np.float32(1.0) / s)[:, None]).astype(np.float32)
    J = 1.0 / (geo[:, 0] * geo[:, 3] - geo[:, 1] * geo[:, 2])
    h = np.sqrt(J)
    g = np.zeros_like(geo) if linear else geo * h[:, None]
    X = np.concatenate([X, g.astype(np.float32)], axis=1)
    return X, s


def _act(A, linear):
    return A if linear else np.maximum(A, 0.0)


def forward(W1, W2, X, T, linear=False):
    """Hidden activations (BF16-rounded), output residuals dY and the loss
    (library convention: mean over samples and outputs of 0.5 dY^2)."""
    W1b, W2b, Xb = bf16(W1).astype(np.float64), bf16(W2).astype(np.float64), bf16(X).astype(np.float64)
    A = (Xb @ W1b.T).astype(np.float32)
    Hs = bf16(_act(A, linear)).astype(np.float64)
    Y = (Hs @ W2b.T).astype(np.float32)
    dY = (Y - np.asarray(T, np.float32)).astype(np.float64)
    loss = 0.5 * float((dY * dY).sum()) / (X.shape[0] * W2.shape[0])
    return Hs, dY, loss


def gradients(W1, W2, X, T, linear=False):
    """dL/dW1, dL/dW2 (L = sum_b 0.5 ||dY_b||^2 / B) under the kernel rounding
    rules, and the library's loss value."""
    B = X.shape[0]
    Hs, dY, loss = forward(W1, W2, X, T, linear)
    W2b = bf16(W2).astype(np.float64)
    mask = 1.0 if linear else (Hs > 0)
    dH = bf16(((dY @ W2b) * mask).astype(np.float32)).astype(np.float64)
    Xb = bf16(X).astype(np.float64)
    gW2 = dY.T @ Hs / B
    gW1 = dH.T @ Xb / B
    return gW1, gW2, loss


def gradients_exact(W1, W2, X, T):
    """FP64 gradients of the same loss without any rounding (for the finite
    difference check of the restatement itself)."""
    B = X.shape[0]
    A = X @ W1.T
    Hs = np.maximum(A, 0.0)
    dY = Hs @ W2.T - T
    dH = (dY @ W2) * (A > 0)
    return dH.T @ X / B, dY.T @ Hs / B, 0.5 * float((dY * dY).sum()) / B


def precond(W1, W2, zb_ring, EToE, EToF, geo, perm, linear=False):
    """Learned preconditioner output in ring order."""
    X, s = features(zb_ring, EToE, EToF, geo, perm, linear)
    W1b, W2b = bf16(W1).astype(np.float64), bf16(W2).astype(np.float64)
    Hs = bf16(_act((bf16(X).astype(np.float64) @ W1b.T).astype(np.float32), linear)).astype(np.float64)
    Y = (Hs @ W2b.T).astype(np.float32).astype(np.float64)
    return zb_ring + s.astype(np.float64)[:, None] * Y


def energy_gradients(W1, W2, r_ring, zb_ring, EToE, EToF, geo, perm, S_apply_ring, linear=False):
    """Gradients of the training loss for one residual (ring order): the
    output gradient dY = s ((a/b) S z - r) (a = r.z, b = z.S z; the loss
    -(r.z)|r.z| / (z.S z) has gradient 2|a|/b times this) chained through the
    network, averaged over the K elements like the batch gradients.
    Returns gW1, gW2 and the reported loss -(a^2)/b."""
    X, s = features(zb_ring, EToE, EToF, geo, perm, linear)
    W1b, W2b = bf16(W1).astype(np.float64), bf16(W2).astype(np.float64)
    Xb = bf16(X).astype(np.float64)
    Hs = bf16(_act((Xb @ W1b.T).astype(np.float32), linear)).astype(np.float64)
    Y = (Hs @ W2b.T).astype(np.float32).astype(np.float64)
    s64 = s.astype(np.float64)[:, None]
    z = zb_ring + s64 * Y
    w = S_apply_ring(z)
    a = float((r_ring * z).sum())
    b = float((z * w).sum())
    dY = (s64 * ((a / b) * w - r_ring)).astype(np.float32).astype(np.float64)
    dH = bf16(((dY @ W2b) * (1.0 if linear else (Hs > 0))).astype(np.float32)).astype(np.float64)
    K = X.shape[0]
    return dH.T @ Xb / K, dY.T @ Hs / K, -(a * a) / b


# ---------------------------------------------------------------------------
# Learned additive-Schwarz form: M r = P r + sum_m G_m^T W^T W G_m r, with
# G_m the gather of element m and its three rotated neighbours (raw residual,
# no scaling), W in BF16 and FP32 activations.


def schwarz_gather(v_ring, EToE, EToF, perm):
    """K x 4 Np rows G_m v (ring order)."""
    K, Np = v_ring.shape
    blocks = [v_ring]
    for f in range(3):
        nb = EToE[:, f]
        bnd = nb < 0
        nbc = np.where(bnd, 0, nb)
        fn = np.where(bnd, 0, EToF[:, f])
        vn = v_ring[nbc][np.arange(K)[:, None], perm[fn]]
        vn[bnd] = 0.0
        blocks.append(vn)
    return np.concatenate(blocks, axis=1)


def schwarz_scatter(U, EToE, EToF, perm):
    """sum_m G_m^T U_m (K x Np): the element's own slot plus, through each face
    f with neighbour m (m's face fn), m's slot fn + 1 at the node permutation
    of face f."""
    K = U.shape[0]
    Np = U.shape[1] // 4
    z = U[:, :Np].astype(np.float64).copy()
    for f in range(3):
        nb = EToE[:, f]
        ok = nb >= 0
        fn = EToF[:, f]
        k = np.nonzero(ok)[0]
        src = U[nb[k][:, None], (fn[k][:, None] + 1) * Np + np.arange(Np)[None, :]]
        np.add.at(z, (k[:, None], perm[f][None, :].repeat(k.size, 0)), src)
    return z


def schwarz_apply(W, r_ring, zb_ring, EToE, EToF, perm):
    Wb = bf16(W).astype(np.float64)
    X = schwarz_gather(r_ring, EToE, EToF, perm).astype(np.float32).astype(np.float64)
    U = ((X @ Wb.T) @ Wb)
    return zb_ring + schwarz_scatter(U, EToE, EToF, perm)


def schwarz_energy_gradients(W, r_ring, zb_ring, EToE, EToF, perm, S_apply_ring):
    """dL/dW = (2a/b) W (X^T A + A^T X), X = G r, A = G g, g = (a/b) S z - r,
    and the loss -(a^2)/b, for L(r) = -(r.z)|r.z| / (z.S z)."""
    z = schwarz_apply(W, r_ring, zb_ring, EToE, EToF, perm)
    w = S_apply_ring(z)
    a = float((r_ring * z).sum())
    b = float((z * w).sum())
    g = (a / b) * w - r_ring
    X = schwarz_gather(r_ring, EToE, EToF, perm)
    A = schwarz_gather(g, EToE, EToF, perm)
    C = X.T @ A + A.T @ X
    return (2 * a / b) * (W.astype(np.float64) @ C), -(a * a) / b


# ---------------------------------------------------------------------------
# Two-layer learned additive-Schwarz form (tied weights, leaky relu between):
#     M(r) = P r + sum_m G_m^T W^T act(W G_m r),   W: 128 x 4 Np in BF16,
#     act(h) = max(h, slope h), slope in [0, 1] (0: relu).
# Every term is >= 0 against r, M is positively homogeneous but not linear.
# The kernels compute the local stage with BF16 hi + lo operands (FP32
# accuracy) and the training gradient with X = G r, A = G g, h = relu(X W^T)
# and D (W a) rounded to BF16 once, FP32 accumulation.


def _leaky(P, slope):
    return np.maximum(P, slope * P)


def schwarz_mlp_apply(W, r_ring, zb_ring, EToE, EToF, perm, exact=False, slope=0.0):
    """M(r) in ring order; W rounded to BF16 unless exact."""
    Wb = np.asarray(W, np.float64) if exact else bf16(W).astype(np.float64)
    X = schwarz_gather(r_ring, EToE, EToF, perm)
    U = _leaky(X @ Wb.T, slope) @ Wb
    return zb_ring + schwarz_scatter(U, EToE, EToF, perm)


def schwarz_mlp_loss(W, r_ring, zb_ring, EToE, EToF, perm, S_apply_ring, exact=True, slope=0.0):
    """The energy loss -(r.z)|r.z| / (z.S z) of z = M(r)."""
    z = schwarz_mlp_apply(W, r_ring, zb_ring, EToE, EToF, perm, exact=exact, slope=slope)
    a = float((r_ring * z).sum())
    b = float((z * S_apply_ring(z)).sum())
    return -a * abs(a) / b


def schwarz_mlp_energy_gradients(W, r_ring, zb_ring, EToE, EToF, perm, S_apply_ring, exact=False, slope=0.0):
    """dL/dW = (2a/b) sum_m [h_m a_m^T + (D_m W a_m) x_m^T] with x_m = G_m r,
    a_m = G_m g, g = (a/b) S z - r, h_m = act(W x_m), D_m = diag act'(W x_m)
    (1 where W x_m > 0, else slope), and the loss -(a^2)/b.  exact=False
    applies the kernels' rounding rules (W, X, A, h and D W a in BF16);
    exact=True is the FP64 derivative."""
    z = schwarz_mlp_apply(W, r_ring, zb_ring, EToE, EToF, perm, exact=exact, slope=slope)
    w = S_apply_ring(z)
    a = float((r_ring * z).sum())
    b = float((z * w).sum())
    g = (a / b) * w - r_ring
    X = schwarz_gather(r_ring, EToE, EToF, perm)
    A = schwarz_gather(g, EToE, EToF, perm)
    if exact:
        Wb = np.asarray(W, np.float64)
    else:
        Wb = bf16(W).astype(np.float64)
        X = bf16(X.astype(np.float32)).astype(np.float64)
        A = bf16(A.astype(np.float32)).astype(np.float64)
    P = X @ Wb.T
    h = _leaky(P, slope)
    Bm = (A @ Wb.T) * np.where(P > 0, 1.0, slope)
    if not exact:
        h = bf16(h.astype(np.float32)).astype(np.float64)
        Bm = bf16(Bm.astype(np.float32)).astype(np.float64)
    return (2 * a / b) * (h.T @ A + Bm.T @ X), -(a * a) / b


# ---------------------------------------------------------------------------
# The same additive-Schwarz form without learning: W^T W = theta * C with C the
# mean over interior patches of the inverse of the patch operator G_m S G_m^T
# (the element and its three rotated neighbours, the gather order of
# schwarz_gather), the classical overlapping-Schwarz local solve shared by all
# patches.


def schwarz_patch_inverse_mean(S_diag, S_off, EToE, EToF, ring, perm):
    """C (4 Np x 4 Np) from the SPD operator's element blocks in reference node
    order: S_diag (K, Np, Np), S_off (K, 3, Np, Np) coupling element k's rows
    with neighbour EToE[k, f]'s columns.  Only patches with three neighbours
    enter the mean."""
    K, Np = S_diag.shape[0], ring.size
    D = S_diag[:, ring][:, :, ring]
    O = S_off[:, :, ring][:, :, :, ring]
    F = 4 * Np
    ar = np.arange(K)
    interior = (EToE >= 0).all(1) & (EToE != ar[:, None]).all(1)
    Sp = np.zeros((K, F, F))
    Sp[:, :Np, :Np] = D
    for f in range(3):
        nb = EToE[:, f]
        ok = (nb >= 0) & (nb != ar)
        fn = np.where(ok, EToF[:, f], 0)
        nbc = np.where(ok, nb, 0)
        pm = perm[fn]
        blk = O[:, f][ar[:, None], :, pm].transpose(0, 2, 1)
        blk[~ok] = 0
        Sp[:, :Np, (f + 1) * Np:(f + 2) * Np] = blk
        Sp[:, (f + 1) * Np:(f + 2) * Np, :Np] = blk.transpose(0, 2, 1)
        Dn = D[nbc][ar[:, None, None], pm[:, :, None], pm[:, None, :]]
        Dn[~ok] = np.eye(Np)
        Sp[:, (f + 1) * Np:(f + 2) * Np, (f + 1) * Np:(f + 2) * Np] = Dn
    return np.linalg.inv(Sp[interior]).mean(0)


def schwarz_weights_from(C, theta, rows):
    """W (rows x F) with W^T W = theta C (C symmetric positive semi-definite)."""
    lam, V = np.linalg.eigh(C)
    F = C.shape[0]
    W = np.zeros((rows, F), np.float32)
    k = min(rows, F)
    order = np.argsort(lam)[::-1][:k]
    W[:k] = (np.sqrt(theta * np.maximum(lam[order], 0.0))[:, None] * V[:, order].T).astype(np.float32)
    return W
