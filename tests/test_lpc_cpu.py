"""The learned preconditioner's CPU restatement (oracle/lpc_oracle.py) pinned
on its own: BF16 rounding, the exact FP64 gradients against central finite
differences, the kernel-rule gradients against the exact ones, and the node
rotation permutations against the library's node set."""
import numpy as np
import pytest

from oracle import lpc_oracle as lo


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 2.0 ** -9, 1.0 + 3 * 2.0 ** -9, -2.5, 0.0], np.float32)
    got = lo.bf16(x)
    # BF16 keeps 7 mantissa bits: the step at 1 is 2^-7, so 1 + 2^-8 is a tie
    assert got[0] == 1.0
    assert got[1] == 1.0                      # tie -> even
    assert got[2] == 1.0                      # below half a step
    assert got[3] == np.float32(1.0 + 2.0 ** -7)  # above half a step
    assert got[4] == -2.5 and got[5] == 0.0


def _problem(seed=0, B=64, F=12, H=16, Np=5):
    rng = np.random.default_rng(seed)
    W1 = rng.standard_normal((H, F)) * 0.5
    W2 = rng.standard_normal((Np, H)) * 0.5
    X = rng.standard_normal((B, F))
    T = rng.standard_normal((B, Np))
    return W1, W2, X, T


def test_exact_gradients_finite_differences():
    W1, W2, X, T = _problem()
    g1, g2, L0 = lo.gradients_exact(W1, W2, X, T)
    eps = 1e-6
    rng = np.random.default_rng(1)
    for W, g in ((W1, g1), (W2, g2)):
        for _ in range(12):
            i = tuple(rng.integers(0, n) for n in W.shape)
            old = W[i]
            W[i] = old + eps
            Lp = lo.gradients_exact(W1, W2, X, T)[2]
            W[i] = old - eps
            Lm = lo.gradients_exact(W1, W2, X, T)[2]
            W[i] = old
            fd = (Lp - Lm) / (2 * eps)
            assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_kernel_rule_gradients_close_to_exact():
    W1, W2, X, T = _problem(seed=3, B=256)
    g1, g2, _ = lo.gradients_exact(W1, W2, X, T)
    b1, b2, loss = lo.gradients(W1, W2, X, T)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel(b1, g1) < 3e-2 and rel(b2, g2) < 3e-2
    # the library's loss is the mean over outputs
    assert loss > 0


def test_rotation_perms_against_library_nodes():
    from hopefoam_gb300.euler import reference_operators

    for N in (1, 2, 3, 4, 5, 6, 7):
        ops = reference_operators(N)
        ring = lo.ring_order(N)
        assert sorted(ring.tolist()) == list(range(ring.size))
        perm = lo.rotation_perms(ops["r"], ops["s"], ring)
        for fn in range(3):
            assert sorted(perm[fn].tolist()) == list(range(ring.size))
        assert np.array_equal(perm[0], np.arange(ring.size))
        # rotating face 1 onto face 0 three times is the identity
        p = np.arange(ring.size)
        for _ in range(3):
            p = p[perm[1]]
        assert np.array_equal(p, np.arange(ring.size))


def test_schwarz_scatter_is_the_transpose_of_gather():
    from hopefoam_gb300.euler import reference_operators
    from hopefoam_gb300.mesh import delaunay_square, periodic_square

    for N, mesh in ((3, delaunay_square(60, seed=4)), (2, periodic_square(3, 3, seed=2))):
        ops = reference_operators(N)
        ring = lo.ring_order(N)
        perm = lo.rotation_perms(ops["r"], ops["s"], ring)
        rng = np.random.default_rng(N)
        Np = ring.size
        v = rng.standard_normal((mesh.K, Np))
        Y = rng.standard_normal((mesh.K, 4 * Np))
        lhs = float((lo.schwarz_gather(v, mesh.EToE, mesh.EToF, perm) * Y).sum())
        rhs = float((v * lo.schwarz_scatter(Y, mesh.EToE, mesh.EToF, perm)).sum())
        assert abs(lhs - rhs) <= 1e-12 * max(1.0, abs(lhs))


def _mlp_problem(seed=0, N=2):
    from hopefoam_gb300.euler import reference_operators
    from hopefoam_gb300.mesh import delaunay_square

    mesh = delaunay_square(30, seed=seed)
    ops = reference_operators(N)
    ring = lo.ring_order(N)
    perm = lo.rotation_perms(ops["r"], ops["s"], ring)
    Np = ring.size
    rng = np.random.default_rng(seed + 7)
    n = mesh.K * Np
    Q = rng.standard_normal((n, n)) / np.sqrt(n)
    S = Q @ Q.T + np.eye(n)  # SPD stand-in for the SIPG operator

    def S_ring(z):
        return (S @ z.reshape(-1)).reshape(z.shape)

    r = rng.standard_normal((mesh.K, Np))
    zb = rng.standard_normal((mesh.K, Np)) * 0.3
    W = rng.standard_normal((16, 4 * Np)) * 0.3
    return mesh, perm, S_ring, r, zb, W


@pytest.mark.parametrize("slope", [0.0, 0.3])
def test_schwarz_mlp_exact_gradients_finite_differences(slope):
    """dL/dW of the two-layer Schwarz form against central differences of its
    energy loss (FP64, no rounding), relu and leaky activation."""
    mesh, perm, S_ring, r, zb, W = _mlp_problem()
    args = (r, zb, mesh.EToE, mesh.EToF, perm, S_ring)
    g, L0 = lo.schwarz_mlp_energy_gradients(W, *args, exact=True, slope=slope)
    assert abs(L0 - lo.schwarz_mlp_loss(W, *args, slope=slope)) <= 1e-12 * abs(L0)
    rng = np.random.default_rng(3)
    eps = 1e-6
    for _ in range(16):
        i = tuple(rng.integers(0, n) for n in W.shape)
        old = W[i]
        W[i] = old + eps
        Lp = lo.schwarz_mlp_loss(W, *args, slope=slope)
        W[i] = old - eps
        Lm = lo.schwarz_mlp_loss(W, *args, slope=slope)
        W[i] = old
        fd = (Lp - Lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, g[i])


def test_schwarz_mlp_positive_and_rounding_rules():
    """r . (M(r) - P r) >= 0 for every r (tied weights), M(a r) = a M(r) for
    a > 0, and the kernels' BF16 rules stay within 3 % of the exact gradient."""
    mesh, perm, S_ring, r, zb, W = _mlp_problem(seed=1)
    rng = np.random.default_rng(5)
    for _ in range(5):
        v = rng.standard_normal(r.shape)
        corr = lo.schwarz_mlp_apply(W, v, np.zeros_like(v), mesh.EToE, mesh.EToF, perm, exact=True)
        assert float((v * corr).sum()) >= 0.0
        c2 = lo.schwarz_mlp_apply(W, 2.5 * v, np.zeros_like(v), mesh.EToE, mesh.EToF, perm, exact=True)
        assert np.allclose(c2, 2.5 * corr, rtol=1e-12, atol=1e-12)
    args = (r, zb, mesh.EToE, mesh.EToF, perm, S_ring)
    g, _ = lo.schwarz_mlp_energy_gradients(W, *args, exact=True)
    gb, _ = lo.schwarz_mlp_energy_gradients(W, *args, exact=False)
    assert np.linalg.norm(gb - g) / np.linalg.norm(g) < 3e-2
