"""Learned element-block preconditioner on the GPU against its CPU
restatement (oracle/lpc_oracle.py), through the C ABI:
  * the BF16 training kernels' gradients on a random batch (rel L2 5e-3:
    BF16 rounding of the hidden layer may fall differently where the FP32
    sums differ in the last bit);
  * the inference kernel (features, block Jacobi with FP32 blocks, network)
    on a random residual (rel L2 1e-4 of z, 5e-3 of the network's part);
  * the energy-loss gradients of one residual (rel L2 5e-3; the library's
    S z runs in FP32 arithmetic, the oracle's in FP64);
  * training on the method's own PCG residuals lowers the energy loss
    below block Jacobi's, and a learned solve still ends at 1e-10 (through
    its block-Jacobi fallback when the learned iteration does not get there).
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TAU = 1.0


def _setup(n_interior=300, N=3, seed=5, hidden=32, capacity=0, form="relu"):
    from hopefoam_gb300.mesh import delaunay_square, load_cubature
    from hopefoam_gb300.poisson import PressureSolver
    from oracle import oracle

    mesh = delaunay_square(n_interior, seed=seed)
    ps = PressureSolver(mesh, N, tau_coef=TAU)
    ps.lpc_setup(hidden=hidden, seed=1, capacity=capacity, form=form)
    orc = oracle.Oracle(mesh, N, load_cubature(3 * (N + 1)))
    diag, off, _ = orc.ipdg_blocks(tau_coef=TAU)
    return mesh, ps, orc, diag, off


def _geometry(mesh):
    v = mesh.VXY
    xr, xs = (v[:, 1, 0] - v[:, 0, 0]) / 2, (v[:, 2, 0] - v[:, 0, 0]) / 2
    yr, ys = (v[:, 1, 1] - v[:, 0, 1]) / 2, (v[:, 2, 1] - v[:, 0, 1]) / 2
    J = xr * ys - xs * yr
    return np.stack([ys / J, -yr / J, -xs / J, xr / J], axis=1)


def _ring_tools(N):
    from hopefoam_gb300.euler import reference_operators
    from oracle import lpc_oracle as lo

    ops = reference_operators(N)
    ring = lo.ring_order(N)
    perm = lo.rotation_perms(ops["r"], ops["s"], ring)
    return ring, perm


def _random_weights(ps, seed=3, scale=1.0):
    rng = np.random.default_rng(seed)
    W1 = (rng.standard_normal((ps.lpc_hidden, ps.lpc_F)) * np.sqrt(2.0 / ps.lpc_F)).astype(np.float32)
    W2 = (rng.standard_normal((ps.Np, ps.lpc_hidden)) * scale / np.sqrt(ps.lpc_hidden)).astype(np.float32)
    ps.lpc_set_weights(W1, W2)
    return W1, W2


@pytest.mark.parametrize("linear", [False, True])
def test_mlp_gradients_match_oracle(gpu_lib, linear):
    from oracle import lpc_oracle as lo

    _, ps, _, _, _ = _setup(hidden=64, form="linear" if linear else "relu")
    W1, W2 = _random_weights(ps, seed=11, scale=0.5)
    rng = np.random.default_rng(2)
    B = 512
    X = lo.bf16(rng.standard_normal((B, ps.lpc_F)).astype(np.float32))
    T = rng.standard_normal((B, ps.Np)).astype(np.float32)
    g1, g2, loss = ps.lpc_gradients(X, T)
    o1, o2, oloss = lo.gradients(W1, W2, X, T, linear=linear)
    assert rel_l2(g1, o1) < 5e-3, rel_l2(g1, o1)
    assert rel_l2(g2, o2) < 5e-3, rel_l2(g2, o2)
    assert abs(loss - oloss) <= 1e-4 * abs(oloss)


@pytest.mark.parametrize("linear", [False, True])
def test_apply_matches_oracle(gpu_lib, linear):
    from oracle import lpc_oracle as lo

    mesh, ps, _, diag, _ = _setup(form="linear" if linear else "relu")
    W1, W2 = _random_weights(ps, seed=4, scale=1.0)
    ring, perm = _ring_tools(3)
    rng = np.random.default_rng(9)
    r = rng.standard_normal(ps.K * ps.Np)
    z = ps.lpc_apply(r).reshape(ps.K, ps.Np)
    zb = lo.block_jacobi32(-diag, r)
    zb_ring = zb[:, ring]
    z_ring = lo.precond(W1, W2, zb_ring, mesh.EToE, mesh.EToF, _geometry(mesh), perm, linear=linear)
    z_ref = np.empty_like(z_ring)
    z_ref[:, ring] = z_ring
    assert rel_l2(z, z_ref) < 1e-4, rel_l2(z, z_ref)
    zbr = np.empty_like(zb_ring)
    zbr[:, ring] = zb_ring
    assert rel_l2(z - zbr, z_ref - zbr) < 5e-3, rel_l2(z - zbr, z_ref - zbr)


def test_energy_gradients_match_oracle(gpu_lib):
    from oracle import lpc_oracle as lo

    mesh, ps, orc, diag, off = _setup()
    W1, W2 = _random_weights(ps, seed=6, scale=0.3)
    ring, perm = _ring_tools(3)
    rng = np.random.default_rng(10)
    r = rng.standard_normal(ps.K * ps.Np)
    g1, g2, loss = ps.lpc_energy_gradients(r)
    Np = ps.Np

    def S_ring(z_ring):
        zr = np.empty_like(z_ring)
        zr[:, ring] = z_ring
        y = -orc.blk_apply(diag, off, zr.reshape(-1)).reshape(-1, Np)
        return y[:, ring]

    zb_ring = lo.block_jacobi32(-diag, r)[:, ring]
    o1, o2, oloss = lo.energy_gradients(W1, W2, r.reshape(-1, Np)[:, ring], zb_ring, mesh.EToE, mesh.EToF,
                                        _geometry(mesh), perm, S_ring)
    assert rel_l2(g1, o1) < 5e-3, rel_l2(g1, o1)
    assert rel_l2(g2, o2) < 5e-3, rel_l2(g2, o2)
    assert abs(loss - oloss) <= 1e-5 * abs(oloss)


def test_schwarz_apply_matches_oracle(gpu_lib):
    from oracle import lpc_oracle as lo

    mesh, ps, _, diag, _ = _setup(form="schwarz", hidden=32)
    rng = np.random.default_rng(8)
    W = (rng.standard_normal((32, 4 * ps.Np)) * 0.2).astype(np.float32)
    ps.lpc_set_weights(W)
    ring, perm = _ring_tools(3)
    r = rng.standard_normal(ps.K * ps.Np)
    z = ps.lpc_apply(r).reshape(ps.K, ps.Np)
    zb_ring = lo.block_jacobi32(-diag, r)[:, ring]
    z_ring = lo.schwarz_apply(W, r.reshape(-1, ps.Np)[:, ring], zb_ring, mesh.EToE, mesh.EToF, perm)
    z_ref = np.empty_like(z_ring)
    z_ref[:, ring] = z_ring
    assert rel_l2(z, z_ref) < 1e-5, rel_l2(z, z_ref)


def test_schwarz_energy_gradients_match_oracle(gpu_lib):
    from oracle import lpc_oracle as lo

    mesh, ps, orc, diag, off = _setup(form="schwarz", hidden=32)
    rng = np.random.default_rng(12)
    W = (rng.standard_normal((32, 4 * ps.Np)) * 0.1).astype(np.float32)
    ps.lpc_set_weights(W)
    ring, perm = _ring_tools(3)
    r = rng.standard_normal(ps.K * ps.Np)
    g1, _, loss = ps.lpc_energy_gradients(r)
    Np = ps.Np

    def S_ring(z_ring):
        zr = np.empty_like(z_ring)
        zr[:, ring] = z_ring
        y = -orc.blk_apply(diag, off, zr.reshape(-1)).reshape(-1, Np)
        return y[:, ring]

    zb_ring = lo.block_jacobi32(-diag, r)[:, ring]
    o1, oloss = lo.schwarz_energy_gradients(W, r.reshape(-1, Np)[:, ring], zb_ring, mesh.EToE, mesh.EToF, perm, S_ring)
    assert rel_l2(g1, o1) < 5e-3, rel_l2(g1, o1)
    assert abs(loss - oloss) <= 1e-4 * abs(oloss)


def test_training_gains_and_solve(gpu_lib):
    """Trained on the solver's own residuals, the Schwarz form lowers the energy
    loss below block Jacobi's and its PCG reaches 1e-10 on its own in fewer
    iterations than block-Jacobi PCG."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.poisson import poisson_rhs

    snaps = (1, 2, 3, 5, 8, 13, 21, 34, 55, 89, 144, 233)
    mesh, ps, _, _, _ = _setup(n_interior=800, N=3, hidden=32, capacity=8 * len(snaps), form="schwarz")
    rhs = [poisson_rhs(mesh, 3, seed=40 + i)[0] for i in range(8)]
    n = ps.lpc_collect(rhs, snapshots=snaps)
    assert n == 8 * len(snaps)
    ps.lpc_train(epochs=15, lr=1e-3, seed=0)
    loss, loss_bj = ps.lpc_train(epochs=10, lr=3e-4, seed=1)
    assert loss < 1.5 * loss_bj, (loss, loss_bj)
    b = poisson_rhs(mesh, 3, seed=99)[0]
    x, st = ps.solve(b, rtol=1e-10, pc=L.DG_PC_LEARNED_ONLY, maxit=5000)
    xb, stb = ps.solve(b, rtol=1e-10, pc=L.DG_PC_BLOCK_JACOBI, maxit=5000)
    assert st["rel_residual"] <= 1e-10 and st["iterations"] > 0
    assert st["iterations"] < stb["iterations"], (st["iterations"], stb["iterations"])
    assert rel_l2(x, xb) < 1e-8
    # the learned local stage under the coarse-space correction: the same
    # solution, fewer iterations than either preconditioner alone
    for prec in (L.DG_PREC_SPLIT, L.DG_PREC_FP64):
        xm, stm = ps.solve(b, rtol=1e-10, pc=L.DG_PC_MULTILEVEL, maxit=5000, precision=prec)
        xl, stl = ps.solve(b, rtol=1e-10, pc=L.DG_PC_LEARNED_MULTILEVEL, maxit=5000, precision=prec)
        print("learned %d, multilevel %d, learned + multilevel %d iterations" %
              (st["iterations"], stm["iterations"], stl["iterations"]))
        assert stl["rel_residual"] <= 1e-10 and stl["iterations"] < st["iterations"]
        assert stl["iterations"] <= 1.2 * stm["iterations"]
        assert rel_l2(xl, xb) < 1e-8


def _s_ring(orc, diag, off, ring, Np):
    def S_ring(z_ring):
        zr = np.empty_like(z_ring)
        zr[:, ring] = z_ring
        y = -orc.blk_apply(diag, off, zr.reshape(-1)).reshape(-1, Np)
        return y[:, ring]
    return S_ring


@pytest.mark.parametrize("N,n_interior", [(1, 200), (3, 200), (4, 200), (6, 200), (4, 12000)])
def test_schwarz_mlp_apply_matches_oracle(gpu_lib, N, n_interior):
    """The tensor-core local stage of the two-layer form (BF16 hi + lo
    operands, FP32 accumulation) against the FP64 restatement: rel L2 2e-5
    of z and 1e-4 of the network's part (n_interior 12000: more tiles than
    CTAs, so each CTA runs several tiles)."""
    from oracle import lpc_oracle as lo

    mesh, ps, _, diag, _ = _setup(n_interior=n_interior, N=N, form="mlp", hidden=128)
    rng = np.random.default_rng(8 + N)
    W = (rng.standard_normal((128, 4 * ps.Np)) * 0.1).astype(np.float32)
    ps.lpc_set_weights(W)
    ring, perm = _ring_tools(N)
    r = rng.standard_normal(ps.K * ps.Np)
    z = ps.lpc_apply(r).reshape(ps.K, ps.Np)
    zb_ring = lo.block_jacobi32(-diag, r)[:, ring]
    z_ring = lo.schwarz_mlp_apply(W, r.reshape(-1, ps.Np)[:, ring], zb_ring, mesh.EToE, mesh.EToF, perm)
    z_ref = np.empty_like(z_ring)
    z_ref[:, ring] = z_ring
    zbr = np.empty_like(zb_ring)
    zbr[:, ring] = zb_ring
    assert rel_l2(z - zbr, z_ref - zbr) < 1e-4, rel_l2(z - zbr, z_ref - zbr)
    assert rel_l2(z, z_ref) < 2e-5, rel_l2(z, z_ref)


@pytest.mark.parametrize("N,n_interior,slope", [(3, 300, 0.0), (4, 300, 0.0), (4, 12000, 0.0), (4, 300, 0.5)])
def test_schwarz_mlp_energy_gradients_match_oracle(gpu_lib, N, n_interior, slope):
    """The BF16 tensor-core weight gradient against the restatement under the
    same rounding rules (rel L2 5e-3: a BF16 rounding or a relu mask may fall
    differently where the FP32 sums differ in the last bit) and against the
    exact FP64 gradient (rel L2 3e-2); n_interior 12000: several tiles per
    CTA."""
    from oracle import lpc_oracle as lo

    mesh, ps, orc, diag, off = _setup(n_interior=n_interior, N=N, form="mlp", hidden=128)
    rng = np.random.default_rng(12 + N)
    W = (rng.standard_normal((128, 4 * ps.Np)) * 0.05).astype(np.float32)
    ps.lpc_set_weights(W)
    ps.lpc_set_slope(slope)
    ring, perm = _ring_tools(N)
    r = rng.standard_normal(ps.K * ps.Np)
    g1, g2, loss = ps.lpc_energy_gradients(r)
    assert g2 is None
    Np = ps.Np
    S_ring = _s_ring(orc, diag, off, ring, Np)
    zb_ring = lo.block_jacobi32(-diag, r)[:, ring]
    args = (r.reshape(-1, Np)[:, ring], zb_ring, mesh.EToE, mesh.EToF, perm, S_ring)
    o1, oloss = lo.schwarz_mlp_energy_gradients(W, *args, slope=slope)
    e1, _ = lo.schwarz_mlp_energy_gradients(W, *args, exact=True, slope=slope)
    assert rel_l2(g1, o1) < 5e-3, rel_l2(g1, o1)
    assert rel_l2(g1, e1) < 3e-2, rel_l2(g1, e1)
    assert abs(loss - oloss) <= 1e-4 * abs(oloss)


def test_schwarz_mlp_training_and_solve(gpu_lib):
    """The two-layer form trained on the solver's own residuals with the
    tensor-core kernels: its energy loss ends below block Jacobi's, and its
    flexible PCG reaches 1e-10 on its own in fewer iterations than
    block-Jacobi PCG, at the same solution."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.poisson import poisson_rhs

    snaps = (1, 2, 3, 5, 8, 13, 21, 34, 55, 89, 144, 233)
    mesh, ps, _, _, _ = _setup(n_interior=800, N=3, hidden=128, capacity=8 * len(snaps), form="mlp")
    rhs = [poisson_rhs(mesh, 3, seed=40 + i)[0] for i in range(8)]
    assert ps.lpc_collect(rhs, snapshots=snaps) == 8 * len(snaps)
    ps.lpc_train(epochs=15, lr=1e-3, seed=0)
    loss, loss_bj = ps.lpc_train(epochs=10, lr=3e-4, seed=1)
    assert loss < 1.5 * loss_bj, (loss, loss_bj)
    b = poisson_rhs(mesh, 3, seed=99)[0]
    x, st = ps.solve(b, rtol=1e-10, pc=L.DG_PC_LEARNED_ONLY, maxit=5000)
    xb, stb = ps.solve(b, rtol=1e-10, pc=L.DG_PC_BLOCK_JACOBI, maxit=5000)
    print("two-layer learned %d, block Jacobi %d iterations; loss %.3f (block Jacobi %.3f)" %
          (st["iterations"], stb["iterations"], loss, loss_bj))
    assert st["rel_residual"] <= 1e-10 and st["iterations"] > 0
    assert st["iterations"] < stb["iterations"], (st["iterations"], stb["iterations"])
    assert rel_l2(x, xb) < 1e-8
    # the coarse-space combination takes the linear form only
    with pytest.raises(L.DGError):
        ps.solve(b, rtol=1e-10, pc=L.DG_PC_LEARNED_MULTILEVEL, maxit=10)


def test_learned_gains_over_same_form_without_learning(gpu_lib):
    """What training adds: the learned Schwarz form against the same form with
    a hand-built local map, W^T W = theta C, C the mean inverse of the
    interior patch operators of this mesh (the classical overlapping-Schwarz
    local solve shared by the patches, full rank, best theta of four), both
    to 1e-10 with plain CG.  The learned weights come from the training mesh
    (another mesh) and still need fewer iterations."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.poisson import PressureSolver, poisson_rhs, train_learned_preconditioner
    from oracle import lpc_oracle as lo

    N = 3
    mesh, ps, _, diag, off = _setup(n_interior=800, N=N, hidden=32, form="schwarz")
    ring, perm = _ring_tools(N)
    C = lo.schwarz_patch_inverse_mean(-diag, -off, mesh.EToE, mesh.EToF, ring, perm)
    W, _, _ = train_learned_preconditioner(N, tau_coef=TAU, form="schwarz", hidden=32)
    ps.lpc_set_weights(W)
    b = poisson_rhs(mesh, N, seed=99)[0]
    x, st = ps.solve(b, rtol=1e-10, pc=L.DG_PC_LEARNED_ONLY, maxit=5000)
    _, stb = ps.solve(b, rtol=1e-10, pc=L.DG_PC_BLOCK_JACOBI, maxit=5000)
    best = None
    for theta in (0.125, 0.25, 0.5, 1.0):
        p2 = PressureSolver(mesh, N, tau_coef=TAU)
        p2.lpc_setup(hidden=64, seed=0, capacity=0, form="schwarz")
        p2.lpc_set_weights(lo.schwarz_weights_from(C, theta, 64))
        xh, sth = p2.solve(b, rtol=1e-10, pc=L.DG_PC_LEARNED_ONLY, maxit=5000)
        p2.ctx.close()
        assert sth["rel_residual"] <= 1e-10 and rel_l2(xh, x) < 1e-8
        best = sth["iterations"] if best is None else min(best, sth["iterations"])
    print("learned %d, same form without learning (best theta) %d, block Jacobi %d iterations" %
          (st["iterations"], best, stb["iterations"]))
    assert st["rel_residual"] <= 1e-10
    assert st["iterations"] < 0.8 * best < 0.8 * stb["iterations"], (st["iterations"], best, stb["iterations"])


def test_learned_stage_trained_under_the_coarse_space(gpu_lib):
    """Trained with the coarse-space correction in its loss, the learned local
    stage under DG_PC_MULTILEVEL's correction needs about the multilevel
    preconditioner's own iteration count (trained alone it needs more), at
    the same solution."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.poisson import poisson_rhs, train_learned_preconditioner

    N = 3
    mesh, ps, _, _, _ = _setup(n_interior=800, N=N, hidden=32, form="schwarz")
    b = poisson_rhs(mesh, N, seed=99)[0]
    xm, stm = ps.solve(b, rtol=1e-10, pc=L.DG_PC_MULTILEVEL, maxit=5000)
    Wc, _, info = train_learned_preconditioner(N, tau_coef=TAU, coarse=True)
    assert info["loss"] < info["loss_block_jacobi"]  # below the coarse-corrected block Jacobi's loss
    ps.lpc_set_weights(Wc)
    xl, stl = ps.solve(b, rtol=1e-10, pc=L.DG_PC_LEARNED_MULTILEVEL, maxit=5000)
    print("multilevel %d, learned stage trained under it %d iterations" % (stm["iterations"], stl["iterations"]))
    assert stl["rel_residual"] <= 1e-10 and stl["iterations"] <= 1.1 * stm["iterations"]
    assert rel_l2(xl, xm) < 1e-8
