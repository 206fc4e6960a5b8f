"""Batched cases on the GPU: the batch (cases of one order concatenated into
one context, per-element time steps, all stages in one CUDA graph) must give
every case exactly the result of that case run alone through its own context
(bit-identical in FP64: the per-element arithmetic does not depend on the
batching), after tuning as well as before, and graph replays must continue
the same trajectory."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases():
    from hopefoam_gb300.batch import batch_cases

    cs = batch_cases(n=7, seed=3, orders=(2, 3, 4), kmin=60, kmax=300)
    return cs


def _alone(case, nsteps, precision, cfl=0.5, gamma=1.4):
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.batch import _cfl_dt
    from hopefoam_gb300.euler import EulerContext, isentropic_vortex, node_coords, reference_operators
    from hopefoam_gb300.mesh import periodic_square

    N = case["order"]
    ops = reference_operators(N)
    m = periodic_square(case["m"], case["m"], 10.0, 10.0, perturb=0.1, seed=case["seed"])
    x, y = node_coords(m, ops["r"], ops["s"])
    q = isentropic_vortex(x, y, 0.0, beta=case["beta"], x0=5.0, y0=5.0, uinf=case["mach"] * np.sqrt(gamma),
                          gamma=gamma)
    ctx = EulerContext(m, N, gamma=gamma)
    ctx.upload(q)
    ctx.lserk4(_cfl_dt(m, q, N, cfl, gamma), nsteps, flux=L.DG_FLUX_LF, precision=precision)
    out = ctx.download()
    ctx.close()
    return out


def test_batch_matches_cases_alone_fp64(gpu_lib):
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.batch import EulerBatch

    cases = _cases()
    b = EulerBatch(cases)
    b.run(3, precision=L.DG_PREC_FP64)
    got = b.states()
    for i, c in enumerate(cases):
        ref = _alone(c, 3, L.DG_PREC_FP64)
        assert np.array_equal(got[i], ref), i
    b.close()


def test_batch_split_tuned_and_replayed(gpu_lib):
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.batch import EulerBatch

    cases = _cases()
    b1 = EulerBatch(cases)
    b1.run(2, precision=L.DG_PREC_SPLIT)
    b1.run(2, precision=L.DG_PREC_SPLIT)  # graph replay
    s1 = b1.states()
    b1.close()
    b2 = EulerBatch(cases)
    shape = b2.tune(precision=L.DG_PREC_SPLIT, steps_per_trial=1)
    assert shape["concurrent"] in (0, 1, 2) and len(shape["groups"]) == len({c["order"] for c in cases})
    assert shape["ms_fused"] > 0  # the one-launch-per-stage schedule was measured
    b2.run(4, precision=L.DG_PREC_SPLIT)
    s2 = b2.states()
    b2.close()
    for i, c in enumerate(cases):
        assert np.array_equal(s1[i], s2[i]), i
        ref = _alone(c, 4, L.DG_PREC_FP64)
        err = np.linalg.norm(s1[i] - ref) / np.linalg.norm(ref)
        # the split path's per-step bound on small meshes (TOL_STEP_SPLIT of
        # test_split_gpu.py) over the 4 steps
        assert err < 4e-8, (i, err)


@pytest.mark.parametrize("schedule", [1, 2])
def test_batch_schedules_bit_identical(gpu_lib, schedule):
    """Side by side on streams (1) and one mixed-order launch per stage (2)
    give every case the bits of the groups run one after another (0): each
    tile's arithmetic does not depend on which launch or CTA runs it."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.batch import EulerBatch

    cases = _cases()
    ref = EulerBatch(cases)
    ref.set_schedule(0)
    ref.run(3, precision=L.DG_PREC_SPLIT)
    s0 = ref.states()
    ref.close()
    b = EulerBatch(cases)
    b.set_schedule(schedule)
    b.run(2, precision=L.DG_PREC_SPLIT)
    b.run(1, precision=L.DG_PREC_SPLIT)  # a second graph (another step count) continues the trajectory
    s1 = b.states()
    b.close()
    for i in range(len(cases)):
        assert np.array_equal(s0[i], s1[i]), i


def test_batch_fused_rejected_in_fp64(gpu_lib):
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.batch import EulerBatch

    b = EulerBatch(_cases())
    with pytest.raises(L.DGError):
        b.set_schedule(2, precision=L.DG_PREC_FP64)
    b.close()


def test_batch_conservation_full_size(gpu_lib):
    """The batched configuration at its full size (512 cases, N 2..6, 3.1M
    elements), split precision, 10 LSERK4 steps in one graph: every case's
    domain totals of the conserved variables stay put (periodic cases) to
    FP32 round-off times dt -- a size-independent check of every case of the
    batch.  Measured worst case 1.6e-10 after 10 steps relative to the case's
    largest total (coarse cases take large steps); bound 5e-10."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.batch import EulerBatch, batch_cases
    from hopefoam_gb300.euler import reference_operators
    from hopefoam_gb300.mesh import periodic_square

    cases = batch_cases(512, seed=0)
    b = EulerBatch(cases)
    q0 = b.states()
    b.run(10, precision=L.DG_PREC_SPLIT)
    q1 = b.states()
    b.close()
    worst = 0.0
    w = {}
    for i, c in enumerate(cases):
        N = c["order"]
        if N not in w:
            w[N] = reference_operators(N)["Mref"].sum(axis=0)
        m = periodic_square(c["m"], c["m"], 10.0, 10.0, perturb=0.1, seed=c["seed"])
        v = m.VXY
        J = 0.25 * ((v[:, 1, 0] - v[:, 0, 0]) * (v[:, 2, 1] - v[:, 0, 1]) -
                    (v[:, 2, 0] - v[:, 0, 0]) * (v[:, 1, 1] - v[:, 0, 1]))
        t0 = np.einsum("k,vkp,p->v", J, q0[i], w[N])
        t1 = np.einsum("k,vkp,p->v", J, q1[i], w[N])
        assert np.all(np.isfinite(t1))
        worst = max(worst, float(np.max(np.abs(t1 - t0)) / np.max(np.abs(t0))))
    print("512 cases, 10 split steps: worst relative drift of a case's totals %.2e" % worst)
    assert worst < 5e-10
