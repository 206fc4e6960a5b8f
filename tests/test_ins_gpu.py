"""The incompressible (Chorin) step on the GPU against the oracle
(oracle/ins_oracle.py), through the C ABI (dg_ins_*).

Tolerances: the operators are FP64 restatements of the same formulas:
1e-12 relative.  Whole steps: the GPU solves with block-Jacobi PCG to a
relative residual of 1e-13 where the oracle factorises (the reference uses
PETSc LU); 1e-9 relative on the state after 20 steps."""
import numpy as np
import pytest

from conftest import golden_mesh, rel_l2

pytestmark = pytest.mark.gpu


def _pair(mesh, N, **kw):
    from hopefoam_gb300.ins import ChorinSolver
    from hopefoam_gb300.mesh import load_cubature
    from oracle.ins_oracle import ChorinOracle

    g = ChorinSolver(mesh, N, **kw)
    o = ChorinOracle(mesh, N, load_cubature(3 * (N + 1)), **kw)
    return g, o


def _mesh(name):
    from hopefoam_gb300.ins import pearson_mesh

    return golden_mesh(name) if name.startswith("pearson_") and name[8:9] in "h0" else pearson_mesh(int(name))


@pytest.mark.parametrize("name,N", [("pearson_0.25h", 2), ("6", 4), ("5", 7)])
def test_operators_against_oracle(gpu_lib, name, N):
    from hopefoam_gb300.euler import face_nodes

    m = _mesh(name)
    g, o = _pair(m, N)
    x, y = o.x, o.y
    U = np.stack([np.sin(3 * x + 1) * np.cos(2 * y) + 0.3, np.cos(x - 2 * y) * 0.8 - 0.2 * x])
    p = np.cos(2 * x) * np.sin(3 * y + 0.5) + x * y
    # boundary values of the fixed-value faces: another smooth field at the face nodes
    ub_fn = lambda xx, yy: np.stack([0.5 * np.cos(xx + yy), 0.4 * np.sin(2 * xx - yy) + 0.1])
    fn = face_nodes(N)
    ub_kf = np.zeros((m.K, 3, 2, N + 1))
    for f in range(3):
        ub_kf[:, f] = ub_fn(x[:, fn[f]], y[:, fn[f]]).transpose(1, 0, 2)
    ub_slot = ub_kf[g.bk, g.bf]
    # the oracle takes the interior trace on fixed-gradient faces only through its caller
    trace = np.stack([U[:, :, fn[f]] for f in range(3)], 1).transpose(2, 1, 0, 3)
    ub_or = np.where(o.inlet[:, :, None, None], ub_kf, trace)
    Ng = g.operator(0, U, dict(u_value=ub_slot))
    No = o.O.convection(U, ub_or)
    assert rel_l2(Ng, No) < 1e-12
    assert rel_l2(g.operator(1, U), o.O.div_nodal(U)) < 1e-12
    assert rel_l2(g.operator(2, p), o.O.grad_nodal(p)) < 1e-12
    assert rel_l2(g.operator(3, U), o.O.curlcurl(U)) < 1e-11
    g.close()


def test_chorin_steps_against_oracle(gpu_lib):
    from hopefoam_gb300.ins import PearsonVortex

    m = golden_mesh("pearson_0.25h")
    g, o = _pair(m, 2, nu=0.01, dt=1e-3)
    pv = PearsonVortex(g)
    U0, p0 = pv.initial_state()
    g.set_state(U0, p0)
    t = 0.0
    for i in range(20):
        st = g.step(pv.bdata(t))
        o.step()
        t += g.dt
    Ug, pg = g.get_state()
    eu, ep = rel_l2(Ug, o.U), rel_l2(pg, o.p)
    print("20 Chorin steps, GPU vs oracle: U %.2e  p %.2e; last step PCG its p %d u %s" %
          (eu, ep, st["iterations_p"], st["iterations_u"]))
    assert eu < 1e-9 and ep < 1e-9
    g.close()


def test_pearson_vortex_convergence_on_gpu(gpu_lib):
    """The tutorial's run (N = 2, dt = 1e-3, 100 steps, nu = 0.01) on its three
    meshes: the GPU's pressure error equals the oracle's and converges."""
    from hopefoam_gb300.ins import PearsonVortex
    from hopefoam_gb300.mesh import load_cubature
    from oracle.ins_oracle import ChorinOracle

    errs = []
    for name in ("pearson_h", "pearson_0.5h", "pearson_0.25h"):
        m = golden_mesh(name)
        from hopefoam_gb300.ins import ChorinSolver

        g = ChorinSolver(m, 2, nu=0.01, dt=1e-3)
        pv = PearsonVortex(g)
        g.set_state(*pv.initial_state())
        t = 0.0
        for _ in range(100):
            g.step(pv.bdata(t))
            t += g.dt
        _, p = g.get_state()
        e = pv.pressure_error(p, t)
        o = ChorinOracle(m, 2, load_cubature(9), nu=0.01, dt=1e-3)
        for _ in range(100):
            o.step()
        eo = o.pressure_error()
        print(name, "pressure error avg/max GPU", e, "oracle", eo)
        assert abs(e[0] - eo[0]) < 1e-9 * max(1.0, eo[0]) + 1e-12
        errs.append(e[0])
        g.close()
    assert np.all(np.log2(np.array(errs[:-1]) / np.array(errs[1:])) > 2.0)


def test_cylinder_steps_against_oracle(gpu_lib):
    """The cylinder tutorial as it stands (its polyMesh with the arc patches,
    N = 3, nu = 0.001, dt = 2e-4) for ten steps against the oracle's
    CylinderCase.

    Tolerances: this case's pressure systems are far less well conditioned
    than the Pearson meshes' (graded mesh around the cylinder, Dirichlet data
    on the outlet only: condition number about 1e8) and their right-hand
    sides are small against |A| |p| (ratio up to 2e6 after the first steps),
    so an FP64 residual cannot fall much below 1e-10 of |b| -- the oracle's
    direct LU solutions leave 1e-12 to 2e-10 -- and PCG stops at a relative
    residual of 1e-10.  The condition number carries that into differences of
    order 1e-8 in the state: 1e-8 relative after the first step, 2e-7 after
    ten."""
    from hopefoam_gb300.ins import ChorinSolver, CylinderFlow
    from hopefoam_gb300.mesh import load_cubature
    from oracle.ins_oracle import ChorinOracle, CylinderCase

    m = golden_mesh("cylinder")
    N, nu, dt = CylinderFlow.ORDER, CylinderFlow.NU, CylinderFlow.DT
    uk, pk = CylinderFlow.kinds(m)
    g = ChorinSolver(m, N, nu=nu, dt=dt, u_kind=uk, p_kind=pk)
    cf = CylinderFlow(g)
    g.set_state(*cf.initial_state())
    o = ChorinOracle(m, N, load_cubature(3 * (N + 1)), nu=nu, dt=dt, case=CylinderCase(nu, dt))
    t = 0.0
    for i in range(10):
        st = g.step(cf.bdata(t), rtol=1e-10)
        o.step()
        t += dt
        if i == 0:
            U1, p1 = g.get_state()
            assert rel_l2(U1, o.U) < 1e-8 and rel_l2(p1, o.p) < 1e-8
    Ug, pg = g.get_state()
    eu, ep = rel_l2(Ug, o.U), rel_l2(pg, o.p)
    print("cylinder, 10 Chorin steps, GPU vs oracle: U %.2e  p %.2e; PCG its p %d u %s" %
          (eu, ep, st["iterations_p"], st["iterations_u"]))
    assert np.abs(Ug).max() > 1e-4 and eu < 2e-7 and ep < 2e-7
    g.close()


@pytest.mark.parametrize("N", [2, 3])
def test_chorin_steps_mixed_precision_solves(gpu_lib, N):
    """The step with mixed-precision linear solves (FP32 operator on FP64
    offsets, FP64 vectors, the same 1e-10 on the true FP64 residual) against
    the all-FP64 step: 20 Pearson-vortex steps agree to 1e-8 (both solves stop
    at a relative residual of 1e-10, so their solutions differ at that level
    times the systems' conditioning)."""
    from hopefoam_gb300 import _lib as L
    from hopefoam_gb300.ins import ChorinSolver, PearsonVortex

    m = golden_mesh("pearson_0.25h")
    res = []
    for prec in (L.DG_PREC_FP64, L.DG_PREC_SPLIT):
        g = ChorinSolver(m, N, nu=0.01, dt=1e-3, precision=prec)
        pv = PearsonVortex(g)
        g.set_state(*pv.initial_state())
        t = 0.0
        for _ in range(20):
            st = g.step(pv.bdata(t), rtol=1e-10)
            t += g.dt
        assert st["rel_residual_p"] <= 1e-10 and st["rel_residual_u"] <= 1e-10
        res.append(g.get_state())
        g.close()
    eu, ep = rel_l2(res[1][0], res[0][0]), rel_l2(res[1][1], res[0][1])
    print("N = %d, 20 steps, mixed vs FP64 solves: U %.2e  p %.2e" % (N, eu, ep))
    assert eu < 1e-8 and ep < 1e-8
