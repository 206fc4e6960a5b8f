"""Curved arc patches on the GPU: the slope limiter reads the relocated node
locations (dg_set_node_locations, set by EulerContext for a mesh with curves)
and matches the oracle given the same locations (oracle.oracle.curved_nodes);
the operators keep the straight element's metrics, as the reference's do.
Tolerance 1e-12 relative, as the limiter's straight-mesh parity test."""
import numpy as np
import pytest

from conftest import golden_mesh, rel_l2

pytestmark = pytest.mark.gpu


def _radial(x, y):
    rr = np.hypot(x, y)
    return 0.05 * x / rr, 0.05 * y / rr


@pytest.mark.parametrize("N", [2, 4])
def test_limiter_on_curved_nodes(gpu_lib, N):
    from hopefoam_gb300 import euler
    from hopefoam_gb300.mesh import load_cubature
    from oracle.oracle import Oracle, curved_nodes

    m = golden_mesh("cylinder")
    ctx = euler.EulerContext(m, N)  # hands the curved node locations to the limiter
    orc = Oracle(m, N, load_cubature(3 * (N + 1)))
    xs, ys = orc.nodes()
    xc, yc = curved_nodes(orc, m, ("upcylinder", "downcylinder"), _radial)
    # a state with a steep front near the cylinder so that the limiter acts there
    rho = 1 + 0.5 * np.tanh((np.hypot(xs, ys) - 0.06) / 0.01) + 0.2 * np.sin(20 * xs)
    u, v = 0.3 + 0.1 * np.cos(15 * ys), 0.05 * np.sin(11 * xs)
    pr = 1 + 0.3 * np.tanh((xs + 0.02) / 0.02)
    q = np.stack([rho, rho * u, rho * v, pr / 0.4 + 0.5 * rho * (u * u + v * v)])
    kk, ff = euler.boundary_faces(m)
    fn = euler.face_nodes(N)
    bnd = np.stack([q[:, k, fn[f]] for k, f in zip(kk, ff)])
    kinds = np.zeros(len(kk), np.int32)
    names = list(m.patch_names)
    pid = m.patch[kk, ff]
    kinds[np.isin(pid, [names.index("upcylinder"), names.index("downcylinder"), names.index("channel")])] = 1
    kinds[pid == names.index("outlet")] = 2
    ctx.upload(q)
    ctx.set_boundary_traces(bnd)
    ctx.set_boundary_kinds(kinds)
    ctx.limit()
    qg = ctx.download()
    q_straight = orc.limiter(q, bnd, kinds)
    orc.set_nodes(xc, yc)
    qo = orc.limiter(q, bnd, kinds)
    err = rel_l2(qg, qo)
    print("limiter on curved nodes N=%d: GPU vs oracle %.2e; curved vs straight nodes %.2e" %
          (N, err, rel_l2(qo, q_straight)))
    assert err < 1e-12 and rel_l2(qo, q_straight) > 1e-10
    # node locations set after the limiter state exists replace the ones it holds
    ctx.set_node_locations(xs, ys)
    ctx.upload(q)
    ctx.limit()
    assert rel_l2(ctx.download(), q_straight) < 1e-12
    ctx.close()
