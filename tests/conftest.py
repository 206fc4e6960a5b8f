import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libdgcu.so")


def golden_mesh(name):
    from hopefoam_gb300.mesh import Mesh, connect

    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    EToV, VXY = d["EToV"], d["VXY"]
    EToE, EToF, ROT, BC = connect(EToV)
    m = Mesh(EToV, VXY, EToE, EToF, ROT, BC, name=name)
    if "patch" in d:
        m.patch = d["patch"]
        m.patch_names = tuple(str(x) for x in d["patch_names"])
    if "patch_first_face" in d:
        m.patch_first_face = d["patch_first_face"]
    if "arc_names" in d:
        from hopefoam_gb300.curved import ArcCurve

        m.curves = {str(n): ArcCurve.from_code(str(c), tuple(u), name=str(n))
                    for n, c, u in zip(d["arc_names"], d["arc_codes"], d["arc_u_range"])}
    return m


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.fixture(scope="session")
def gpu_lib():
    """The product library on a GPU; fails (not skips) when it cannot load."""
    import __graft_entry__ as g

    g.build()
    from hopefoam_gb300 import _lib

    return _lib.lib()
