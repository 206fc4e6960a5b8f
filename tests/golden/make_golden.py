"""Generates the golden fixtures in this directory from the reference tree.

* ``vortex0256.npz`` / ``vortex1024.npz``: the isentropic-vortex tutorial
  meshes (HopeFOAM-0.1/tutorials/DG/2D/isentropicVortex/vortex0256.msh,
  vortex1024.msh) converted by hopefoam_gb300.meshio to (EToV, VXY) arrays, so
  the known-answer tests run where the reference tree is absent.
* ``pearson_h.npz`` / ``pearson_0.5h.npz`` / ``pearson_0.25h.npz``: the
  Pearson-vortex tutorial meshes (tutorials/DG/2D/pearsonVortex/vortexh.msh,
  vortex0.5h.msh, vortex0.25h.msh) with their inlet / outlet boundary patches.
* ``doublemach.npz``: the double-Mach-reflection tutorial mesh
  (tutorials/DG/2D/doubleMach/doubleMach.msh) with its patches and each
  patch's first face in file order.
* ``cylinder.npz``: the cylinder tutorial's polyMesh
  (tutorials/DG/2D/cylinder/constant/polyMesh) read by
  hopefoam_gb300.polymesh, with its patches and the code and u range of its
  two ``arc`` patches (the cylinder's halves).
* ``vortex_kat.json``: the reference's published accuracy table for that case
  ("2017-07-24-OpenFOAM workshop.pptx", slide 18: Roe flux, SSP-RK2, exact
  fixed-value boundary, t = 2; mean absolute nodal error of rho and |rhoU|),
  plus the time step that reproduces each entry with the oracle.

Usage: python tests/golden/make_golden.py [reference root]
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from hopefoam_gb300.meshio import read_fluent_msh  # noqa: E402
from hopefoam_gb300.polymesh import read_polymesh  # noqa: E402

# slide 18: order -> (rho err h, h/2, h/4, rhoU err h, h/2, h/4)
SLIDE18 = {
    1: (1.101e-02, 3.344e-03, 8.759e-04, 2.361e-02, 7.182e-03, 1.793e-03),
    2: (3.481e-03, 3.621e-04, 3.972e-05, 6.384e-03, 8.060e-04, 9.689e-05),
    3: (6.523e-04, 5.471e-05, 3.173e-06, 1.610e-03, 1.226e-04, 7.141e-06),
    4: (2.352e-04, 8.808e-06, 3.690e-07, 5.187e-04, 1.866e-05, 8.533e-07),
    5: (6.597e-05, 1.477e-06, 5.505e-08, 1.388e-04, 2.695e-06, 1.591e-07),
    6: (2.530e-05, 2.675e-07, 1.232e-08, 4.675e-05, 4.760e-07, 3.837e-08),
}


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HOPEFOAM_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_golden.py <reference root> (or set HOPEFOAM_REFERENCE_ROOT)")
    tut = os.path.join(root, "HopeFOAM-0.1", "tutorials", "DG", "2D", "isentropicVortex")
    for name in ["vortex0256", "vortex1024"]:
        m = read_fluent_msh(os.path.join(tut, name + ".msh"))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), EToV=m.EToV, VXY=m.VXY)
    pv = os.path.join(root, "HopeFOAM-0.1", "tutorials", "DG", "2D", "pearsonVortex")
    for src, name in (("vortexh", "pearson_h"), ("vortex0.5h", "pearson_0.5h"), ("vortex0.25h", "pearson_0.25h")):
        m = read_fluent_msh(os.path.join(pv, src + ".msh"))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), EToV=m.EToV, VXY=m.VXY, patch=m.patch,
                            patch_names=np.array(m.patch_names))
    m = read_fluent_msh(os.path.join(root, "HopeFOAM-0.1", "tutorials", "DG", "2D", "doubleMach", "doubleMach.msh"))
    np.savez_compressed(os.path.join(HERE, "doublemach.npz"), EToV=m.EToV, VXY=m.VXY, patch=m.patch,
                        patch_names=np.array(m.patch_names), patch_first_face=m.patch_first_face)
    cyl = os.path.join(root, "HopeFOAM-0.1", "tutorials", "DG", "2D", "cylinder", "constant", "polyMesh")
    m = read_polymesh(cyl)
    text = open(os.path.join(cyl, "boundary")).read()
    arcs = sorted(m.curves)
    codes, ranges = [], []
    for n in arcs:
        body = re.search(r"\b%s\s*\{((?:[^{}]|#\{.*?#\})*)\}" % n, text, re.S).group(1)
        codes.append(re.search(r"code\s*#\{(.*?)#\}", body, re.S).group(1).strip())
        ranges.append(m.curves[n].u_range)
    np.savez_compressed(os.path.join(HERE, "cylinder.npz"), EToV=m.EToV, VXY=m.VXY, patch=m.patch,
                        patch_names=np.array(m.patch_names), arc_names=np.array(arcs), arc_codes=np.array(codes),
                        arc_u_range=np.array(ranges))
    kat = {
        "source": "2017-07-24-OpenFOAM workshop.pptx, slide 18",
        "case": "isentropic vortex beta=5 centre (5,0) u_inf=1, gamma=1.4, Roe flux, SSP-RK2, exact fixed-value "
                "boundary, t_end=2, error = mean |q_exact - q| over nodes",
        "meshes": ["vortex0256", "vortex1024", "vortex4096"],
        "table": {str(k): {"rho": list(v[:3]), "rhoU": list(v[3:])} for k, v in SLIDE18.items()},
    }
    with open(os.path.join(HERE, "vortex_kat.json"), "w") as f:
        json.dump(kat, f, indent=1)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
