"""Writes the committed fixtures of tests/golden/.

patch_test.json -- known answer of the reference's own patch test
  (tutorials/solids/linearElasticity/patchTest): displacement prescribed as
  D = a + b.x on every boundary (0/D, linearSpatialDisplacement with
  a = (1e-6 4e-6 0), b = (2e-6 3e-6 0; 5e-6 6e-6 0; 0 0 0)), E = 200 GPa,
  nu = 0.3; the strain must be constant, exx = 2e-6, eyy = 6e-6,
  exy = 4e-6 (patchTest/README.md, "Expected Results").

oracle_small.npz -- outputs of the CPU oracle on two small seeded cases
  (linear total displacement on a jittered 6x5x4 box, neo-Hookean total
  Lagrangian on a jittered 5x4x4 box, 3 load increments), a regression pin
  of the oracle and a fixture the GPU tests compare against without running
  the oracle.

foam_prisms/ -- not written by this script: a hand-written OpenFOAM case
  (ASCII polyMesh of a unit cube split along x = y into two triangular
  prisms, faces as a faceCompactList, and a 0/D boundaryField) whose
  volumes, centroids and area vectors are known exactly.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def patch_test():
    return {
        "source": "solids4foam tutorials/solids/linearElasticity/patchTest (0/D, README.md)",
        "a": [1e-6, 4e-6, 0.0],
        "b": [[2e-6, 3e-6, 0.0], [5e-6, 6e-6, 0.0], [0.0, 0.0, 0.0]],
        "E": 200e9,
        "nu": 0.3,
        "expected_strain": {"xx": 2e-6, "yy": 6e-6, "xy": 4e-6, "zz": 0.0, "xz": 0.0, "yz": 0.0},
    }


def small_cases():
    import solids4foam_gb300 as sg
    from oracle import pyoracle
    from solids4foam_gb300.cases import oracle_bcs

    out = {}
    m = sg.box_mesh(6, 5, 4, 1.2, 1.0, 0.8, 0.2, 11)
    ps = m["patch_size"]
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", np.tile([1e5, 0.0, -2e5], (int(ps[5]), 1)),
                    np.full(int(ps[5]), 3e5))}
    D, sig, G, perf = pyoracle.solve(m, oracle_bcs(m, bcs), E=70e9, nu=0.33, n_correctors=50)
    out.update(lin_D=D, lin_sigma=sig, lin_gradD=G, lin_ncorr=perf["n_correctors"],
               lin_iters=perf["total_lin_iters"])
    m2 = sg.box_mesh(5, 4, 4, 1.0, 0.8, 0.8, 0.15, 12)
    ps2 = m2["patch_size"]
    bcs2 = {"zmin": ("fixedDisplacement", None, None),
            "zmax": ("solidTraction", np.tile([0.0, 2e5, 0.0], (int(ps2[5]), 1)), None)}
    D2, s2, G2, p2 = pyoracle.solve(m2, oracle_bcs(m2, bcs2), model=1, law=1, use_mu_K=1,
                                    mu=1e6, K=2e7, n_correctors=40, n_increments=3)
    out.update(tl_D=D2, tl_sigma=s2, tl_gradD=G2, tl_ncorr=p2["n_correctors"],
               tl_iters=p2["total_lin_iters"])
    return out


def main():
    with open(os.path.join(HERE, "patch_test.json"), "w") as f:
        json.dump(patch_test(), f, indent=1)
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), **small_cases())


if __name__ == "__main__":
    main()
