"""Serving (s4g_server_*): requests of uneven sizes and two models run at
the same time on one GPU, and each result is the same alone and in the mix
(tolerance 1e-12 relative L2; the runs are in fact bit-identical), and the
same as a direct solve of the same inputs."""
import numpy as np
import pytest

import solids4foam_gb300 as sg
from solids4foam_gb300 import _lib

pytestmark = pytest.mark.gpu
TOL = 1e-12
# a result comes back with the solve's status: converged, or the corrector
# limit reached (the total Lagrangian request stops at 40 correctors per
# increment, as the reference's "Max iterations reached" warning would)
DONE = (_lib.OK, _lib.NOT_CONVERGED)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def requests():
    lin = dict(type="linearElastic", E=200e9, nu=0.3)
    neo = dict(type="neoHookeanElastic", mu=1e6, K=2e7)
    out = []
    for n, seed, prec, sub in ((10, 1, "FP64", False), (16, 2, "FP32_REFINE", True),
                               (12, 3, "FP64", True), (8, 4, "FP32_REFINE", False)):
        m = sg.box_mesh(n, n, n, 1.0, 1.0, 1.0, 0.2, seed)
        bcs = {"zmin": ("fixedDisplacement", None, None),
               "zmax": ("solidTraction", [1e5 * seed, 0.0, -1e6], None)}
        out.append(dict(mesh=m, law=lin, bcs=bcs, precision=prec, dic_subdomains=sub,
                        outer=dict(nCorrectors=2000)))
    m = sg.box_mesh(6, 5, 5, 1.0, 0.8, 0.8, 0.15, 12)
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", np.tile([0.0, 2e5, 0.0], (int(m["patch_size"][5]), 1)), None)}
    out.append(dict(mesh=m, law=neo, bcs=bcs, model="nonLinearGeometryTotalLagrangian",
                    n_increments=3, outer=dict(nCorrectors=40)))
    return out


def test_alone_and_in_the_mix_agree(ctx):
    reqs = requests()
    srv = sg.Server(max_slots=4)
    alone = []
    for r in reqs:  # one at a time
        rid = srv.submit(**r)
        st, D, sig, perf = srv.result(rid)
        assert st in DONE
        alone.append((D, sig, st))
    ids = [srv.submit(**r) for r in reqs + reqs]  # all together, twice over
    for k, rid in enumerate(ids):
        st, D, sig, perf = srv.result(rid)
        Da, sa, sta = alone[k % len(reqs)]
        assert st == sta
        assert rel(D, Da) <= TOL and rel(sig, sa) <= TOL
    stats = srv.stats()
    assert stats["completed"] == 3 * len(reqs) and stats["rejected"] == 0
    assert 0 < stats["p50_ms"] <= stats["p99_ms"]
    srv.close()
    # the same as a direct solve through a SolidModel
    r = reqs[1]
    model = sg.SolidModel(ctx, r["mesh"], r["law"], r["bcs"], outer=r["outer"],
                          precision=r["precision"], dic_subdomains=r["dic_subdomains"])
    D, sig, _ = model.evolve()
    model.close()
    assert rel(D, alone[1][0]) <= TOL and rel(sig, alone[1][1]) <= TOL


def test_admission_rejects_what_cannot_fit():
    srv = sg.Server(max_slots=2, memory_budget=32 << 20)
    m = sg.box_mesh(40, 40, 40, 1.0, 1.0, 1.0, 0.1, 1)
    with pytest.raises(_lib.S4GError, match="ADMISSION_REJECTED"):
        srv.submit(m, dict(type="linearElastic", E=70e9, nu=0.33),
                   {"zmin": ("fixedDisplacement", None, None)})
    assert srv.stats()["rejected"] == 1
    srv.close()
