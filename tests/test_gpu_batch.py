"""Batched load cases (s4g_solve_cases): every case of a batch must equal,
bit for bit, the single solve of the same mesh with that case's boundary
values -- same corrector and PCG iteration counts, same D and sigma -- and
cases converge independently (a zero-load case and strong cases side by
side).  Many meshes in one launch (s4g_solve_batch) likewise."""
import numpy as np
import pytest

import solids4foam_gb300 as sg
from solids4foam_gb300 import _lib

pytestmark = pytest.mark.gpu


def cube_cases(n, n_cases, seed):
    m = sg.box_mesh(n, n, n, 1.0, 1.0, 1.0, 0.2, seed)
    rng = np.random.default_rng(seed)
    tractions = rng.normal(0.0, 1e6, (n_cases, 3))
    tractions[1] = 0.0  # a case with no load
    cases = [{"zmin": ("fixedDisplacement", None, None),
              "zmax": ("solidTraction", t, None)} for t in tractions]
    return m, cases


@pytest.mark.parametrize("precision", ["FP64", "FP32_REFINE"])
def test_each_case_equals_its_single_solve(ctx, precision):
    m, cases = cube_cases(12, 5, 3)
    law = dict(type="linearElastic", E=200e9, nu=0.3)
    kw = dict(outer=dict(nCorrectors=2000), precision=precision, part_size=128,
              dic_subdomains=True)
    batch = sg.SolidModel(ctx, m, law, cases[0], **kw)
    Db, sb, perfs = batch.evolve_cases(cases)
    batch.close()
    counts = set()
    for c, bcs in enumerate(cases):
        single = sg.SolidModel(ctx, m, law, bcs, **kw)
        D, sig, perf = single.evolve()
        single.close()
        assert perfs[c]["n_correctors"] == perf["n_correctors"]
        assert perfs[c]["total_lin_iters"] == perf["total_lin_iters"]
        assert perfs[c]["converged"] == perf["converged"] == 1
        assert np.array_equal(Db[c], D) and np.array_equal(sb[c], sig)
        counts.add(perf["n_correctors"])
    assert np.all(Db[1] == 0.0)
    assert len(counts) > 1  # the cases did not all stop together


def test_batch_after_single_and_growth(ctx):
    """A single solve, a batch that grows the per-case arrays, then the
    single solve again: identical results (the mesh's own boundary values
    are restored after the batch)."""
    m, cases = cube_cases(8, 3, 5)
    law = dict(type="linearElastic", E=70e9, nu=0.33)
    model = sg.SolidModel(ctx, m, law, cases[2], outer=dict(nCorrectors=2000),
                          part_size=64, dic_subdomains=True)
    D0, s0, _ = model.evolve()
    Db, sb, _ = model.evolve_cases(cases)
    D1, s1, _ = model.evolve()
    assert np.array_equal(D0, D1) and np.array_equal(s0, s1)
    assert np.array_equal(Db[2], D0)
    model.close()


def test_batch_needs_the_local_dic(ctx):
    m, cases = cube_cases(6, 2, 7)
    model = sg.SolidModel(ctx, m, dict(type="linearElastic", E=70e9, nu=0.33), cases[0])
    with pytest.raises(_lib.S4GError, match="dic_subdomains"):
        model.evolve_cases(cases)
    model.close()


def test_solve_batch_equals_single_solves_and_the_oracle():
    """s4g_solve_batch: meshes of the many-mesh batch form (jittered boxes of
    uneven sizes and aspect ratios, E and nu drawn per mesh, field
    relaxation where nu is high) advanced by one CUDA-graph launch, each
    mesh's device-resident loop a branch of it.  Every mesh's result is
    bit-identical to its own s4g_solve, and one is checked against the
    oracle."""
    from oracle import pyoracle
    from solids4foam_gb300.cases import mesh_batch, oracle_bcs
    cases = mesh_batch(6, seed=11)
    c0 = sg.Context(0)
    models = [sg.SolidModel(c0, c["mesh"], c["law"], c["bcs"], outer=c["outer"],
                            precision="FP32_REFINE", parts=c["parts"]) for c in cases]
    res = sg.solve_batch(models)
    for (D, sig, perf), m in zip(res, models):
        assert perf["converged"] == 1 and perf["device_loop"] == 1
        D1, s1, p1 = m.evolve()
        assert np.array_equal(D, D1) and np.array_equal(sig, s1)
        assert p1["n_correctors"] == perf["n_correctors"]
        assert p1["total_lin_iters"] == perf["total_lin_iters"]
    k = min(range(len(cases)), key=lambda i: cases[i]["mesh"]["V"].shape[0])
    c = cases[k]
    Do, so, _, po = pyoracle.solve(c["mesh"], oracle_bcs(c["mesh"], c["bcs"]), dic_domain=c["parts"],
                                   E=c["law"]["E"], nu=c["law"]["nu"],
                                   n_correctors=c["outer"]["nCorrectors"],
                                   field_relaxation=c["outer"].get("fieldRelaxation", 1.0),
                                   solution_tol=c["outer"].get("solutionTolerance", 1e-6),
                                   alternative_tol=c["outer"].get("alternativeTolerance", 1e-7),
                                   n_threads=8)
    assert po["converged"] == 1
    D, sig, _ = res[k]
    assert np.linalg.norm(D - Do) / np.linalg.norm(Do) < 1e-6
    assert np.linalg.norm(sig - so) / np.linalg.norm(so) < 1e-5
    for m in models:
        m.close()
    c0.close()
