"""GPU parity of the processor-local (decomposed) DIC: the DIC restricted to
the library's scheduling parts, against the oracle given the same cell
decomposition -- what a decomposed OpenFOAM run with one processor per part
computes."""
import numpy as np
import pytest

import solids4foam_gb300 as sg
from solids4foam_gb300.cases import oracle_bcs
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("precision", ["FP64", "FP32_REFINE"])
def test_decomposed_dic_matches_oracle(ctx, precision):
    m = sg.box_mesh(12, 12, 12, 1.0, 1.0, 1.0, 0.2, 9)
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", None, np.full(int(m["patch_size"][5]), 1e7))}
    model = sg.SolidModel(ctx, m, dict(type="linearElastic", E=70e9, nu=0.33), bcs,
                          outer=dict(nCorrectors=2000), precision=precision, part_size=128,
                          dic_subdomains=True)
    D, sig, perf = model.evolve()
    perm, parts = model.permutation(), model.parts()
    assert len(set(parts.tolist())) == model.info()["n_parts"] > 1
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=perm, dic_domain=parts, E=70e9,
                                   nu=0.33, n_correctors=2000)
    assert perf["converged"] == 1 and po["converged"] == 1
    assert rel(D, Do) < 1e-6 and rel(sig, so) < 1e-5
    if precision == "FP64":
        # Same preconditioner and same iteration; the dot products are summed
        # in another order, so an inner solve may stop one iteration apart.
        assert abs(perf["n_correctors"] - po["n_correctors"]) <= 1
        assert abs(perf["total_lin_iters"] - po["total_lin_iters"]) <= 0.005 * po["total_lin_iters"]
    model.close()


def test_decomposed_tl_neo_hookean_matches_oracle(ctx):
    """The fused processor-local iteration inside the total Lagrangian loop
    (3 load increments), against the oracle with the same decomposition."""
    m = sg.box_mesh(8, 6, 6, 1.0, 0.8, 0.8, 0.15, 12)
    ps = m["patch_size"]
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", np.tile([0.0, 2e5, 0.0], (int(ps[5]), 1)), None)}
    law = dict(type="neoHookeanElastic", mu=1e6, K=2e7)
    model = sg.SolidModel(ctx, m, law, bcs, model="nonLinearGeometryTotalLagrangian",
                          outer=dict(nCorrectors=40), part_size=64, dic_subdomains=True)
    D, sig, perf = model.evolve(n_increments=3)
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(),
                                   dic_domain=model.parts(), model=1, law=1, use_mu_K=1,
                                   mu=1e6, K=2e7, n_correctors=40, n_increments=3)
    assert abs(perf["n_correctors"] - po["n_correctors"]) <= 1
    assert rel(D, Do) < 1e-6 and rel(sig, so) < 1e-5
    model.close()


@pytest.mark.parametrize("precision", ["FP64", "FP32_REFINE"])
def test_generic_part_tables_match_oracle(ctx, precision):
    """Caller parts (4^3-cell blocks of a 12^3 cube) in a shuffled cell
    order: rows have up to six lower in-part neighbours, so the
    preconditioner runs on the generic part tables, not the fixed slots;
    against the oracle with the same subdomains in the same order, and the
    autotuned and default variants bit-identical."""
    from oracle.box_mesh import block_parts
    m0 = sg.box_mesh(12, 12, 12, 1.0, 1.0, 1.0, 0.2, 9)
    shuffle = np.random.default_rng(2).permutation(12 ** 3)
    m = pyoracle.renumber_mesh(m0, shuffle)
    parts = block_parts(12, 12, 12, 4)[shuffle]
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", None, np.full(int(m["patch_size"][5]), 1e7))}
    # the shuffled order makes a weaker preconditioner and a slower outer
    # loop: both sides converge to 1e-9 so that where each stops stays well
    # inside the bars
    out = []
    for tune in (True, False):
        model = sg.SolidModel(ctx, m, dict(type="linearElastic", E=70e9, nu=0.33), bcs,
                              outer=dict(nCorrectors=6000, solutionTolerance=1e-9,
                                         alternativeTolerance=1e-9),
                              precision=precision, parts=parts, autotune=tune)
        assert model.info()["local_slots"] == 0
        D, sig, perf = model.evolve()
        out.append((D, sig, perf))
        model.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    D, sig, perf = out[0]
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), dic_domain=parts, E=70e9, nu=0.33,
                                   n_correctors=6000, solution_tol=1e-9, alternative_tol=1e-9)
    counts = (perf["n_correctors"], po["n_correctors"], perf["total_lin_iters"],
              po["total_lin_iters"])
    assert perf["converged"] == 1 and po["converged"] == 1, counts
    assert rel(D, Do) < 1e-6 and rel(sig, so) < 1e-5, (rel(D, Do), counts)
    if precision == "FP64":
        assert abs(perf["n_correctors"] - po["n_correctors"]) <= 0.01 * po["n_correctors"], counts


def test_decomposed_ragged_parts(ctx):
    """Small ragged parts (the smallest part size) and an uneven split still
    match the oracle."""
    m = sg.box_mesh(7, 5, 3, 1.0, 0.8, 0.6, 0.1, 4)
    bcs = {"xmin": ("fixedDisplacement", None, None),
           "xmax": ("solidTraction", np.tile([0.0, -1e5, 0.0], (int(m["patch_size"][1]), 1)), None)}
    law = dict(type="linearElastic", E=1e9, nu=0.3)
    for part in (32, 48):
        model = sg.SolidModel(ctx, m, law, bcs, outer=dict(nCorrectors=3000), part_size=part,
                              dic_subdomains=True)
        D, sig, perf = model.evolve()
        Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(),
                                       dic_domain=model.parts(), E=1e9, nu=0.3,
                                       n_correctors=3000)
        assert perf["converged"] == 1 and po["converged"] == 1
        assert rel(D, Do) < 1e-6 and rel(sig, so) < 1e-5
        model.close()


@pytest.mark.parametrize("precision", ["FP64", "FP32_REFINE"])
def test_autotuned_variants_are_bit_identical(ctx, precision):
    """The autotuner only picks among kernel variants whose sums run in the
    same order: the tuned and the untuned run give identical bits, whatever
    preconditioner variant (rows per thread in flight) and SpMV form
    each picks."""
    m = sg.box_mesh(14, 12, 10, 1.0, 0.9, 0.7, 0.2, 21)
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", None, np.full(int(m["patch_size"][5]), 1e7))}
    law = dict(type="linearElastic", E=70e9, nu=0.33)
    out = []
    for tune in (True, False):
        model = sg.SolidModel(ctx, m, law, bcs, outer=dict(nCorrectors=2000), precision=precision,
                              part_size=128, dic_subdomains=True, autotune=tune)
        D, sig, perf = model.evolve()
        assert perf["part_threads"] in (64, 128) and perf["spmv_unroll"] in (0, 1, 6)
        out.append((D, sig, perf["total_lin_iters"], perf["n_correctors"]))
        model.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2:] == out[1][2:]
