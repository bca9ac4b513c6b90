"""GPU parity: the CUDA path through the C ABI against the CPU oracle run in
the same DIC order, operator by operator and for whole solves.

Bars (written here, from the solve's specification): relative L2 error of
D <= 1e-6 and of sigma <= 1e-5 against the FP64 oracle at the same
settings.  With identical DIC orders the two runs take the same iteration
counts, so the errors are at round-off level; the tests also assert that.
"""
import os

import numpy as np
import pytest

import solids4foam_gb300 as sg
from solids4foam_gb300 import _lib
from solids4foam_gb300.cases import oracle_bcs
from oracle import pyoracle

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
TOL_D, TOL_S = 1e-6, 1e-5


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def cube(n, seed=1, jitter=0.2, pressure=1e7):
    m = sg.box_mesh(n, n, n, 1.0, 1.0, 1.0, jitter, seed)
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", None, np.full(int(m["patch_size"][5]), pressure))}
    return m, bcs


def impK_of(E, nu):
    mu = E / (2 * (1 + nu))
    lam = nu * E / ((1 + nu) * (1 - 2 * nu))
    return 2 * mu + lam


@pytest.mark.parametrize("renumber", ["none", "RCM", "tiled"])
def test_operators_match_oracle(ctx, renumber):
    m, bcs = cube(10, seed=3)
    law = dict(type="linearElastic", E=70e9, nu=0.33)
    model = sg.SolidModel(ctx, m, law, bcs, renumber=renumber, part_size=64)
    perm = model.permutation()
    mo = pyoracle.renumber_mesh(m, perm)
    bo = oracle_bcs(m, bcs)
    do, uo = pyoracle.matrix(mo, bo, impK_of(70e9, 0.33))
    diag, upper = model.op_matrix()
    assert rel(diag[perm], do) < 1e-14
    # upper: map caller faces to the renumbered face order of the oracle
    ni = m["neighbour"].shape[0]
    inv = np.empty(m["V"].shape[0], np.int64)
    inv[perm] = np.arange(perm.shape[0])
    a, b = inv[m["owner"][:ni]], inv[m["neighbour"]]
    key_caller = np.minimum(a, b) * 10**7 + np.maximum(a, b)
    key_oracle = mo["owner"][:ni].astype(np.int64) * 10**7 + mo["neighbour"]
    pos = np.searchsorted(key_oracle, key_caller)
    assert rel(upper, uo[pos]) < 1e-14
    x = np.random.default_rng(0).standard_normal((perm.shape[0], 3))
    y = model.op_amul(x)
    w = model.op_precondition(x)
    for k in range(3):
        yo = pyoracle.amul(mo, do, uo, x[perm, k])
        wo = pyoracle.dic(mo, do, uo, x[perm, k])
        assert rel(y[perm, k], yo) < 1e-14
        assert rel(w[perm, k], wo) < 1e-13
    # one column at a time gives the same result
    w1 = model.op_precondition(x[:, 1].copy())
    assert rel(w1, w[:, 1]) < 1e-15
    model.close()


@pytest.mark.parametrize("renumber,part", [("none", 128), ("RCM", 96), ("tiled", 64), ("tiled", 512)])
def test_linear_solve_matches_oracle(ctx, renumber, part):
    m, bcs = cube(12, seed=5)
    law = dict(type="linearElastic", E=70e9, nu=0.33)
    outer = dict(nCorrectors=2000, solutionTolerance=1e-6)
    model = sg.SolidModel(ctx, m, law, bcs, outer=outer, renumber=renumber, part_size=part)
    D, sig, perf = model.evolve()
    perm = model.permutation()
    Do, so, Go, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=perm, E=70e9, nu=0.33,
                                    n_correctors=2000)
    assert perf["converged"] == 1 and po["converged"] == 1
    assert perf["n_correctors"] == po["n_correctors"]
    assert perf["total_lin_iters"] == po["total_lin_iters"]
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S
    assert rel(D, Do) < 1e-12
    G = model.gradD()
    assert rel(G, Go) < 1e-10
    model.close()


def test_cantilever_matches_oracle(ctx):
    """The 80x8x8 cantilever at its 2000-corrector cap (not converged in the
    reference either): same corrector count, same fields."""
    c = sg.cantilever_case()
    model = sg.SolidModel(ctx, c["mesh"], c["law"], c["bcs"], solver=c["solver"], outer=c["outer"])
    D, sig, perf = model.evolve()
    perm = model.permutation()
    Do, so, _, po = pyoracle.solve(c["mesh"], oracle_bcs(c["mesh"], c["bcs"]), perm=perm,
                                   E=200e9, nu=0.3, n_correctors=2000)
    assert perf["n_correctors"] == po["n_correctors"] == 2000
    assert perf["converged"] == po["converged"]
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S
    model.close()


def test_diagonal_preconditioner_matches_oracle(ctx):
    m, bcs = cube(8, seed=2)
    law = dict(type="linearElastic", E=200e9, nu=0.3)
    model = sg.SolidModel(ctx, m, law, bcs, solver=dict(preconditioner="diagonal"),
                          outer=dict(nCorrectors=80))
    D, sig, perf = model.evolve()
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(), E=200e9,
                                   nu=0.3, n_correctors=80, preconditioner=1)
    assert perf["total_lin_iters"] == po["total_lin_iters"]
    assert rel(D, Do) < 1e-12 and rel(sig, so) < 1e-11
    model.close()


def test_golden_fixture_linear(ctx):
    g = np.load(os.path.join(HERE, "golden", "oracle_small.npz"))
    m = sg.box_mesh(6, 5, 4, 1.2, 1.0, 0.8, 0.2, 11)
    ps = m["patch_size"]
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", np.tile([1e5, 0.0, -2e5], (int(ps[5]), 1)),
                    np.full(int(ps[5]), 3e5))}
    model = sg.SolidModel(ctx, m, dict(type="linearElastic", E=70e9, nu=0.33), bcs,
                          outer=dict(nCorrectors=50), renumber="none")
    D, sig, perf = model.evolve()
    assert perf["n_correctors"] == int(g["lin_ncorr"])
    assert rel(D, g["lin_D"]) < 1e-12 and rel(sig, g["lin_sigma"]) < 1e-11
    model.close()


def test_determinism(ctx):
    m, bcs = cube(10, seed=8)
    model = sg.SolidModel(ctx, m, dict(type="linearElastic", E=70e9, nu=0.33), bcs,
                          outer=dict(nCorrectors=50))
    D1, s1, _ = model.evolve()
    D2, s2, _ = model.evolve()
    assert np.array_equal(D1, D2) and np.array_equal(s1, s2)
    model.close()


def test_not_converged_returns_result(ctx):
    m, bcs = cube(6)
    model = sg.SolidModel(ctx, m, dict(type="linearElastic", E=70e9, nu=0.33), bcs,
                          outer=dict(nCorrectors=3))
    D, sig, perf = model.evolve()
    assert perf["converged"] == 0 and perf["n_correctors"] == 3
    assert np.isfinite(D).all() and np.abs(D).max() > 0
    model.close()


def test_bad_arguments(ctx):
    m, bcs = cube(4)
    model = sg.SolidModel(ctx, m, dict(type="linearElastic", E=70e9, nu=0.33), bcs)
    with pytest.raises(sg.S4GError):
        model.set_bc(0, "solidTraction", np.full(3, np.nan))
    with pytest.raises(sg.S4GError):
        model.set_law(dict(type="linearElastic", E=70e9, nu=0.7))
    with pytest.raises(sg.S4GError) as e:
        sg.SolidModel(ctx, m, dict(type="linearElastic", E=70e9, nu=0.33), bcs,
                      model="nonLinearGeometryTotalLagrangian").evolve()
    assert e.value.status == _lib.BAD_ARG
    model.close()


def test_tl_neo_hookean_matches_oracle(ctx):
    """nonLinearGeometryTotalLagrangian + neoHookeanElastic, 3 load
    increments, against the oracle in the same DIC order."""
    m = sg.box_mesh(6, 5, 5, 1.0, 0.8, 0.8, 0.15, 12)
    ps = m["patch_size"]
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", np.tile([0.0, 2e5, 0.0], (int(ps[5]), 1)), None)}
    law = dict(type="neoHookeanElastic", mu=1e6, K=2e7)
    model = sg.SolidModel(ctx, m, law, bcs, model="nonLinearGeometryTotalLagrangian",
                          outer=dict(nCorrectors=40))
    D, sig, perf = model.evolve(n_increments=3)
    Do, so, Go, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(), model=1,
                                    law=1, use_mu_K=1, mu=1e6, K=2e7, n_correctors=40,
                                    n_increments=3)
    assert perf["n_correctors"] == po["n_correctors"]
    assert perf["total_lin_iters"] == po["total_lin_iters"]
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S
    assert rel(D, Do) < 1e-10
    assert rel(model.gradD(), Go) < 1e-9
    model.close()


def test_traction_relaxation_matches_oracle(ctx):
    """solidTraction relaxationFactor 0.5 on the linear-geometry model."""
    m, _ = cube(8, seed=3)
    t = np.tile([1e5, 0.0, -1e6], (int(m["patch_size"][5]), 1))
    bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", t, None, 0.5)}
    law = dict(type="linearElastic", E=200e9, nu=0.3)
    model = sg.SolidModel(ctx, m, law, bcs, outer=dict(nCorrectors=4000))
    D, sig, perf = model.evolve()
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(), E=200e9,
                                   nu=0.3, n_correctors=4000)
    assert po["converged"] == 1
    assert perf["n_correctors"] == po["n_correctors"]
    assert perf["total_lin_iters"] == po["total_lin_iters"]
    assert rel(D, Do) < 1e-10 and rel(sig, so) < 1e-9
    model.close()


def test_tl_traction_increments_relaxed_match_oracle(ctx):
    """Total Lagrangian traction load over two increments with
    relaxationFactor 0.5: the first update of the second increment relaxes
    against the gradient the last corrector of the first one used."""
    m = sg.box_mesh(6, 5, 5, 1.0, 0.8, 0.8, 0.15, 12)
    t = np.tile([0.0, 2e4, 0.0], (int(m["patch_size"][5]), 1))
    bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", t, None, 0.5)}
    law = dict(type="neoHookeanElastic", mu=1e6, K=2e7)
    model = sg.SolidModel(ctx, m, law, bcs, model="nonLinearGeometryTotalLagrangian",
                          outer=dict(nCorrectors=6000))
    D, sig, perf = model.evolve(n_increments=2)
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(), model=1,
                                   law=1, use_mu_K=1, mu=1e6, K=2e7, n_correctors=6000,
                                   n_increments=2)
    assert po["converged"] == 1 and perf["converged"] == 1
    assert perf["n_correctors"] == po["n_correctors"]
    assert perf["total_lin_iters"] == po["total_lin_iters"]
    assert rel(D, Do) < 1e-10 and rel(sig, so) < 1e-9
    model.close()


@pytest.mark.parametrize("load,n_increments", [("traction", 2), ("displacement", 3)])
def test_tl_total_displacement_matches_oracle(ctx, load, n_increments):
    """nonLinearGeometryTotalLagrangianTotalDisplacement + neoHookeanElastic
    over several increments, against the oracle in the same DIC order."""
    m = sg.box_mesh(6, 5, 5, 1.0, 0.8, 0.8, 0.15, 12)
    top = int(m["patch_size"][5])
    if load == "traction":
        zmax = ("solidTraction", np.tile([0.0, 2e4, 0.0], (top, 1)), None)
    else:
        zmax = ("fixedDisplacement", np.tile([0.0, 0.05, 0.1], (top, 1)), None)
    bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": zmax}
    law = dict(type="neoHookeanElastic", mu=1e6, K=2e7)
    model = sg.SolidModel(ctx, m, law, bcs,
                          model="nonLinearGeometryTotalLagrangianTotalDisplacement",
                          outer=dict(nCorrectors=6000))
    D, sig, perf = model.evolve(n_increments=n_increments)
    Do, so, Go, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(), model=2,
                                    law=1, use_mu_K=1, mu=1e6, K=2e7, n_correctors=6000,
                                    n_increments=n_increments)
    assert po["converged"] == 1 and perf["converged"] == 1
    # The right-hand side is summed in another order on the GPU (residual
    # form, face pass), so over ~10^3 converged correctors an inner solve
    # may stop one iteration apart.
    assert abs(perf["n_correctors"] - po["n_correctors"]) <= 1
    assert abs(perf["total_lin_iters"] - po["total_lin_iters"]) <= 0.005 * po["total_lin_iters"]
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S
    assert rel(model.gradD(), Go) < TOL_S
    if perf["total_lin_iters"] == po["total_lin_iters"]:
        assert rel(D, Do) < 1e-10 and rel(sig, so) < 1e-9
    model.close()


@pytest.mark.parametrize("dic_subdomains", [False, True])
def test_prism_mesh_from_polymesh_matches_oracle(ctx, tmp_path, dic_subdomains):
    """A mesh of triangular prisms written and read back as an OpenFOAM
    polyMesh: the GPU solve against the oracle in the same DIC order (exact
    DIC, or processor-local DIC over 64-cell parts)."""
    from solids4foam_gb300.foam_case import prism_box_polymesh, read_case, write_polymesh
    write_polymesh(str(tmp_path / "constant" / "polyMesh"),
                   **prism_box_polymesh(6, 5, 4, 1.0, 0.9, 0.8))
    m, _ = read_case(str(tmp_path), d_file=None)
    top = int(m["patch_size"][5])
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", np.tile([1e5, 0.0, -1e6], (top, 1)), None)}
    law = dict(type="linearElastic", E=200e9, nu=0.3)
    model = sg.SolidModel(ctx, m, law, bcs, outer=dict(nCorrectors=3000), ls_boundary_delta=1,
                          part_size=64, dic_subdomains=dic_subdomains)
    D, sig, perf = model.evolve()
    kw = dict(perm=model.permutation(), E=200e9, nu=0.3, n_correctors=3000, ls_boundary_delta=1)
    if dic_subdomains:
        kw["dic_domain"] = model.parts()
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), **kw)
    assert po["converged"] == 1 and perf["converged"] == 1
    assert abs(perf["n_correctors"] - po["n_correctors"]) <= 1
    assert abs(perf["total_lin_iters"] - po["total_lin_iters"]) <= 0.005 * po["total_lin_iters"]
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S
    model.close()


def test_golden_fixture_tl(ctx):
    g = np.load(os.path.join(HERE, "golden", "oracle_small.npz"))
    m = sg.box_mesh(5, 4, 4, 1.0, 0.8, 0.8, 0.15, 12)
    ps = m["patch_size"]
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", np.tile([0.0, 2e5, 0.0], (int(ps[5]), 1)), None)}
    model = sg.SolidModel(ctx, m, dict(type="neoHookeanElastic", mu=1e6, K=2e7), bcs,
                          model="nonLinearGeometryTotalLagrangian", outer=dict(nCorrectors=40),
                          renumber="none")
    D, sig, perf = model.evolve(n_increments=3)
    assert perf["n_correctors"] == int(g["tl_ncorr"])
    assert rel(D, g["tl_D"]) < 1e-10 and rel(sig, g["tl_sigma"]) < 1e-9
    model.close()


@pytest.mark.parametrize("renumber", ["tiled", "none"])
def test_fp32_refine_converges_to_fp64_fixed_point(ctx, renumber):
    """FP32 inner PCG with FP64 refinement: converged tightly, the result
    equals the FP64 oracle's converged result to <= 1e-6 (D) / 1e-5 (sigma)."""
    m, bcs = cube(12, seed=6)
    law = dict(type="linearElastic", E=70e9, nu=0.33)
    outer = dict(nCorrectors=5000, solutionTolerance=1e-10, alternativeTolerance=1e-11)
    model = sg.SolidModel(ctx, m, law, bcs, outer=outer, precision="FP32_REFINE",
                          renumber=renumber, part_size=128)
    D, sig, perf = model.evolve()
    assert perf["converged"] == 1
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), E=70e9, nu=0.33, n_correctors=5000,
                                   solution_tol=1e-10, alternative_tol=1e-11)
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S
    model.close()


def test_fp32_refine_default_tolerance_error(ctx):
    """At the same converged residual tolerance (the default 1e-6) the FP32
    inner solve with FP64 refinement matches the FP64 oracle in the same DIC
    order within the bars."""
    m, bcs = cube(12, seed=6)
    law = dict(type="linearElastic", E=70e9, nu=0.33)
    model = sg.SolidModel(ctx, m, law, bcs, outer=dict(nCorrectors=2000), precision="FP32_REFINE")
    D, sig, perf = model.evolve()
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(), E=70e9,
                                   nu=0.33, n_correctors=2000)
    assert perf["converged"] == 1 and po["converged"] == 1
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S
    model.close()


@pytest.mark.parametrize("precision,sub", [("FP64", False), ("FP32_REFINE", True)])
def test_cuda_graph_batches_are_bit_identical(precision, sub):
    """PCG batches replayed from captured CUDA graphs give the same bits as
    kernel-by-kernel launches."""
    m, bcs = cube(10, seed=8)
    law = dict(type="linearElastic", E=70e9, nu=0.33)
    out = []
    for graphs in (True, False):
        c = sg.Context(0, graphs=graphs)
        model = sg.SolidModel(c, m, law, bcs, outer=dict(nCorrectors=2000), precision=precision,
                              part_size=64, dic_subdomains=sub)
        D, sig, perf = model.evolve()
        out.append((D, sig, perf["total_lin_iters"]))
        model.close()
        c.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]
