"""GPU tests of the device features beside the plain loop, each against the
CPU oracle: field relaxation (relaxField "fixed"), a caller's decomposition
into DIC subdomains on the benchmark's cube form at 32^3, batched load cases
and served requests of the benchmark's streams, the bounded-wait timeout and
the NaN stop (failure paths that fault nothing), and the total Lagrangian
paths that only the oracle had run: the enforceLinear switch and fixed
values carried across increments (rigid rotation).

Bars, from the solve's specification: relative L2 error of D <= 1e-6 and
of sigma <= 1e-5 against the FP64 oracle at the same settings.
"""
import os

import numpy as np
import pytest

import solids4foam_gb300 as sg
from solids4foam_gb300 import _lib
from solids4foam_gb300.cases import oracle_bcs
from oracle import pyoracle
from oracle.box_mesh import block_parts, box_mesh as oracle_box_mesh

pytestmark = pytest.mark.gpu
TOL_D, TOL_S = 1e-6, 1e-5
THREADS = min(16, os.cpu_count() or 1)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_field_relaxation_linear_matches_oracle(ctx):
    """relaxationFactors { fields { D 0.7; } } on a jittered box at nu = 0.45
    under a shear traction, where the unrelaxed loop runs away: cells and
    boundary faces relaxed after each solve, as the oracle does."""
    m = sg.box_mesh(10, 10, 10, 1.0, 1.0, 1.0, 0.2, 3)
    t = np.tile([1e5, 0.0, -1e6], (int(m["patch_size"][5]), 1))
    bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", t, None)}
    # converged tightly: with relaxation the loop contracts slowly, so two
    # runs that each pass solutionTolerance 1e-6 can stand ~1e-5 apart
    outer = dict(nCorrectors=6000, fieldRelaxation=0.7, solutionTolerance=1e-10,
                 alternativeTolerance=1e-11)
    model = sg.SolidModel(ctx, m, dict(type="linearElastic", E=200e9, nu=0.45), bcs, outer=outer)
    D, sig, perf = model.evolve()
    Do, so, Go, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(), E=200e9,
                                    nu=0.45, n_correctors=6000, field_relaxation=0.7,
                                    solution_tol=1e-10, alternative_tol=1e-11, n_threads=THREADS)
    assert po["converged"] == 1 and perf["converged"] == 1
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S
    assert rel(model.gradD(), Go) < TOL_S
    # Over ~10^3 slowly converging correctors one inner solve in some
    # corrector may stop an iteration apart (round-off at the relTol
    # threshold), after which the two trajectories differ while converging
    # to the same fixed point: the counts then differ by some percent, and
    # the fields agree within the bars above (the corrector-by-corrector
    # agreement is the next test's).
    assert abs(perf["n_correctors"] - po["n_correctors"]) <= 0.15 * po["n_correctors"]
    model.close()


def test_field_relaxation_first_correctors_match_oracle(ctx):
    """The relaxation itself, corrector by corrector: after the first 25
    correctors of the same solve (before any inner solve could stop an
    iteration apart) the device and the oracle agree to round-off."""
    m = sg.box_mesh(10, 10, 10, 1.0, 1.0, 1.0, 0.2, 3)
    t = np.tile([1e5, 0.0, -1e6], (int(m["patch_size"][5]), 1))
    bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", t, None)}
    for n in (1, 2, 25):
        outer = dict(nCorrectors=n, fieldRelaxation=0.7)
        model = sg.SolidModel(ctx, m, dict(type="linearElastic", E=200e9, nu=0.45), bcs,
                              outer=outer)
        D, sig, perf = model.evolve()
        Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(), E=200e9,
                                       nu=0.45, n_correctors=n, field_relaxation=0.7)
        model.close()
        assert perf["n_correctors"] == po["n_correctors"] == n
        assert perf["total_lin_iters"] == po["total_lin_iters"]
        assert rel(D, Do) < 1e-11 and rel(sig, so) < 1e-10


def test_field_relaxation_tl_matches_oracle(ctx):
    """Field relaxation of DD in the incremental total Lagrangian model
    (neoHookean, K/mu = 10, three traction increments): the relaxed
    boundary values carry from one increment into the next."""
    m = sg.box_mesh(6, 5, 5, 1.0, 0.8, 0.8, 0.15, 12)
    t = np.tile([0.0, 5e4, -5e4], (int(m["patch_size"][5]), 1))
    bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", t, None)}
    law = dict(type="neoHookeanElastic", mu=1e6, K=1e7)
    model = sg.SolidModel(ctx, m, law, bcs, model="nonLinearGeometryTotalLagrangian",
                          outer=dict(nCorrectors=6000, fieldRelaxation=0.7,
                                     solutionTolerance=1e-9, alternativeTolerance=1e-10))
    D, sig, perf = model.evolve(n_increments=3)
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(), model=1,
                                   law=1, use_mu_K=1, mu=1e6, K=1e7, n_correctors=6000,
                                   n_increments=3, field_relaxation=0.7, solution_tol=1e-9,
                                   alternative_tol=1e-10, n_threads=THREADS)
    assert po["converged"] == 1 and perf["converged"] == 1
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S
    assert abs(perf["n_correctors"] - po["n_correctors"]) <= 0.15 * po["n_correctors"]
    model.close()


def test_aitken_relaxation_matches_oracle(ctx):
    """relaxationMethod Aitken (solidModel.C:842-896): a factor per cell and
    boundary face, the field's relaxation factor (or 1) at the first
    corrector, then adapted from the last two residuals and bounded to
    [0, 2]; D -= alpha (D.prevIter - D), fixed-value faces left as they are.
    The first correctors corrector by corrector, then whole solves: linear
    geometry (nu = 0.3, without and with a first factor) and the incremental
    total Lagrangian model over two increments."""
    m = sg.box_mesh(10, 10, 10, 1.0, 1.0, 1.0, 0.2, 3)
    t = np.tile([0.0, 1e5, -1e5], (int(m["patch_size"][5]), 1))
    bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", t, None)}
    law = dict(type="linearElastic", E=200e9, nu=0.3)
    for n in (1, 2, 6):
        model = sg.SolidModel(ctx, m, law, bcs, outer=dict(nCorrectors=n, relaxationMethod="Aitken"))
        D, sig, perf = model.evolve()
        Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(), E=200e9,
                                       nu=0.3, n_correctors=n, relaxation_method=1)
        model.close()
        assert perf["n_correctors"] == po["n_correctors"] == n
        assert perf["total_lin_iters"] == po["total_lin_iters"]
        assert rel(D, Do) < 1e-11 and rel(sig, so) < 1e-10
    for fr in (1.0, 0.7):
        outer = dict(nCorrectors=4000, relaxationMethod="Aitken", fieldRelaxation=fr,
                     solutionTolerance=1e-10, alternativeTolerance=1e-10)
        model = sg.SolidModel(ctx, m, law, bcs, outer=outer)
        D, sig, perf = model.evolve()
        Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(), E=200e9,
                                       nu=0.3, n_correctors=4000, relaxation_method=1,
                                       field_relaxation=fr, solution_tol=1e-10,
                                       alternative_tol=1e-10, n_threads=THREADS)
        model.close()
        assert po["converged"] == 1 and perf["converged"] == 1
        assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S
    mt = sg.box_mesh(6, 5, 5, 1.0, 0.8, 0.8, 0.15, 12)
    tt = np.tile([0.0, 5e4, -5e4], (int(mt["patch_size"][5]), 1))
    bt = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", tt, None)}
    model = sg.SolidModel(ctx, mt, dict(type="neoHookeanElastic", mu=1e6, K=5e6), bt,
                          model="nonLinearGeometryTotalLagrangian",
                          outer=dict(nCorrectors=6000, relaxationMethod="Aitken",
                                     solutionTolerance=1e-9, alternativeTolerance=1e-10))
    D, sig, perf = model.evolve(n_increments=2)
    Do, so, _, po = pyoracle.solve(mt, oracle_bcs(mt, bt), perm=model.permutation(), model=1,
                                   law=1, use_mu_K=1, mu=1e6, K=5e6, n_correctors=6000,
                                   n_increments=2, relaxation_method=1, solution_tol=1e-9,
                                   alternative_tol=1e-10, n_threads=THREADS)
    model.close()
    assert po["converged"] == 1 and perf["converged"] == 1
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S


def cube32_case():
    """The benchmark's cube form at 32^3: unit cube, interior vertices
    jittered +-0.2 h (seed 1), E = 70 GPa, nu = 0.33, bottom fixed, top
    pressure 10 MPa; the oracle builds the same mesh with its own generator."""
    m = oracle_box_mesh(32, 32, 32, 1.0, 1.0, 1.0, 0.2, 1)
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", None, np.full(int(m["patch_size"][5]), 10e6))}
    return m, bcs


@pytest.mark.parametrize("precision", ["FP64", "FP32_REFINE"])
def test_caller_blocks_cube32_match_oracle(ctx, precision):
    """The benchmark's decomposition -- 8^3-cell blocks given by the caller
    (part_of_cell), each block's DIC in the caller's cell order -- on the
    32^3 cube, against the oracle with the same subdomains (dic_domain) and
    the mesh from the oracle's own generator.  Plain FP64 takes the
    oracle's iteration counts; FP32 + refinement stays within the bars."""
    m, bcs = cube32_case()
    parts = block_parts(32, 32, 32, 8)
    model = sg.SolidModel(ctx, m, dict(type="linearElastic", E=70e9, nu=0.33), bcs,
                          outer=dict(nCorrectors=2000), precision=precision, parts=parts)
    D, sig, perf = model.evolve()
    assert np.array_equal(model.parts(), parts)
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), dic_domain=parts, E=70e9, nu=0.33,
                                   n_correctors=2000, n_threads=THREADS)
    model.close()
    assert po["converged"] == 1 and perf["converged"] == 1
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S
    if precision == "FP64":
        assert abs(perf["n_correctors"] - po["n_correctors"]) <= 1
        assert abs(perf["total_lin_iters"] - po["total_lin_iters"]) <= 0.005 * po["total_lin_iters"]


def test_library_parts_cube32_match_oracle(ctx):
    """The library's own decomposition (coordinate-bisection parts, BFS
    order inside) on the 32^3 cube in plain FP64, against the oracle run in
    the library's DIC order with the same subdomains."""
    m, bcs = cube32_case()
    # both sides converge to 1e-8: the dot products are summed in another
    # order, so solves that each pass 1e-6 can stop ~1e-6 apart
    model = sg.SolidModel(ctx, m, dict(type="linearElastic", E=70e9, nu=0.33), bcs,
                          outer=dict(nCorrectors=4000, solutionTolerance=1e-8,
                                     alternativeTolerance=1e-8), dic_subdomains=True)
    D, sig, perf = model.evolve()
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(),
                                   dic_domain=model.parts(), E=70e9, nu=0.33,
                                   n_correctors=4000, solution_tol=1e-8, alternative_tol=1e-8,
                                   n_threads=THREADS)
    model.close()
    assert po["converged"] == 1 and perf["converged"] == 1
    # the same preconditioner; the dot products are summed in another order,
    # so an inner solve may stop an iteration apart and the trajectories part
    assert abs(perf["n_correctors"] - po["n_correctors"]) <= 0.01 * po["n_correctors"]
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S


def test_load_cases_match_oracle(ctx):
    """Batched load cases of the 64^3 benchmark form at 24^3 (E = 200 GPa,
    nu = 0.3, top tractions N(0, 1 MPa) per component), FP32 + refinement
    over 8^3 caller blocks: every case against its own oracle solve."""
    n = 24
    m = oracle_box_mesh(n, n, n, 1.0, 1.0, 1.0, 0.2, 2)
    parts = block_parts(n, n, n, 8)
    tr = np.random.default_rng(3).normal(0.0, 1e6, (4, 3))
    cases = [{"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", tr[c], None)}
             for c in range(4)]
    # both sides converge to 1e-8 so that where each stops stays well inside
    # the bars (solves that each pass 1e-6 can stand ~1e-6 apart)
    model = sg.SolidModel(ctx, m, dict(type="linearElastic", E=200e9, nu=0.3), cases[0],
                          outer=dict(nCorrectors=4000, solutionTolerance=1e-8,
                                     alternativeTolerance=1e-8),
                          precision="FP32_REFINE", parts=parts)
    Db, sb, perfs = model.evolve_cases(cases)
    model.close()
    top = int(m["patch_size"][5])
    for c in range(4):
        bo = [(1, None, None)] * 4 + [(0, None, None), (1, np.tile(tr[c], (top, 1)), None)]
        Do, so, _, po = pyoracle.solve(m, bo, dic_domain=parts, E=200e9, nu=0.3, n_correctors=4000,
                                       solution_tol=1e-8, alternative_tol=1e-8, n_threads=THREADS)
        assert po["converged"] == 1 and perfs[c]["converged"] == 1
        assert rel(Db[c], Do) < TOL_D and rel(sb[c], so) < TOL_S


def test_served_requests_match_oracle():
    """Requests of the served stream's kinds through the server at once --
    linear at nu = 0.45 with field relaxation 0.7, and neoHookean total
    Lagrangian with field relaxation over traction increments -- each
    against its oracle solve (8^3 caller blocks, FP32 + refinement)."""
    reqs = []
    for i, (n, kind) in enumerate([(10, "lin"), (14, "lin"), (6, "tl"), (9, "lin")]):
        m = oracle_box_mesh(n, n, n, 1.0, 1.0, 1.0, 0.2, 40 + i)
        top = int(m["patch_size"][5])
        parts = block_parts(n, n, n, 8)
        if kind == "lin":
            t = np.array([2e5, -1e5, -1e6])
            kw = dict(law=dict(type="linearElastic", E=100e9, nu=0.45),
                      outer=dict(nCorrectors=8000, fieldRelaxation=0.7, solutionTolerance=1e-8,
                                 alternativeTolerance=1e-9))
            okw = dict(E=100e9, nu=0.45, field_relaxation=0.7, n_correctors=8000,
                       solution_tol=1e-8, alternative_tol=1e-9)
            ninc = 1
        else:
            t = np.array([0.0, 5e4, -5e4])
            kw = dict(law=dict(type="neoHookeanElastic", mu=1e6, K=1e7),
                      model="nonLinearGeometryTotalLagrangian", n_increments=3,
                      outer=dict(nCorrectors=6000, fieldRelaxation=0.7, solutionTolerance=1e-8,
                                 alternativeTolerance=1e-9))
            okw = dict(model=1, law=1, use_mu_K=1, mu=1e6, K=1e7, n_increments=3,
                       field_relaxation=0.7, n_correctors=6000, solution_tol=1e-8,
                       alternative_tol=1e-9)
            ninc = 3
        bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", t, None)}
        reqs.append((m, bcs, parts, kw, okw, ninc))
    srv = sg.Server(max_slots=4)
    ids = [srv.submit(m, bcs=bcs, precision="FP32_REFINE", parts=parts, **kw)
           for m, bcs, parts, kw, _, _ in reqs]
    res = [srv.result(i) for i in ids]
    srv.close()
    for (m, bcs, parts, kw, okw, ninc), (st, D, sig, perf) in zip(reqs, res):
        assert st == _lib.OK and perf["converged"] == 1
        Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), dic_domain=parts, n_threads=THREADS,
                                       **okw)
        assert po["converged"] == 1
        assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S


def test_bounded_wait_times_out_and_the_context_stays_usable():
    """A bounded device wait that runs out ends the call with S4G_TIMEOUT
    and leaves the context usable.  The exact DIC's sweeps wait for the
    parts they depend on; with a limit of one poll those waits give up (the
    kernel records it, skips the wait and returns -- nothing hangs), and a
    solve on the same context afterwards is clean."""
    c = sg.Context(0, spin_limit=1)
    m = sg.box_mesh(16, 16, 16, 1.0, 1.0, 1.0, 0.2, 4)
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", None, np.full(256, 1e6))}
    law = dict(type="linearElastic", E=70e9, nu=0.33)
    model = sg.SolidModel(c, m, law, bcs, part_size=64)
    with pytest.raises(sg.S4GError) as e:
        model.evolve()
    assert e.value.status == _lib.TIMEOUT
    model.close()
    # the processor-local DIC has no waits: a clean solve on the same context
    model = sg.SolidModel(c, m, law, bcs, dic_subdomains=True, part_size=64)
    D, sig, perf = model.evolve()
    assert perf["converged"] == 1 and perf["device_status"] == 0 and np.isfinite(D).all()
    model.close()
    c.close()


def test_non_finite_field_is_detected_on_the_device(ctx):
    """A neoHookean total-displacement solve that blows up (K/mu = 10, ten
    traction increments, no relaxation -- the oracle stops on NaN too)
    ends with S4G_NAN_DETECTED, and the context solves cleanly afterwards."""
    m = sg.box_mesh(8, 8, 8, 1.0, 1.0, 1.0, 0.2, 5)
    t = np.tile(np.random.default_rng(5).normal(0, 1e5, 3), (int(m["patch_size"][5]), 1))
    bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", t, None)}
    _, _, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), model=2, law=1, use_mu_K=1, mu=1e6,
                                 K=1e7, n_correctors=3000, n_increments=10)
    assert po["nan_detected"] == 1
    model = sg.SolidModel(ctx, m, dict(type="neoHookeanElastic", mu=1e6, K=1e7), bcs,
                          model="nonLinearGeometryTotalLagrangianTotalDisplacement",
                          outer=dict(nCorrectors=3000))
    with pytest.raises(sg.S4GError) as e:
        model.evolve(n_increments=10)
    assert e.value.status == _lib.NAN_DETECTED
    model.close()
    bcs2 = {"zmin": ("fixedDisplacement", None, None),
            "zmax": ("solidTraction", None, np.full(64, 1e6))}
    model = sg.SolidModel(ctx, m, dict(type="linearElastic", E=70e9, nu=0.33), bcs2)
    D, sig, perf = model.evolve()
    assert perf["converged"] == 1 and np.isfinite(D).all()
    model.close()


def test_enforce_linear_switch_matches_oracle(ctx):
    """checkEnforceLinear (nonLinGeomTotalLagSolid.C:203-207 via
    solidModel.C:1894-1913): a box crushed to half its height in one
    increment takes J below 0.01 somewhere, so linear geometry is enforced
    for the rest of the increment, on the device as in the oracle."""
    m = sg.box_mesh(6, 5, 5, 1.0, 0.8, 0.8, 0.15, 12)
    z = np.tile([0.0, 0.0, -0.5], (int(m["patch_size"][5]), 1))
    bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("fixedDisplacement", z, None)}
    law = dict(type="neoHookeanElastic", mu=1e6, K=1e7)
    model = sg.SolidModel(ctx, m, law, bcs, model="nonLinearGeometryTotalLagrangian",
                          outer=dict(nCorrectors=1000))
    D, sig, perf = model.evolve(n_increments=1)
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(), model=1,
                                   law=1, use_mu_K=1, mu=1e6, K=1e7, n_correctors=1000)
    model.close()
    assert po["enforce_linear"] == 1 and perf["enforce_linear"] == 1
    assert po["converged"] == 1 and perf["converged"] == 1
    assert abs(perf["n_correctors"] - po["n_correctors"]) <= 1
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S


@pytest.mark.parametrize("model_name,model_id", [("nonLinearGeometryTotalLagrangian", 1),
                                                 ("nonLinearGeometryTotalLagrangianTotalDisplacement", 2)])
def test_rigid_rotation_matches_oracle(ctx, model_name, model_id):
    """A rigid rotation of 90 degrees about z prescribed on every boundary
    over 45 increments: the incremental form carries nonzero fixed values
    from one increment into the next (D.oldTime on the boundary).  The
    device recovers D = (R - I) C stress-free, as the oracle does."""
    m = sg.box_mesh(6, 5, 4, 1.0, 0.9, 0.8, 0.2, 3)
    th = np.radians(90.0)
    R = np.array([[np.cos(th), -np.sin(th), 0.0], [np.sin(th), np.cos(th), 0.0], [0.0, 0.0, 1.0]])
    names = ["xmin", "xmax", "ymin", "ymax", "zmin", "zmax"]
    bcs = {}
    for p in range(6):
        s, n = int(m["patch_start"][p]), int(m["patch_size"][p])
        bcs[names[p]] = ("fixedDisplacement", m["Cf"][s:s + n] @ (R - np.eye(3)).T, None)
    law = dict(type="neoHookeanElastic", mu=1e6, K=5e6)
    outer = dict(nCorrectors=4000, solutionTolerance=1e-10, alternativeTolerance=1e-11)
    model = sg.SolidModel(ctx, m, law, bcs, model=model_name, outer=outer, ls_boundary_delta=1)
    D, sig, perf = model.evolve(n_increments=45)
    Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, bcs), perm=model.permutation(), model=model_id,
                                   law=1, use_mu_K=1, mu=1e6, K=5e6, n_correctors=4000,
                                   n_increments=45, solution_tol=1e-10, alternative_tol=1e-11,
                                   ls_boundary_delta=1)
    model.close()
    assert po["converged"] == 1 and perf["converged"] == 1 and perf["enforce_linear"] == 0
    exact = m["C"] @ (R - np.eye(3)).T
    assert np.abs(D - exact).max() < 1e-7 * np.abs(exact).max()
    assert np.abs(sig).max() < 1.0                    # below 1e-6 mu
    assert rel(D, Do) < TOL_D


@pytest.mark.parametrize("kind", ["tl", "cases", "exact"])
def test_device_loop_is_bit_identical_to_the_host_loop(kind):
    """The device-resident corrector loop (one CUDA graph whose conditional
    WHILE nodes run the correctors and the PCG iterations, decided on the
    device) computes exactly what the host-driven loop computes: same bits,
    same corrector and iteration counts.  Total Lagrangian increments,
    batched load cases and the exact DIC's sweeps."""
    m = sg.box_mesh(10, 9, 8, 1.0, 0.9, 0.8, 0.2, 6)
    top = int(m["patch_size"][5])
    out = []
    for graphs in (True, False):
        c = sg.Context(0, graphs=graphs)
        if kind == "tl":
            bcs = {"zmin": ("fixedDisplacement", None, None),
                   "zmax": ("solidTraction", np.tile([0.0, 5e4, -5e4], (top, 1)), None, 0.5)}
            model = sg.SolidModel(c, m, dict(type="neoHookeanElastic", mu=1e6, K=1e7), bcs,
                                  model="nonLinearGeometryTotalLagrangian",
                                  outer=dict(nCorrectors=3000, fieldRelaxation=0.7),
                                  precision="FP32_REFINE", parts=block_parts(10, 9, 8, 4))
            D, sig, perf = model.evolve(n_increments=3)
            res = [(D, sig, perf)]
        elif kind == "cases":
            tr = np.random.default_rng(9).normal(0.0, 1e6, (3, 3))
            cases = [{"zmin": ("fixedDisplacement", None, None),
                      "zmax": ("solidTraction", tr[k], None)} for k in range(3)]
            model = sg.SolidModel(c, m, dict(type="linearElastic", E=200e9, nu=0.3), cases[0],
                                  precision="FP32_REFINE", parts=block_parts(10, 9, 8, 4))
            Db, sb, perfs = model.evolve_cases(cases)
            res = [(Db[k], sb[k], perfs[k]) for k in range(3)]
        else:
            bcs = {"zmin": ("fixedDisplacement", None, None),
                   "zmax": ("solidTraction", None, np.full(top, 1e6))}
            model = sg.SolidModel(c, m, dict(type="linearElastic", E=70e9, nu=0.33), bcs,
                                  part_size=64)
            D, sig, perf = model.evolve()
            res = [(D, sig, perf)]
        model.close()
        c.close()
        out.append(res)
    for (D1, s1, p1), (D2, s2, p2) in zip(out[0], out[1]):
        assert p1["device_loop"] == 1 and p2["device_loop"] == 0
        assert p1["converged"] == 1
        assert np.array_equal(D1, D2) and np.array_equal(s1, s2)
        assert p1["n_correctors"] == p2["n_correctors"]
        assert p1["total_lin_iters"] == p2["total_lin_iters"]


@pytest.mark.parametrize("model_name", ["linearGeometryTotalDisplacement",
                                        "nonLinearGeometryTotalLagrangian"])
def test_point_interpolation_on_the_device_equals_the_host_step(ctx, model_name):
    """pointD after the loop on the device (s4g_get_pointD), from the D and
    gradD the solve left in device memory, equals the host step
    s4g_point_interpolate on the same fields bit for bit."""
    from solids4foam_gb300.foam_case import box_polymesh
    from solids4foam_gb300.post import point_cells, point_displacement
    m = box_polymesh(9, 7, 6, 1.0, 0.8, 0.7, 0.2, 13)
    top = int(m["patch_size"][5])
    if model_name == "linearGeometryTotalDisplacement":
        law, n_inc = dict(type="linearElastic", E=70e9, nu=0.33), 1
        bcs = {"zmin": ("fixedDisplacement", None, None),
               "zmax": ("solidTraction", np.tile([1e5, 0.0, -1e6], (top, 1)), None)}
    else:
        law, n_inc = dict(type="neoHookeanElastic", mu=1e6, K=1e7), 2
        bcs = {"zmin": ("fixedDisplacement", None, None),
               "zmax": ("solidTraction", np.tile([0.0, 2e4, -2e4], (top, 1)), None, 0.5)}
    model = sg.SolidModel(ctx, m, law, bcs, model=model_name, outer=dict(nCorrectors=3000))
    D, sig, perf = model.evolve(n_increments=n_inc)
    pc = point_cells(m)
    model.set_points(m["points"], *pc)
    pd = model.point_displacement_device()
    ph = point_displacement(m, D, model.gradD(), pc)
    model.close()
    assert perf["converged"] == 1
    assert np.array_equal(pd, ph)
    assert np.abs(pd).max() > 0


@pytest.mark.parametrize("model_name", ["nonLinearGeometryTotalLagrangian",
                                        "nonLinearGeometryTotalLagrangianTotalDisplacement"])
def test_time_steps_equal_load_increments(ctx, model_name):
    """s4g_solve_step: three time steps whose traction is (n/3) b equal
    s4g_solve with three load increments bit for bit -- the same products
    n/3 times b, and the old-time fields carried from step to step on the
    device -- and the steps' corrector counts add up to the solve's."""
    m = sg.box_mesh(6, 5, 5, 1.0, 0.8, 0.8, 0.15, 12)
    b = np.tile([0.0, 5e4, -5e4], (int(m["patch_size"][5]), 1))
    bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", b, None)}
    model = sg.SolidModel(ctx, m, dict(type="neoHookeanElastic", mu=1e6, K=5e6), bcs,
                          model=model_name,
                          outer=dict(nCorrectors=6000, solutionTolerance=1e-8,
                                     alternativeTolerance=1e-9))
    D, sig, perf = model.evolve(n_increments=3)
    n_corr = 0
    for n in (1, 2, 3):
        Ds, ss, ps = model.step({"zmax": ("solidTraction", b * (n / 3), None)})
        assert ps["converged"] == 1
        n_corr += ps["n_correctors"]
    model.close()
    assert np.array_equal(Ds, D) and np.array_equal(ss, sig)
    assert n_corr == perf["n_correctors"]


def test_linear_time_steps_continue_from_the_last_step(ctx):
    """Linear geometry in time steps: the first step is s4g_solve bit for
    bit; the next starts from the last step's D (its D.oldTime) and, the
    problem being steady, ends at the solution for its own load; after
    reset_state a step starts from zero again, as a fresh solve does."""
    m = sg.box_mesh(10, 8, 6, 2.0, 0.8, 0.6, 0.2, 5)
    t1 = [0.0, -1e5, 2e4]
    bcs = {"xmin": ("fixedDisplacement", None, None), "xmax": ("solidTraction", t1, None)}
    law = dict(type="linearElastic", E=70e9, nu=0.3)
    outer = dict(nCorrectors=5000, solutionTolerance=1e-10, alternativeTolerance=1e-10)
    model = sg.SolidModel(ctx, m, law, bcs, outer=outer)
    D1, s1, p1 = model.evolve()
    Ds1, ss1, ps1 = model.step()
    assert np.array_equal(Ds1, D1) and np.array_equal(ss1, s1)
    assert ps1["n_correctors"] == p1["n_correctors"]
    t2 = [3e4, -2e5, 0.0]
    Ds2, ss2, ps2 = model.step({"xmax": ("solidTraction", t2, None)})
    fresh = sg.SolidModel(ctx, m, law, {"xmin": ("fixedDisplacement", None, None),
                                        "xmax": ("solidTraction", t2, None)}, outer=outer)
    D2, s2, p2 = fresh.evolve()
    fresh.close()
    assert ps2["converged"] == 1 and p2["converged"] == 1
    # two slowly contracting loops that each pass 1e-10 stand ~1e-8 apart
    assert rel(Ds2, D2) < 1e-7 and rel(ss2, s2) < 1e-6
    model.reset_state()
    Ds3, ss3, _ = model.step()
    model.close()
    assert np.array_equal(Ds3, D2) and np.array_equal(ss3, s2)


def test_case_load_table_runs_time_steps(ctx, tmp_path):
    """A meshed case whose traction is a table that loads and unloads
    (tractionSeries, not a ramp from zero) is stepped through its
    controlDict time steps (load_case time_steps, run_time_steps: one
    s4g_solve_step each, the series evaluated at the step's time).  The
    linear model being steady, each step ends at the solution for its own
    load: the last step against a fresh solve at the load of endTime."""
    from solids4foam_gb300.foam_case import box_polymesh, load_case, write_box_case
    write_box_case(str(tmp_path / "constant" / "polyMesh"),
                   box_polymesh(8, 6, 6, 1.0, 0.8, 0.8, 0.2, 7))
    (tmp_path / "constant" / "timeVsTraction").write_text(
        "((0 (0 0 0)) (5 (2e4 0 -1e5)) (10 (4e3 0 -2e4)))")
    (tmp_path / "system").mkdir()
    (tmp_path / "system" / "controlDict").write_text(
        "FoamFile { version 2.0; format ascii; class dictionary; object controlDict; }\n"
        "startTime 0;\nendTime 10;\ndeltaT 2.5;\n")
    (tmp_path / "0").mkdir()
    free = "{ type solidTraction; traction uniform (0 0 0); pressure uniform 0; }"
    (tmp_path / "0" / "D").write_text(
        "FoamFile { version 2.0; format ascii; class volVectorField; object D; }\n"
        "boundaryField {\n"
        f"  xmin {free} xmax {free} ymin {free} ymax {free}\n"
        "  zmin { type fixedDisplacement; value uniform (0 0 0); }\n"
        "  zmax { type solidTraction; pressure uniform 0;\n"
        "         tractionSeries { file \"$FOAM_CASE/constant/timeVsTraction\"; } }\n"
        "}\n")
    head = "FoamFile { version 2.0; format ascii; class dictionary; object x; }\n"
    (tmp_path / "constant" / "solidProperties").write_text(
        head + "solidModel linearGeometryTotalDisplacement;\n"
        "linearGeometryTotalDisplacementCoeffs { nCorrectors 5000; solutionTolerance 1e-10; "
        "alternativeTolerance 1e-10; }\n")
    (tmp_path / "constant" / "mechanicalProperties").write_text(
        head + "planeStress no;\nmechanical ( steel { type linearElastic; rho rho [1 -3 0 0 0 0 0] 1000; "
        "E E [1 -1 -2 0 0 0 0] 200e9; nu nu [0 0 0 0 0 0 0] 0.3; } );\n")
    (tmp_path / "system" / "fvSolution").write_text(
        head + "solvers { D { solver PCG; preconditioner DIC; tolerance 1e-09; relTol 0.1; } }\n")
    c = load_case(str(tmp_path))
    assert c["model"] == "linearGeometryTotalDisplacement"
    assert [t for t, _ in c["time_steps"]] == [2.5, 5.0, 7.5, 10.0]
    outer = dict(nCorrectors=5000, solutionTolerance=1e-10, alternativeTolerance=1e-10)
    law = dict(type="linearElastic", E=200e9, nu=0.3)
    model = sg.SolidModel(ctx, c["mesh"], law, c["bcs"], outer=outer)
    D, sig, perfs = model.run_time_steps(c["time_steps"])
    model.close()
    assert len(perfs) == 4 and all(p["converged"] == 1 for p in perfs)
    end = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", [4e3, 0.0, -2e4], None)}
    fresh = sg.SolidModel(ctx, c["mesh"], law, end, outer=outer)
    Df, sf, pf = fresh.evolve()
    fresh.close()
    # the step starts next to its answer, so its convergence tests (relative
    # to the step's change) stop it elsewhere within the outer tolerance
    assert rel(D, Df) < TOL_D and rel(sig, sf) < TOL_S
