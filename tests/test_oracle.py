"""CPU tests of the FP64 oracle: the reference's known answers and the
properties its discretisation must have (no GPU needed)."""
import json
import os

import numpy as np
import pytest

from oracle import pyoracle
import solids4foam_gb300 as sg
from solids4foam_gb300.cases import oracle_bcs

from cases2d import cooks_membrane

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def patch():
    with open(os.path.join(HERE, "golden", "patch_test.json")) as f:
        return json.load(f)


def _linear_field(p, X):
    a = np.asarray(p["a"])
    b = np.asarray(p["b"])
    return a + X @ b.T


def _patch_bcs(mesh, p):
    bcs = []
    for k in range(6):
        s, n = int(mesh["patch_start"][k]), int(mesh["patch_size"][k])
        bcs.append((0, _linear_field(p, mesh["Cf"][s:s + n]), None))
    return bcs


def _strain(G):
    G = G.reshape(-1, 3, 3)
    return 0.5 * (G + G.transpose(0, 2, 1))


@pytest.mark.parametrize("jitter,lsdelta", [(0.0, 0), (0.25, 1)])
def test_patch_test_constant_strain(patch, jitter, lsdelta):
    """patchTest: a linear displacement on every boundary gives the constant
    strain of the reference's README (exx 2e-6, eyy 6e-6, exy 4e-6), to
    round-off, on a distorted mesh once the least-squares boundary vectors
    are consistent (full Cf - C), and on an orthogonal mesh with either."""
    m = sg.box_mesh(6, 5, 4, 1.0, 0.9, 0.8, jitter, 3)
    D, sig, G, perf = pyoracle.solve(m, _patch_bcs(m, patch), E=patch["E"], nu=patch["nu"],
                                     n_correctors=400, solution_tol=1e-13,
                                     alternative_tol=1e-14, tolerance=1e-15, rel_tol=0.0,
                                     ls_boundary_delta=lsdelta)
    eps = _strain(G)
    exp = patch["expected_strain"]
    for (i, j), key in {(0, 0): "xx", (1, 1): "yy", (0, 1): "xy", (2, 2): "zz"}.items():
        np.testing.assert_allclose(eps[:, i, j], exp[key], atol=1e-15, rtol=1e-8)
    np.testing.assert_allclose(D, _linear_field(patch, m["C"]), atol=1e-15, rtol=1e-8)
    # stresses constant too
    assert np.ptp(sig, axis=0).max() < 1e-6 * np.abs(sig).max()


def test_patch_test_normal_delta_distorted_is_close(patch):
    """With OpenFOAM.com/.org patch-normal boundary deltas the leastSquares
    gradient is not exact next to distorted boundaries (the reference README
    warns about this); the error stays small."""
    m = sg.box_mesh(6, 5, 4, 1.0, 0.9, 0.8, 0.25, 3)
    D, sig, G, perf = pyoracle.solve(m, _patch_bcs(m, patch), E=patch["E"], nu=patch["nu"],
                                     n_correctors=300, solution_tol=1e-12,
                                     alternative_tol=1e-13, tolerance=1e-15, rel_tol=0.0)
    eps = _strain(G)
    assert abs(eps[:, 0, 0].mean() - 2e-6) < 0.05 * 2e-6


def test_matrix_symmetric_positive(patch):
    m = sg.box_mesh(5, 4, 3, 1.0, 1.0, 1.0, 0.2, 5)
    bcs = [(0, None, None)] + [(1, None, None)] * 5
    diag, upper = pyoracle.matrix(m, bcs, 1.0)
    n = diag.shape[0]
    A = np.diag(diag)
    own, nei = m["owner"][:upper.shape[0]], m["neighbour"]
    A[own, nei] = upper
    A[nei, own] = upper
    assert np.allclose(A, A.T)
    assert np.linalg.eigvalsh(A).min() > 0
    # rows of cells away from fixed patches sum to zero (negSumDiag)
    fixed_cells = set(m["owner"][m["patch_start"][0]:m["patch_start"][0] + m["patch_size"][0]])
    interior = [c for c in range(n) if c not in fixed_cells]
    assert np.abs(A[interior].sum(1)).max() < 1e-12 * diag.max()
    # DIC is the exact solve for a 1-row system and a contraction otherwise
    x = np.random.default_rng(1).standard_normal(n)
    w = pyoracle.dic(m, diag, upper, A @ x)
    assert np.linalg.norm(w - x) < np.linalg.norm(x)


def test_renumbered_oracle_equals_permuted_mesh():
    """Running with perm equals running on the renumbered mesh, bit for bit."""
    m = sg.box_mesh(5, 4, 4, 1.0, 1.0, 1.0, 0.2, 9)
    bcs = oracle_bcs(m, {"zmin": ("fixedDisplacement", None, None),
                         "zmax": ("solidTraction", None, np.full(int(m["patch_size"][5]), 1e6))})
    perm = np.random.default_rng(0).permutation(m["V"].shape[0]).astype(np.int32)
    D1, s1, _, p1 = pyoracle.solve(m, bcs, perm=perm, E=70e9, nu=0.33, n_correctors=30)
    mr = pyoracle.renumber_mesh(m, perm)
    D2, s2, _, p2 = pyoracle.solve(mr, bcs, E=70e9, nu=0.33, n_correctors=30)
    assert np.array_equal(D1[perm], D2)
    assert np.array_equal(s1[perm], s2)


def test_cantilever_tip_deflection_trend():
    """Tip deflection of a cantilever under end shear approaches the
    Euler-Bernoulli + Timoshenko estimate as the mesh is refined
    (cantileverAnalyticalSolution is the reference's own check)."""
    E, nu, L, h, P = 200e9, 0.3, 2.0, 0.2, 1e6 * 0.2 * 0.2
    I = h ** 4 / 12
    G = E / (2 * (1 + nu))
    exact = P * L ** 3 / (3 * E * I) + P * L / (5.0 / 6.0 * G * h * h)
    tips = []
    for nx, ny in ((20, 2), (40, 4)):
        m = sg.box_mesh(nx, ny, ny, L, h, h, 0.0, 1)
        ps = m["patch_size"]
        bcs = [(0, None, None), (1, np.tile([0, -1e6, 0], (int(ps[1]), 1)), None)] + [(1, None, None)] * 4
        D, _, _, perf = pyoracle.solve(m, bcs, E=E, nu=nu, n_correctors=30000,
                                       solution_tol=1e-6)
        tips.append(-D[np.argmax(m["C"][:, 0] - 1e-9 * m["C"][:, 1]), 1])
    assert abs(tips[1] - exact) < abs(tips[0] - exact)
    assert abs(tips[1] - exact) / exact < 0.15


def test_fixed_point_residual_small():
    """At convergence D_new = D_old, so fvm and fvc laplacians cancel and
    the correction of one more corrector is tiny."""
    m = sg.box_mesh(6, 6, 6, 1.0, 1.0, 1.0, 0.2, 4)
    bcs = oracle_bcs(m, {"zmin": ("fixedDisplacement", None, None),
                         "zmax": ("solidTraction", None, np.full(int(m["patch_size"][5]), 1e7))})
    D1, _, _, p1 = pyoracle.solve(m, bcs, E=70e9, nu=0.33, n_correctors=5000,
                                  solution_tol=1e-10, alternative_tol=1e-11)
    assert p1["converged"] == 1
    D2, _, _, _ = pyoracle.solve(m, bcs, E=70e9, nu=0.33, n_correctors=p1["n_correctors"] + 5,
                                 solution_tol=0, alternative_tol=0)
    assert np.linalg.norm(D2 - D1) / np.linalg.norm(D1) < 1e-8


def test_oracle_regression_fixture():
    """The oracle still reproduces its committed outputs."""
    g = np.load(os.path.join(HERE, "golden", "oracle_small.npz"))
    m = sg.box_mesh(6, 5, 4, 1.2, 1.0, 0.8, 0.2, 11)
    ps = m["patch_size"]
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", np.tile([1e5, 0.0, -2e5], (int(ps[5]), 1)),
                    np.full(int(ps[5]), 3e5))}
    D, sig, G, perf = pyoracle.solve(m, oracle_bcs(m, bcs), E=70e9, nu=0.33, n_correctors=50)
    np.testing.assert_allclose(D, g["lin_D"], rtol=1e-12, atol=1e-22)
    np.testing.assert_allclose(sig, g["lin_sigma"], rtol=1e-10, atol=1e-6)
    assert perf["total_lin_iters"] == int(g["lin_iters"])


def test_tl_small_strain_matches_linear():
    """Total Lagrangian neo-Hookean under a tiny load reduces to linear
    elasticity with the same mu, K."""
    m = sg.box_mesh(5, 4, 4, 1.0, 0.8, 0.8, 0.15, 12)
    ps = m["patch_size"]
    t = np.tile([0.0, 1e2, 0.0], (int(ps[5]), 1))
    bcs = [(1, None, None)] * 4 + [(0, None, None), (1, t, None)]
    mu, K = 1e6, 2e7
    E = 9 * K * mu / (3 * K + mu)
    nu = (3 * K - 2 * mu) / (2 * (3 * K + mu))
    Dl, _, _, _ = pyoracle.solve(m, bcs, E=E, nu=nu, n_correctors=3000, solution_tol=1e-10,
                                 alternative_tol=1e-11)
    Dn, _, _, _ = pyoracle.solve(m, bcs, model=1, law=1, use_mu_K=1, mu=mu, K=K,
                                 n_correctors=3000, solution_tol=1e-10, alternative_tol=1e-11)
    assert np.linalg.norm(Dn - Dl) / np.linalg.norm(Dl) < 1e-3


def test_traction_relaxation_keeps_the_fixed_point():
    """solidTraction relaxationFactor (solidTractionFvPatchVectorField.C:387-392)
    changes the path of the corrector loop, not where it ends."""
    m = sg.box_mesh(8, 8, 8, 1.0, 1.0, 1.0, 0.2, 3)
    t = np.tile([1e5, 0.0, -1e6], (int(m["patch_size"][5]), 1))
    out = {}
    for rf in (1.0, 0.5):
        bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", t, None, rf)}
        D, _, _, p = pyoracle.solve(m, oracle_bcs(m, bcs), E=200e9, nu=0.3, n_correctors=4000,
                                    solution_tol=1e-10, alternative_tol=1e-11)
        assert p["converged"] == 1
        out[rf] = (D, p["n_correctors"])
    assert out[0.5][1] > out[1.0][1]
    assert np.linalg.norm(out[0.5][0] - out[1.0][0]) / np.linalg.norm(out[1.0][0]) < 1e-6


def test_tl_traction_increments_need_relaxation():
    """Total Lagrangian neo-Hookean, traction load over two increments: with
    the reference's default relaxationFactor 1 the traction-gradient update
    does not settle after the first increment; with 0.5 it converges, and
    (RhieChow off, so the discrete equations do not depend on the split)
    ends at the one-increment answer."""
    m = sg.box_mesh(6, 5, 5, 1.0, 0.8, 0.8, 0.0, 12)
    t = np.tile([0.0, 2e3, 0.0], (int(m["patch_size"][5]), 1))
    kw = dict(model=1, law=1, use_mu_K=1, mu=1e6, K=2e7, n_correctors=8000, stab_scale=0.0,
              solution_tol=1e-9, alternative_tol=1e-10)

    def run(rf, n_increments):
        bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", t, None, rf)}
        D, _, _, p = pyoracle.solve(m, oracle_bcs(m, bcs), n_increments=n_increments, **kw)
        return D, p

    D1, p1 = run(1.0, 1)
    assert p1["converged"] == 1
    _, pd = run(1.0, 2)
    assert pd["converged"] == 0
    D2, p2 = run(0.5, 2)
    assert p2["converged"] == 1
    assert np.linalg.norm(D2 - D1) / np.linalg.norm(D1) < 1e-5


def _tl_box():
    m = sg.box_mesh(6, 5, 5, 1.0, 0.8, 0.8, 0.15, 12)
    t = np.tile([0.0, 2e4, 0.0], (int(m["patch_size"][5]), 1))
    bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", t, None)}
    return m, oracle_bcs(m, bcs)


def test_tl_total_one_increment_equals_incremental():
    """With one increment (D.oldTime = 0) the total form
    (nonLinGeomTotalLagTotalDispSolid) and the incremental form
    (nonLinGeomTotalLagSolid) solve the same equations: bit for bit the
    same correctors and fields."""
    m, bcs = _tl_box()
    kw = dict(law=1, use_mu_K=1, mu=1e6, K=2e7, n_correctors=3000, n_increments=1)
    Di, si, Gi, pi_ = pyoracle.solve(m, bcs, model=1, **kw)
    Dt, st, Gt, pt = pyoracle.solve(m, bcs, model=2, **kw)
    assert pi_["converged"] == pt["converged"] == 1
    assert pi_["n_correctors"] == pt["n_correctors"]
    assert np.array_equal(Di, Dt) and np.array_equal(si, st) and np.array_equal(Gi, Gt)


def test_tl_total_path_independent_without_stabilisation():
    """The total form solves for D itself: with RhieChow off its discrete
    equations do not depend on the increments, so three increments end at
    the one-increment answer."""
    m, bcs = _tl_box()
    kw = dict(model=2, law=1, use_mu_K=1, mu=1e6, K=2e7, n_correctors=8000, stab_scale=0.0,
              solution_tol=1e-9, alternative_tol=1e-10)
    D1, _, _, p1 = pyoracle.solve(m, bcs, n_increments=1, **kw)
    D3, _, _, p3 = pyoracle.solve(m, bcs, n_increments=3, **kw)
    assert p1["converged"] == p3["converged"] == 1
    assert np.linalg.norm(D3 - D1) / np.linalg.norm(D1) < 1e-6


def test_non_finite_field_stops_the_solve():
    """A neoHookean total Lagrangian solve that blows up (K/mu = 10, ten
    traction increments, no relaxation) stops at the first non-finite
    corrector, unconverged, as the library does (S4G_NAN_DETECTED); the
    NaN must not pass the convergence test."""
    m = sg.box_mesh(8, 8, 8, 1.0, 1.0, 1.0, 0.2, 5)
    t = np.tile(np.random.default_rng(5).normal(0, 1e5, 3), (int(m["patch_size"][5]), 1))
    bcs = [(1, None, None)] * 4 + [(0, None, None), (1, t, None)]
    D, _, _, p = pyoracle.solve(m, bcs, model=2, law=1, use_mu_K=1, mu=1e6, K=1e7,
                                n_correctors=3000, n_increments=10)
    assert p["nan_detected"] == 1 and p["converged"] == 0
    assert p["n_correctors"] < 200


@pytest.mark.parametrize("model", [1, 2])
def test_rigid_rotation_is_stress_free(model):
    """Frame indifference, as the reference's rigidRotation tutorials test
    it: a rigid rotation of 90 degrees about z prescribed on every boundary
    (fixedDisplacement (R - I) x, ramped over 45 increments) is recovered
    exactly -- D = (R - I) C, the leastSquares gradient being exact for a
    linear field -- and the neoHookean stress vanishes, in both total
    Lagrangian forms (1 incremental, 2 total displacement)."""
    m = sg.box_mesh(6, 5, 4, 1.0, 0.9, 0.8, 0.2, 3)
    th = np.radians(90.0)
    R = np.array([[np.cos(th), -np.sin(th), 0.0], [np.sin(th), np.cos(th), 0.0], [0.0, 0.0, 1.0]])
    bcs = []
    for p in range(6):
        s, n = int(m["patch_start"][p]), int(m["patch_size"][p])
        bcs.append((0, m["Cf"][s:s + n] @ (R - np.eye(3)).T, None))
    D, sig, G, p = pyoracle.solve(m, bcs, model=model, law=1, use_mu_K=1, mu=1e6, K=5e6,
                                  n_correctors=4000, n_increments=45, solution_tol=1e-10,
                                  alternative_tol=1e-11, ls_boundary_delta=1)
    assert p["converged"] == 1 and p["nan_detected"] == 0 and p["enforce_linear"] == 0
    exact = m["C"] @ (R - np.eye(3)).T
    assert np.abs(D - exact).max() < 1e-7 * np.abs(exact).max()
    assert np.abs(sig).max() < 1e-6 * 1e6          # below 1e-6 mu


def test_lame_cylinder_converges_at_second_order(tmp_path):
    """Thick-walled cylinder under internal pressure (the reference's
    pressurisedCylinder problem; Lame solution in plane strain) on curved
    annulus meshes written and read back as polyMesh: inner wall loaded by
    the pressure, outer wall and end faces given the exact displacement, so
    that the plane-strain field solves the 3-D problem.  The cell
    displacement converges to it at second order."""
    from solids4foam_gb300.foam_case import annulus_polymesh, read_case, write_polymesh
    a, b, h, E, nu, p = 0.5, 1.0, 0.1, 200e9, 0.3, 1e6

    def u_exact(X):
        r = np.hypot(X[:, 0], X[:, 1])
        ur = p * a ** 2 * (1 + nu) * ((1 - 2 * nu) * r + b ** 2 / r) / (E * (b ** 2 - a ** 2))
        return np.stack([ur * X[:, 0] / r, ur * X[:, 1] / r, 0 * r], axis=1)

    err = []
    for nr, nt in ((8, 64), (16, 128), (32, 256)):
        case = tmp_path / f"c{nr}"
        write_polymesh(str(case / "constant" / "polyMesh"), **annulus_polymesh(nr, nt, 1, a, b, h))
        m, _ = read_case(str(case), d_file=None)
        bcs = []
        for k in range(4):
            s, n = int(m["patch_start"][k]), int(m["patch_size"][k])
            bcs.append((1, None, np.full(n, p)) if k == 0 else (0, u_exact(m["Cf"][s:s + n]), None))
        D, sig, _, pf = pyoracle.solve(m, bcs, E=E, nu=nu, n_correctors=20000,
                                       solution_tol=1e-10, alternative_tol=1e-11)
        assert pf["converged"] == 1
        ue = u_exact(m["C"])
        err.append(np.linalg.norm(D - ue) / np.linalg.norm(ue))
    assert err[2] < 5e-5
    assert np.log2(err[1] / err[2]) > 1.8


def test_field_relaxation_rescues_the_corrector_loop():
    """relaxationFactors { fields { "D|DD" f; } } (the reference's "fixed"
    relaxField, used by its pressurisedCylinder tutorial with f = 0.9): on a
    jittered box at nu = 0.4 with a shear traction the unrelaxed loop runs
    away, while f = 0.9 and f = 0.7 converge to the same fixed point."""
    m = sg.box_mesh(10, 10, 10, 1.0, 1.0, 1.0, 0.2, 3)
    t = np.tile([1e5, 0.0, -1e6], (int(m["patch_size"][5]), 1))
    bcs = [(1, None, None)] * 4 + [(0, None, None), (1, t, None)]
    kw = dict(E=200e9, nu=0.4, n_correctors=3000, solution_tol=1e-10, alternative_tol=1e-11)
    D0, _, _, p0 = pyoracle.solve(m, bcs, **kw)
    assert p0["converged"] == 0 and np.abs(D0).max() > 1.0          # ran away
    D9, _, _, p9 = pyoracle.solve(m, bcs, field_relaxation=0.9, **kw)
    D7, _, _, p7 = pyoracle.solve(m, bcs, field_relaxation=0.7, **kw)
    assert p9["converged"] == 1 and p7["converged"] == 1
    assert np.linalg.norm(D9 - D7) / np.linalg.norm(D7) < 1e-6


def test_aitken_relaxation_keeps_the_fixed_point():
    """relaxationMethod Aitken (solidModel.C:842-896), restated as written:
    D -= alpha (D.prevIter - D), so alpha = 1 at the first corrector steps
    twice the correction, and later factors come from the last two
    residuals.  At nu = 0.3 it converges to the unrelaxed loop's fixed
    point; the factors stay in [0, 2] by construction."""
    m = sg.box_mesh(10, 10, 10, 1.0, 1.0, 1.0, 0.2, 3)
    t = np.tile([0.0, 1e5, -1e5], (int(m["patch_size"][5]), 1))
    bcs = [(1, None, None)] * 4 + [(0, None, None), (1, t, None)]
    kw = dict(E=200e9, nu=0.3, n_correctors=4000, solution_tol=1e-10, alternative_tol=1e-10)
    D0, _, _, p0 = pyoracle.solve(m, bcs, **kw)
    for fr in (0.0, 0.7):
        Da, _, _, pa = pyoracle.solve(m, bcs, relaxation_method=1, field_relaxation=fr, **kw)
        assert p0["converged"] == 1 and pa["converged"] == 1
        assert np.linalg.norm(Da - D0) / np.linalg.norm(D0) < 1e-7
    # one corrector: alpha = 1 doubles the step of the unrelaxed first solve
    D1, _, _, _ = pyoracle.solve(m, bcs, E=200e9, nu=0.3, n_correctors=1)
    A1, _, _, _ = pyoracle.solve(m, bcs, E=200e9, nu=0.3, n_correctors=1, relaxation_method=1)
    assert np.allclose(A1, 2.0 * D1, rtol=1e-12, atol=1e-20)


@pytest.mark.parametrize("model", [1, 2])
def test_homogeneous_finite_deformation(model):
    """A homogeneous deformation x = F X with stretch and shear (J = 1.188),
    prescribed on every boundary over 20 increments, is reproduced exactly
    by both total Lagrangian forms, and the stress everywhere is the
    neoHookean Cauchy stress of F, sigma = (mu dev(J^-2/3 F F^T) +
    K/2 (J^2 - 1) I) / J (neoHookeanElastic.C:275-303), restated here
    independently."""
    m = sg.box_mesh(6, 5, 4, 1.0, 0.9, 0.8, 0.2, 3)
    F = np.array([[1.2, 0.1, 0.0], [0.0, 0.9, 0.05], [0.0, 0.0, 1.1]])
    bcs = []
    for p in range(6):
        s, n = int(m["patch_start"][p]), int(m["patch_size"][p])
        bcs.append((0, m["Cf"][s:s + n] @ (F - np.eye(3)).T, None))
    mu, K = 1e6, 5e6
    J = np.linalg.det(F)
    bbar = J ** (-2.0 / 3.0) * F @ F.T
    S = (mu * (bbar - np.trace(bbar) / 3 * np.eye(3)) + 0.5 * K * (J ** 2 - 1) * np.eye(3)) / J
    expected = np.array([S[0, 0], S[0, 1], S[0, 2], S[1, 1], S[1, 2], S[2, 2]])
    D, sig, _, p = pyoracle.solve(m, bcs, model=model, law=1, use_mu_K=1, mu=mu, K=K,
                                  n_correctors=4000, n_increments=20, solution_tol=1e-10,
                                  alternative_tol=1e-11, ls_boundary_delta=1)
    assert p["converged"] == 1 and p["enforce_linear"] == 0
    assert np.abs(D - m["C"] @ (F - np.eye(3)).T).max() < 1e-7
    assert np.abs(sig - expected).max() < 1e-6 * np.abs(expected).max()


def test_pressurised_cylinder_readme_stresses(tmp_path):
    """The reference's pressurisedCylinder case (tutorials/solids/
    linearElasticity/pressurisedCylinder/README.md: r_i = 7 m, R_o =
    18.625 m, E = 10 GPa, nu = 0.3, p = 10 MPa in its plot script, 30 cells
    radially) against the analytical stresses that README gives,
    sigma_r = p r_i^2/(R_o^2 - r_i^2) (1 - R_o^2/r^2) and sigma_theta with
    (1 + R_o^2/r^2).  Those hold for plane stress and plane strain alike;
    the full annulus here is in plane strain (exact displacement on the
    outer wall and the end faces).  At the README's resolution the cell
    stresses agree to 1% (L2), and halving the cells improves them."""
    from solids4foam_gb300.foam_case import annulus_polymesh, read_case, write_polymesh
    a, b, E, nu, p, h = 7.0, 18.625, 10e9, 0.3, 10e6, 0.5

    def u_exact(X):
        r = np.hypot(X[:, 0], X[:, 1])
        ur = p * a ** 2 * (1 + nu) * ((1 - 2 * nu) * r + b ** 2 / r) / (E * (b ** 2 - a ** 2))
        return np.stack([ur * X[:, 0] / r, ur * X[:, 1] / r, 0 * r], axis=1)

    err = []
    for nr, nt in ((15, 60), (30, 120)):
        case = tmp_path / f"c{nr}"
        write_polymesh(str(case / "constant" / "polyMesh"), **annulus_polymesh(nr, nt, 1, a, b, h))
        m, _ = read_case(str(case), d_file=None)
        bcs = []
        for k in range(4):
            s, n = int(m["patch_start"][k]), int(m["patch_size"][k])
            bcs.append((1, None, np.full(n, p)) if k == 0 else (0, u_exact(m["Cf"][s:s + n]), None))
        _, sig, _, pf = pyoracle.solve(m, bcs, E=E, nu=nu, n_correctors=20000, solution_tol=1e-9,
                                       alternative_tol=1e-10)
        assert pf["converged"] == 1
        r = np.hypot(m["C"][:, 0], m["C"][:, 1])
        c, s_ = m["C"][:, 0] / r, m["C"][:, 1] / r
        sr = sig[:, 0] * c * c + 2 * sig[:, 1] * c * s_ + sig[:, 3] * s_ * s_
        st = sig[:, 0] * s_ * s_ - 2 * sig[:, 1] * c * s_ + sig[:, 3] * c * c
        k0 = p * a ** 2 / (b ** 2 - a ** 2)
        er = np.linalg.norm(sr - k0 * (1 - b ** 2 / r ** 2)) / np.linalg.norm(k0 * (1 - b ** 2 / r ** 2))
        et = np.linalg.norm(st - k0 * (1 + b ** 2 / r ** 2)) / np.linalg.norm(k0 * (1 + b ** 2 / r ** 2))
        err.append((er, et))
    assert err[1][0] < 0.01 and err[1][1] < 0.005
    assert err[1][0] < 0.5 * err[0][0] and err[1][1] < 0.5 * err[0][1]


def test_cooks_membrane_against_the_reference(tmp_path):
    """The reference's cooksMembrane tutorial (README.md "Expected Results"):
    E = 70 MPa, nu = 0.3333, left edge fixed, 6.25 MPa shear on the right,
    plane strain; the solids4foam prediction of the top-right corner's
    vertical displacement on 20 x 20 cells is 32.12 mm (foam-extend-4.1),
    finite-element codes converge to 32.20-32.28 mm.  The oracle in 2-D,
    with foam-extend's full boundary d vectors and the tutorial's controls,
    gives that prediction to 1% (plain leastSquares here against the
    tutorial's extendedLeastSquares 0) and refines towards the converged
    value."""
    from solids4foam_gb300.post import point_displacement
    corner = {}
    for n in (20, 40):
        m, m2 = cooks_membrane(tmp_path, n)
        nr = int(m2["patch_size"][1])
        bcs = [(0, None, None), (1, np.tile([0.0, 6.25e6, 0.0], (nr, 1)), None), (1, None, None)]
        D, _, G, p = pyoracle.solve(m2, bcs, E=70e6, nu=0.3333, n_correctors=5000,
                                    solution_tol=1e-7, alternative_tol=1e-7, tolerance=1e-9,
                                    rel_tol=0.1, max_iter=200, ls_boundary_delta=1,
                                    empty_direction=3)
        assert p["converged"] == 1 and np.all(D[:, 2] == 0.0)
        pts = m["points"]
        k = np.where((np.abs(pts[:, 0] - 0.048) < 1e-12) & (np.abs(pts[:, 1] - 0.060) < 1e-12))[0]
        corner[n] = point_displacement(m, D, G)[k, 1].mean() * 1e3      # mm
    assert abs(corner[20] - 32.12) < 0.01 * 32.12
    assert corner[20] < corner[40] < 32.28 and abs(corner[40] - 32.24) < 0.005 * 32.24


@pytest.mark.parametrize("args", [(3, 4, 5, 1.0, 2.0, 0.5, 0.2, 7), (10, 8, 6, 1.0, 1.0, 1.0, 0.3, 3),
                                  (24, 20, 16, 1.0, 1.0, 1.0, 0.2, 1),
                                  (17, 5, 9, 2.0, 0.2, 0.3, 0.0, 1)])
def test_oracle_box_mesh_equals_the_library_generator(built, args):
    """The oracle's own numpy box generator (oracle/box_mesh.py), which the
    CPU baseline uses so that no product code computes its inputs, gives
    the library generator's mesh bit for bit: addressing, points and the
    primitiveMesh geometry."""
    from oracle.box_mesh import box_mesh
    a = box_mesh(*args, points=True)
    b = sg.box_mesh(*args, points=True)
    for k in ("owner", "neighbour", "C", "V", "Cf", "Sf", "patch_start", "patch_size", "points"):
        assert np.array_equal(a[k], b[k]), k


def test_caller_subdomain_dic_is_thread_count_independent():
    """The processor-local DIC over a caller decomposition (dic_domain)
    gives the same solve on one thread and on several: the subdomains are
    independent and each is swept in cell order (only the OpenMP sums of
    the dot products change their order)."""
    from oracle.box_mesh import box_mesh, block_parts
    m = box_mesh(12, 10, 8, 1.0, 1.0, 1.0, 0.2, 5)
    dom = block_parts(12, 10, 8, 4)
    bcs = [(1, None, None)] * 4 + [(0, None, None), (1, None, np.full(120, 1e6))]
    out = [pyoracle.solve(m, bcs, dic_domain=dom, E=70e9, nu=0.33, n_threads=t, n_correctors=400)
           for t in (1, 4)]
    assert out[0][3]["n_correctors"] == out[1][3]["n_correctors"]
    assert out[0][3]["converged"] == 1
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel(out[1][0], out[0][0]) < 1e-10 and rel(out[1][1], out[0][1]) < 1e-10
