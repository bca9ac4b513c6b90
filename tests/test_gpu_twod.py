"""2-D on the device (s4g_mesh_opts.empty_direction): the empty patches'
faces are left out of the mesh, the leastSquares tensor is inverted as
OpenFOAM's inv() does with an empty direction, and that displacement
component is not solved (plane strain).  Checked on the reference's
cooksMembrane tutorial against the oracle and against the reference's own
published result."""
import numpy as np
import pytest

import solids4foam_gb300 as sg
from cases2d import cooks_membrane
from oracle import pyoracle
from solids4foam_gb300.post import point_displacement

pytestmark = pytest.mark.gpu
TOL_D, TOL_S = 1e-6, 1e-5


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("precision,dic", [("FP64", False), ("FP32_REFINE", False),
                                           ("FP64", True), ("FP32_REFINE", True)])
def test_cooks_membrane_2d_matches_oracle(ctx, tmp_path, precision, dic):
    """Cook's membrane run from its case files as the cooksMembrane tutorial
    sets it up (E = 70 MPa, nu = 0.3333, 6.25 MPa shear, plane strain,
    20 x 20 cells, gradSchemes extendedLeastSquares 0, which selects the full
    boundary delta), in plain FP64 and FP32 + refinement, with the exact
    and the processor-local DIC, against the oracle in the same DIC order.
    The z component stays exactly zero, and the top-right corner deflects by
    the reference's 20 x 20 result, 32.12 mm (README.md "Expected
    Results"), to 1%."""
    from cases2d import cooks_membrane_case
    from solids4foam_gb300.foam_case import load_case
    case = cooks_membrane_case(tmp_path / "case", 20)
    c = load_case(case)
    assert c["ls_boundary_delta"] == 1
    model, n_inc = sg.SolidModel.from_case(ctx, case, precision=precision, dic_subdomains=dic)
    D, sig, perf = model.evolve(n_inc)
    G = model.gradD()
    m2 = c["mesh"]
    nr = int(m2["patch_size"][1])
    t = np.tile([0.0, 6.25e6, 0.0], (nr, 1))
    Do, so, _, po = pyoracle.solve(m2, [(0, None, None), (1, t, None), (1, None, None)],
                                   perm=model.permutation(),
                                   dic_domain=model.parts() if dic else None, E=70e6, nu=0.3333,
                                   n_correctors=5000, solution_tol=1e-7, alternative_tol=1e-7,
                                   tolerance=1e-9, rel_tol=0.1, max_iter=200,
                                   ls_boundary_delta=1, empty_direction=3)
    model.close()
    assert po["converged"] == 1 and perf["converged"] == 1
    assert np.all(D[:, 2] == 0.0)
    if precision == "FP64":
        assert abs(perf["n_correctors"] - po["n_correctors"]) <= 1
        assert abs(perf["total_lin_iters"] - po["total_lin_iters"]) <= 0.005 * po["total_lin_iters"]
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S
    m, _ = cooks_membrane(tmp_path, 20)
    pts = m["points"]
    k = np.where((np.abs(pts[:, 0] - 0.048) < 1e-12) & (np.abs(pts[:, 1] - 0.060) < 1e-12))[0]
    corner = point_displacement(m, D, G)[k, 1].mean() * 1e3
    assert abs(corner - 32.12) < 0.01 * 32.12


def test_cooks_membrane_2d_total_lagrangian_matches_oracle(ctx, tmp_path):
    """The 2-D treatment in the total Lagrangian model: Cook's membrane in
    neoHookean rubber (mu = 0.5 MPa, K = 5 MPa, 50 kPa shear over two
    increments, traction relaxationFactor 0.5), plane strain, against the
    oracle in the same DIC order."""
    _, m2 = cooks_membrane(tmp_path, 12)
    nr = int(m2["patch_size"][1])
    t = np.tile([0.0, 5e4, 0.0], (nr, 1))
    bcs = {"left": ("fixedDisplacement", None, None), "right": ("solidTraction", t, None, 0.5)}
    outer = dict(nCorrectors=5000, solutionTolerance=1e-8, alternativeTolerance=1e-9)
    model = sg.SolidModel(ctx, m2, dict(type="neoHookeanElastic", mu=0.5e6, K=5e6), bcs,
                          model="nonLinearGeometryTotalLagrangian", outer=outer,
                          ls_boundary_delta=1, empty_direction=3)
    D, sig, perf = model.evolve(n_increments=2)
    Do, so, _, po = pyoracle.solve(m2, [(0, None, None), (1, t, None, 0.5), (1, None, None)],
                                   perm=model.permutation(), model=1, law=1, use_mu_K=1, mu=0.5e6,
                                   K=5e6, n_increments=2, n_correctors=5000, solution_tol=1e-8,
                                   alternative_tol=1e-9, ls_boundary_delta=1, empty_direction=3)
    model.close()
    assert po["converged"] == 1 and perf["converged"] == 1
    assert np.all(D[:, 2] == 0.0)
    assert rel(D, Do) < TOL_D and rel(sig, so) < TOL_S
