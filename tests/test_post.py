"""The steps after the corrector loop (s4g_point_cells,
s4g_point_interpolate, s4g_derived_fields) against a plain restatement of
the reference's formulas, and their exact cases.  No GPU needed."""
import numpy as np
import pytest

from oracle import pyoracle
from solids4foam_gb300.foam_case import (box_polymesh, prism_box_polymesh, read_case,
                                         write_polymesh)
from solids4foam_gb300.post import derived_fields, point_cells, point_displacement

A = np.array([1e-6, 4e-6, -2e-6])
B = np.array([[2e-6, 3e-6, 1e-6], [5e-6, 6e-6, 0.0], [-1e-6, 0.0, 4e-6]])  # D = A + B x


def _prisms(tmp_path):
    write_polymesh(str(tmp_path / "constant" / "polyMesh"), **prism_box_polymesh(4, 3, 3, 1.0, 0.9, 0.8))
    return read_case(str(tmp_path), d_file=None)[0]


def _restated(mesh, D, G):
    """enhancedVolPointInterpolate.C:351-423 in numpy (cells of each point
    in increasing order, weights 1/|x_p - C_c|)."""
    start, cells = point_cells(mesh)
    out = np.zeros((mesh["points"].shape[0], 3))
    for p, x in enumerate(mesh["points"]):
        cs = cells[start[p]:start[p + 1]]
        d = x - mesh["C"][cs]
        w = 1.0 / np.linalg.norm(d, axis=1)
        ext = D[cs] + np.einsum("ci,cij->cj", d, G[cs].reshape(-1, 3, 3))
        out[p] = (w[:, None] * ext).sum(0) / w.sum()
    return out


def test_point_cells_of_a_box():
    m = box_polymesh(3, 2, 2)
    start, cells = point_cells(m)
    counts = np.diff(start)
    assert counts.max() == 8 and counts.min() == 1        # interior point, corner point
    assert (counts == 1).sum() == 8
    for p in range(len(counts)):
        assert np.all(np.diff(cells[start[p]:start[p + 1]]) > 0)


@pytest.mark.parametrize("kind", ["box", "prisms"])
def test_linear_field_is_exact_at_the_points(kind, tmp_path):
    m = box_polymesh(5, 4, 3, 1.2, 1.0, 0.8, 0.25, 7) if kind == "box" else _prisms(tmp_path)
    D = A + m["C"] @ B.T
    G = np.broadcast_to(B.T.reshape(9), (len(D), 9))
    pD = point_displacement(m, D, G)
    np.testing.assert_allclose(pD, A + m["points"] @ B.T, rtol=0, atol=1e-18)


def test_matches_the_restatement_on_random_fields():
    m = box_polymesh(4, 3, 3, 1.0, 1.0, 1.0, 0.3, 5)
    rng = np.random.default_rng(4)
    D = rng.normal(size=(len(m["V"]), 3))
    G = rng.normal(size=(len(m["V"]), 9))
    np.testing.assert_allclose(point_displacement(m, D, G), _restated(m, D, G), rtol=1e-13,
                               atol=1e-15)


def test_point_displacement_of_a_solved_patch_test():
    """The oracle's patch-test solution (linear to round-off) interpolated
    to the points gives the linear field at the points."""
    m = box_polymesh(5, 4, 3, 1.0, 0.9, 0.8, 0.25, 3)
    bcs = []
    for p in range(6):
        s, n = int(m["patch_start"][p]), int(m["patch_size"][p])
        bcs.append((0, A + m["Cf"][s:s + n] @ B.T, None))
    D, sig, G, _ = pyoracle.solve(m, bcs, E=200e9, nu=0.3, n_correctors=400, solution_tol=1e-13,
                                  alternative_tol=1e-14, tolerance=1e-15, rel_tol=0.0,
                                  ls_boundary_delta=1)
    pD = point_displacement(m, D, G)
    np.testing.assert_allclose(pD, A + m["points"] @ B.T, rtol=1e-8, atol=1e-15)


def test_derived_fields():
    rng = np.random.default_rng(2)
    sig = rng.normal(size=(50, 6))
    G = rng.normal(size=(50, 9))
    seq, eps, epsEq = derived_fields(sig, G)

    def full(s):
        return np.array([[s[0], s[1], s[2]], [s[1], s[3], s[4]], [s[2], s[4], s[5]]])

    for c in range(50):
        S = full(sig[c])
        dev = S - np.trace(S) / 3 * np.eye(3)
        assert seq[c] == pytest.approx(np.sqrt(1.5 * np.sum(dev * dev)), rel=1e-14)
        g = G[c].reshape(3, 3)
        e = 0.5 * (g + g.T)
        np.testing.assert_allclose(full(eps[c]), e, rtol=1e-15)
        de = e - np.trace(e) / 3 * np.eye(3)
        assert epsEq[c] == pytest.approx(np.sqrt(2 / 3 * np.sum(de * de)), rel=1e-14)
    # uniaxial stress and pure shear
    s, _, _ = derived_fields(np.array([[7.0, 0, 0, 0, 0, 0], [0, 2.0, 0, 0, 0, 0]]))
    np.testing.assert_allclose(s, [7.0, 2.0 * np.sqrt(3.0)], rtol=1e-15)


def _field_lists(path):
    """(internalField rows, {patch: rows}) of an ASCII vol field written by
    s4g_foam_write_field."""
    import re
    text = open(path).read()

    def rows(block):
        n, body = re.match(r"\s*(\d+)\s*\((.*)\)\s*$", block, re.S).groups()
        vals = [list(map(float, r.strip("()").split())) for r in body.strip().splitlines()]
        assert len(vals) == int(n)
        return np.array(vals)

    internal = re.search(r"internalField\s+nonuniform List<\w+>(.*?)\n;", text, re.S).group(1)
    patches = {m.group(1): rows(m.group(2)) for m in re.finditer(
        r"\n    (\w+)\n    \{\n        type            calculated;\n        value           "
        r"nonuniform List<\w+>(.*?)\n;", text, re.S)}
    return rows(internal), patches


def test_written_fields(tmp_path):
    """D, sigma and sigmaEq written into a time directory: cell values as
    given; on the patches the prescribed displacement (fixedDisplacement)
    or, elsewhere, the gradient-extrapolated value -- exact for a linear
    field -- and the adjacent cell's stress."""
    from solids4foam_gb300.foam_case import write_box_case, write_results
    m = box_polymesh(4, 3, 3, 1.0, 0.9, 0.8, 0.2, 5)
    write_box_case(str(tmp_path / "constant" / "polyMesh"), m)
    (tmp_path / "0").mkdir()
    free = "{ type solidTraction; traction uniform (0 0 0); pressure uniform 0; }"
    (tmp_path / "0" / "D").write_text(
        "FoamFile { version 2.0; format ascii; class volVectorField; object D; }\n"
        f"boundaryField {{ xmin {free} xmax {free} ymin {free} ymax {free} zmax {free}\n"
        "  zmin { type fixedDisplacement; value uniform (0 0 1e-3); } }\n")
    D = A + m["C"] @ B.T
    G = np.broadcast_to(B.T.reshape(9), (len(D), 9))
    sig = np.random.default_rng(1).normal(size=(len(D), 6))
    write_results(str(tmp_path), "1", D, sig, G)
    cells, patches = _field_lists(str(tmp_path / "1" / "D"))
    np.testing.assert_allclose(cells, D, rtol=1e-11, atol=1e-20)
    for p, name in enumerate(m["patch_names"]):
        s, n = int(m["patch_start"][p]), int(m["patch_size"][p])
        want = (np.tile([0, 0, 1e-3], (n, 1)) if name == "zmin" else A + m["Cf"][s:s + n] @ B.T)
        np.testing.assert_allclose(patches[name], want, rtol=1e-11, atol=1e-20)
    cells, patches = _field_lists(str(tmp_path / "1" / "sigma"))
    np.testing.assert_allclose(cells, sig, rtol=1e-11)
    s, n = int(m["patch_start"][5]), int(m["patch_size"][5])
    np.testing.assert_allclose(patches["zmax"], sig[m["owner"][s:s + n]], rtol=1e-11)
    cells, _ = _field_lists(str(tmp_path / "1" / "sigmaEq"))
    np.testing.assert_allclose(cells[:, 0], derived_fields(sig)[0], rtol=1e-11)


def test_traction_sngrad_on_the_host():
    """s4g_traction_sngrad against the reference's formulas restated in
    numpy: the linear form ((t - n p) - n.(sigma - impK gradD)) / impK and
    the total Lagrangian form with the deformed normal Finv^T n."""
    import ctypes as ct
    from solids4foam_gb300 import _lib
    rng = np.random.default_rng(3)
    nf, impK = 7, 3.5e9
    t = rng.normal(size=(nf, 3)) * 1e6
    p = rng.normal(size=nf) * 1e5
    n = rng.normal(size=(nf, 3))
    n /= np.linalg.norm(n, axis=1)[:, None]
    s6 = rng.normal(size=(nf, 6)) * 1e6
    G = rng.normal(size=(nf, 3, 3)) * 1e-3
    F = np.eye(3) + 0.1 * rng.normal(size=(nf, 3, 3))
    Fi = np.linalg.inv(F)
    S = np.array([[[a[0], a[1], a[2]], [a[1], a[3], a[4]], [a[2], a[4], a[5]]] for a in s6])

    def call(Finv):
        out = np.zeros((nf, 3))
        args = [np.ascontiguousarray(a) for a in (t, p, n, s6, G.reshape(nf, 9))]
        fi = None if Finv is None else np.ascontiguousarray(Finv.reshape(nf, 9))
        assert _lib.lib().s4g_traction_sngrad(nf, *[a.ctypes.data for a in args],
                                              None if fi is None else fi.ctypes.data,
                                              ct.c_double(impK), out.ctypes.data) == _lib.OK
        return out

    lin = np.einsum("fi,fij->fj", n, S - impK * G)
    np.testing.assert_allclose(call(None), ((t - n * p[:, None]) - lin) / impK, rtol=1e-12, atol=1e-18)
    nc = np.einsum("fij,fi->fj", Fi, n)            # Finv^T & n
    nc /= np.linalg.norm(nc, axis=1)[:, None]
    tl = ((t - nc * p[:, None]) - np.einsum("fi,fij->fj", nc, S)
          + impK * np.einsum("fi,fij->fj", n, G)) / impK
    np.testing.assert_allclose(call(Fi), tl, rtol=1e-12, atol=1e-18)
