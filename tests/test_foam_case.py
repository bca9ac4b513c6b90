"""OpenFOAM case files (s4g_foam_*): the polyMesh reader against the box
generator (written out and read back: bit-identical geometry), against a
hand-written two-prism mesh with known volumes and centroids, the D
boundaryField subset, and the errors it must raise.  No GPU needed."""
import os

import numpy as np
import pytest

from oracle import pyoracle
from solids4foam_gb300 import _lib
from solids4foam_gb300.cases import oracle_bcs
from solids4foam_gb300.foam_case import box_polymesh, read_case, write_box_case

HERE = os.path.dirname(os.path.abspath(__file__))
PRISMS = os.path.join(HERE, "golden", "foam_prisms")
HEADER = "FoamFile\n{\n    version 2.0;\n    format ascii;\n    class volVectorField;\n    object D;\n}\n"


def test_box_written_and_read_back_is_bit_identical(tmp_path):
    m = box_polymesh(5, 4, 3, 1.2, 1.0, 0.8, 0.2, 11)
    write_box_case(str(tmp_path / "constant" / "polyMesh"), m)
    r, bcs = read_case(str(tmp_path), d_file=None)
    assert bcs is None
    for k in ("owner", "neighbour", "C", "V", "Cf", "Sf", "patch_start", "patch_size"):
        assert np.array_equal(r[k], m[k]), k
    assert r["patch_names"] == list(m["patch_names"])
    assert r["patch_types"] == ["patch"] * 6


def test_two_prisms_geometry():
    r, _ = read_case(PRISMS, d_file=None)
    assert r["patch_names"] == ["bottom", "top", "sides"]
    assert r["patch_types"] == ["wall", "patch", "patch"]
    assert list(r["patch_start"]) == [1, 3, 5] and list(r["patch_size"]) == [2, 2, 4]
    np.testing.assert_allclose(r["V"], [0.5, 0.5], rtol=1e-14)
    np.testing.assert_allclose(r["C"], [[2 / 3, 1 / 3, 0.5], [1 / 3, 2 / 3, 0.5]], rtol=1e-14)
    np.testing.assert_allclose(r["Sf"][0], [-1.0, 1.0, 0.0], atol=1e-15)   # diagonal, owner -> neighbour
    np.testing.assert_allclose(r["Sf"][1], [0.0, 0.0, -0.5], atol=1e-15)   # bottom triangle, outward
    np.testing.assert_allclose(r["Cf"][1], [2 / 3, 1 / 3, 0.0], atol=1e-15)
    # closed cells: the area vectors of each cell sum to zero
    for c in range(2):
        s = sum(r["Sf"][f] * (1 if r["owner"][f] == c else -1)
                for f in range(9) if r["owner"][f] == c or (f < 1 and r["neighbour"][f] == c))
        np.testing.assert_allclose(s, 0.0, atol=1e-15)


def test_two_prisms_d_file():
    r, bcs = read_case(PRISMS)
    t, v, p, rf = bcs["bottom"]
    assert t == "fixedDisplacement" and p is None and rf == 1.0 and np.all(v == 0)
    t, v, p, rf = bcs["top"]
    assert t == "solidTraction" and rf == 0.5
    assert np.array_equal(v, [[1e5, 0, -1e6], [2e5, 0, -1e6]]) and np.array_equal(p, [3e5, 3e5])
    t, v, p, rf = bcs["sides"]   # matched by the ".*" key
    assert t == "solidTraction" and np.all(v == 0) and np.all(p == 0) and v.shape == (4, 3)


def test_read_case_solves_like_the_box(tmp_path):
    """A box written as a case with a D file and read back gives the
    oracle exactly the same solve as the box and the same conditions."""
    m = box_polymesh(6, 5, 4, 1.2, 1.0, 0.8, 0.2, 11)
    case = tmp_path
    write_box_case(str(case / "constant" / "polyMesh"), m)
    top = int(m["patch_size"][5])
    tr = np.tile([1e5, 0.0, -2e5], (top, 1))
    lines = " ".join(f"({a:.17g} {b:.17g} {c:.17g})" for a, b, c in tr)
    (case / "0").mkdir()
    (case / "0" / "D").write_text(HEADER + f"""
dimensions [0 1 0 0 0 0 0];
internalField uniform (0 0 0);
boundaryField
{{
    zmin {{ type fixedDisplacement; value uniform (0 0 0); }}
    zmax
    {{
        type solidTraction;
        traction nonuniform List<vector> {top} ({lines});
        pressure uniform 3e5;
        value uniform (0 0 0);
    }}
    "(x|y)(min|max)" {{ type solidTraction; traction uniform (0 0 0); pressure uniform 0; }}
}}
""")
    r, bcs = read_case(str(case))
    direct = {"zmin": ("fixedDisplacement", None, None),
              "zmax": ("solidTraction", tr, np.full(top, 3e5))}
    kw = dict(E=70e9, nu=0.33, n_correctors=300)
    Dr, sr, _, pr = pyoracle.solve(r, oracle_bcs(r, bcs), **kw)
    Db, sb, _, pb = pyoracle.solve(m, oracle_bcs(m, direct), **kw)
    assert pr["n_correctors"] == pb["n_correctors"]
    assert np.array_equal(Dr, Db) and np.array_equal(sr, sb)


def _d_error(tmp_path, body, match):
    case = tmp_path
    write_box_case(str(case / "constant" / "polyMesh"), box_polymesh(2, 2, 2))
    (case / "0").mkdir(exist_ok=True)
    (case / "0" / "D").write_text(HEADER + body)
    with pytest.raises(_lib.S4GError, match=match):
        read_case(str(case))


def test_d_errors_name_the_problem(tmp_path):
    free = "{ type solidTraction; traction uniform (0 0 0); pressure uniform 0; }"
    rest = " ".join(f"{n} {free}" for n in ("xmin", "xmax", "ymin", "ymax", "zmax"))
    _d_error(tmp_path, "boundaryField { zmin { type solidSymmetry; } " + rest + " }",
             "zmin: type solidSymmetry is not built")
    _d_error(tmp_path, "boundaryField { " + rest + " }", "zmin has no entry")
    _d_error(tmp_path, "boundaryField { zmin { type solidTraction; traction uniform (0 0 0); "
             "pressure uniform 0; tractionSeries { file \"t\"; } } " + rest + " }",
             "only one of traction, tractionSeries or tractionField")
    _d_error(tmp_path, "boundaryField { zmin { type solidTraction; tractionField T; "
             "pressure uniform 0; } " + rest + " }", "tractionField is not built")
    _d_error(tmp_path, "boundaryField { zmin { type fixedDisplacement; value nonuniform "
             "List<vector> 3((0 0 0) (0 0 0) (0 0 0)); } " + rest + " }", "3 values for 4 faces")


def test_mesh_errors(tmp_path):
    pm = tmp_path / "constant" / "polyMesh"
    write_box_case(str(pm), box_polymesh(2, 2, 2))
    text = (pm / "points").read_text()
    (pm / "points").write_text(text.replace("format      ascii", "format      binary"))
    with pytest.raises(_lib.S4GError, match="ASCII only"):
        read_case(str(tmp_path), d_file=None)
    (pm / "points").write_text(text)
    (pm / "owner").write_text("3\n(\n0\n1\n2\n)\n")
    with pytest.raises(_lib.S4GError, match="owner has 3 labels"):
        read_case(str(tmp_path), d_file=None)
    with pytest.raises(_lib.S4GError, match="cannot open"):
        read_case(str(tmp_path / "nowhere"), d_file=None)


def _prism_case(tmp_path, nx=4, ny=3, nz=3):
    from solids4foam_gb300.foam_case import prism_box_polymesh, write_polymesh
    write_polymesh(str(tmp_path / "constant" / "polyMesh"), **prism_box_polymesh(nx, ny, nz, 1.0, 0.9, 0.8))
    return read_case(str(tmp_path), d_file=None)[0]


def _linear_bcs(mesh, a, b):
    out = []
    for p in range(6):
        s, n = int(mesh["patch_start"][p]), int(mesh["patch_size"][p])
        out.append((0, a + mesh["Cf"][s:s + n] @ b.T, None))
    return out


def test_prism_mesh_patch_test(tmp_path):
    """The constant-strain patch test on a mesh of triangular prisms written
    and read back as a polyMesh: the linear field is reproduced to
    round-off (leastSquares with full boundary vectors)."""
    m = _prism_case(tmp_path)
    a = np.array([1e-6, 4e-6, 0.0])
    b = np.array([[2e-6, 3e-6, 0.0], [5e-6, 6e-6, 0.0], [0.0, 0.0, 0.0]])
    D, sig, G, perf = pyoracle.solve(m, _linear_bcs(m, a, b), E=200e9, nu=0.3, n_correctors=400,
                                     solution_tol=1e-13, alternative_tol=1e-14, tolerance=1e-15,
                                     rel_tol=0.0, ls_boundary_delta=1)
    np.testing.assert_allclose(D, a + m["C"] @ b.T, atol=1e-15, rtol=1e-8)
    np.testing.assert_allclose(G.reshape(-1, 3, 3), np.broadcast_to(b.T, (len(D), 3, 3)),
                               atol=1e-13)


def test_bad_arguments_are_errors_not_crashes(tmp_path):
    import ctypes as ct
    L = _lib.lib()
    h = ct.c_void_p()
    assert L.s4g_foam_read_mesh(None, ct.byref(h)) == _lib.BAD_ARG
    assert L.s4g_foam_read_mesh(PRISMS.encode(), None) == _lib.BAD_ARG
    d = _lib.MeshDesc()
    assert L.s4g_foam_mesh_desc(None, ct.byref(d), None) == _lib.BAD_ARG
    assert L.s4g_foam_read_mesh(os.path.join(PRISMS, "constant", "polyMesh").encode(),
                                ct.byref(h)) == _lib.OK
    try:
        assert L.s4g_foam_patch_name(h, -1) is None and L.s4g_foam_patch_type(h, 3) is None
        t, v = ct.c_int(), ct.c_void_p()
        assert L.s4g_foam_bc(h, 0, ct.byref(t), ct.byref(v), None, None) == _lib.BAD_ARG
        assert b"no D file" in L.s4g_last_error()
        assert L.s4g_foam_bc(h, 7, None, None, None, None) == _lib.BAD_ARG
        assert L.s4g_foam_apply_bcs(h, None) == _lib.BAD_ARG
        assert L.s4g_foam_read_d(h, None) == _lib.BAD_ARG
    finally:
        L.s4g_foam_free(h)
    L.s4g_foam_free(None)
    fs = np.array([0, 3], np.int32)
    fp = np.array([0, 1, 5], np.int32)
    own = np.zeros(1, np.int32)
    start = np.zeros(4, np.int32)
    assert L.s4g_point_cells(3, 1, fs.ctypes.data, fp.ctypes.data, 0, own.ctypes.data, None,
                             start.ctypes.data, None) == _lib.BAD_ARG
    pts = np.zeros((1, 3))
    pcs, pcc = np.array([0, 1], np.int32), np.array([4], np.int32)
    C, D, G, out = np.zeros((2, 3)), np.zeros((2, 3)), np.zeros((2, 9)), np.zeros((1, 3))
    assert L.s4g_point_interpolate(1, pts.ctypes.data, pcs.ctypes.data, pcc.ctypes.data, 2,
                                   C.ctypes.data, D.ctypes.data, G.ctypes.data,
                                   out.ctypes.data) == _lib.BAD_ARG
    assert b"cell out of range" in L.s4g_last_error()
    assert L.s4g_derived_fields(2, None, None, out.ctypes.data, None, None) == _lib.BAD_ARG
    assert L.s4g_box_mesh_faces(0, 1, 1, out.ctypes.data) == _lib.BAD_ARG
    m = box_polymesh(1, 1, 1)
    names = (ct.c_char_p * 6)(*[n.encode() for n in m["patch_names"]])
    assert L.s4g_foam_write_mesh(str(tmp_path / "missing" / "dir").encode(), 8,
                                 m["points"].ctypes.data, 6, m["face_start"].ctypes.data,
                                 m["face_points"].ctypes.data, 0, m["owner"].ctypes.data, None,
                                 6, names, m["patch_start"].ctypes.data,
                                 m["patch_size"].ctypes.data, None) == _lib.BAD_ARG


def test_d_entries_by_group_and_regex(tmp_path):
    """OpenFOAM's lookup order: a patch's own name, then its groups
    (inGroups in the boundary file), then quoted regular-expression keys."""
    import shutil
    shutil.copytree(os.path.join(PRISMS, "constant"), tmp_path / "constant")
    (tmp_path / "0").mkdir()
    (tmp_path / "0" / "D").write_text(HEADER + """
boundaryField
{
    ".*"  { type solidTraction; traction uniform (0 0 0); pressure uniform 0; }
    wall  { type fixedDisplacement; value uniform (0 0 1e-3); }
    top   { type solidTraction; traction uniform (1 2 3); pressure uniform 4; }
}
""")
    _, bcs = read_case(str(tmp_path))
    assert bcs["bottom"][0] == "fixedDisplacement" and np.all(bcs["bottom"][1] == [0, 0, 1e-3])
    assert bcs["top"][0] == "solidTraction" and np.all(bcs["top"][1] == [1, 2, 3])
    assert bcs["sides"][0] == "solidTraction" and np.all(bcs["sides"][2] == 0)


@pytest.mark.parametrize("kind", ["prisms", "annulus"])
def test_planning_general_meshes(tmp_path, kind):
    """Host-side mesh planning (renumbering, parts, DIC levels) of meshes
    that are not boxes: every renumbering gives a permutation, and the
    processor-local parts cover the cells."""
    import ctypes as ct
    from solids4foam_gb300.foam_case import annulus_polymesh, prism_box_polymesh, write_polymesh
    from solids4foam_gb300.solid_model import RENUMBER, _desc
    pm = (prism_box_polymesh(6, 5, 4, 1.0, 0.9, 0.8) if kind == "prisms"
          else annulus_polymesh(6, 48, 3, 0.5, 1.0, 0.3))
    write_polymesh(str(tmp_path / "constant" / "polyMesh"), **pm)
    m, _ = read_case(str(tmp_path), d_file=None)
    n = len(m["V"])
    for code in RENUMBER.values():
        for sub in (0, 1):
            keep = []
            d = _desc(m, keep)
            info = _lib.MeshInfo()
            perm = np.full(n, -1, np.int32)
            st = _lib.lib().s4g_mesh_plan(ct.byref(d), ct.byref(_lib.MeshOpts(code, 64, 0, sub, 0)),
                                          perm.ctypes.data, ct.byref(info))
            assert st == _lib.OK, _lib.lib().s4g_last_error()
            assert np.array_equal(np.sort(perm), np.arange(n))
            assert info.n_cells == n and info.n_parts >= n // 64 and info.n_levels_global >= 1


def _series_case(tmp_path, zmax, xmin="{ type solidTraction; traction uniform (0 0 0); pressure uniform 0; }"):
    write_box_case(str(tmp_path / "constant" / "polyMesh"), box_polymesh(2, 2, 2))
    (tmp_path / "constant" / "timeVsTraction").write_text(
        "// time (traction)\n(\n    (0 (0 0 0))\n    (4 (-20e6 0 5e6))\n    (10 (-50e6 0 12.5e6))\n)\n")
    (tmp_path / "constant" / "timeVsPressure").write_text("(\n(0 0)\n(10 3e5)\n)\n")
    (tmp_path / "constant" / "bent").write_text("((0 (0 0 0)) (5 (1 0 0)) (10 (1 0 0)))")
    (tmp_path / "0").mkdir(exist_ok=True)
    free = "{ type solidTraction; traction uniform (0 0 0); pressure uniform 0; }"
    (tmp_path / "0" / "D").write_text(HEADER + f"""
boundaryField
{{
    xmin {xmin}
    xmax {free}  ymin {free}  ymax {free}
    zmin {{ type fixedDisplacement; value uniform (0 0 0); }}
    zmax {zmax}
}}
""")
    return read_case(str(tmp_path))


def test_load_series_that_ramp_from_zero(tmp_path):
    """tractionSeries / pressureSeries / displacementSeries that are linear
    ramps from zero (the load-increment ramp) are read as their end value
    and end time; the file may be named by a regex key and $FOAM_CASE."""
    m, bcs = _series_case(tmp_path, """{ type solidTraction;
        tractionSeries { "fileName|file" "$FOAM_CASE/constant/timeVsTraction"; outOfBounds clamp; }
        pressureSeries { file "${FOAM_CASE}/constant/timeVsPressure"; }
        value uniform (0 0 0); }""")
    t, v, p, rf = bcs["zmax"]
    assert t == "solidTraction" and np.all(v == [-50e6, 0, 12.5e6]) and np.all(p == 3e5)
    assert m["load_ramp_end"] == 10.0 and not m["constant_loads_beside_ramp"]
    # a constant load beside a ramp is reported
    m, bcs = _series_case(tmp_path, """{ type fixedDisplacement;
        displacementSeries { file "$FOAM_CASE/constant/timeVsTraction"; } value uniform (0 0 0); }""",
                          xmin="{ type solidTraction; traction uniform (1e5 0 0); pressure uniform 0; }")
    assert bcs["zmax"][0] == "fixedDisplacement" and np.all(bcs["zmax"][1] == [-50e6, 0, 12.5e6])
    assert m["load_ramp_end"] == 10.0 and m["constant_loads_beside_ramp"]
    # no series at all
    m, _ = read_case(PRISMS)
    assert m["load_ramp_end"] is None


def test_load_tables_are_evaluated_in_time(tmp_path):
    """A load series that is not a ramp from zero (here a ramp to a plateau)
    is read whole: read_case reports a table (load_series 2, no ramp end)
    and gives its end value, and bcs_at evaluates it at the time steps'
    times -- linear between points, the end values outside the table
    (outOfBounds clamp, OpenFOAM's default), periodic with repeat, refused
    with error."""
    from solids4foam_gb300.foam_case import bcs_at
    m, bcs = _series_case(tmp_path, """{ type solidTraction; pressure uniform 0;
        tractionSeries { file "$FOAM_CASE/constant/bent"; } }""")
    assert m["load_series"] == 2 and m["load_ramp_end"] is None
    assert np.all(bcs["zmax"][1] == [1, 0, 0])
    times = [0.0, 2.0, 5.0, 7.5, 12.0, -1.0]
    got = [b["zmax"][1][0] for b in bcs_at(str(tmp_path), times)]
    want = np.interp(times, [0, 5, 10], [0, 1, 1])
    assert np.allclose(np.array(got)[:, 0], want, rtol=0, atol=1e-15)
    assert all(np.all(b["zmax"][1] == b["zmax"][1][0]) for b in bcs_at(str(tmp_path), times))
    # the other patches keep their constant values
    assert all(np.all(b["xmin"][1] == 0) and b["zmin"][0] == "fixedDisplacement"
               for b in bcs_at(str(tmp_path), times))
    # ramps from zero with a common end stay the increments' ramp
    m, _ = _series_case(tmp_path, """{ type solidTraction; pressure uniform 0;
        tractionSeries { file "$FOAM_CASE/constant/timeVsTraction"; } }""")
    assert m["load_series"] == 1 and m["load_ramp_end"] == 10.0
    # outOfBounds repeat: periodic over the table's span
    _series_case(tmp_path, """{ type solidTraction; pressure uniform 0;
        tractionSeries { file "$FOAM_CASE/constant/bent"; outOfBounds repeat; } }""")
    got = [b["zmax"][1][0, 0] for b in bcs_at(str(tmp_path), [12.5, 17.5, -7.5])]
    assert np.allclose(got, [0.5, 1.0, 0.5], rtol=0, atol=1e-15)
    # outOfBounds error
    _series_case(tmp_path, """{ type solidTraction; pressure uniform 0;
        tractionSeries { file "$FOAM_CASE/constant/bent"; outOfBounds error; } }""")
    assert bcs_at(str(tmp_path), [10.0])[0]["zmax"][1][0, 0] == 1.0
    with pytest.raises(_lib.S4GError, match="outside the series"):
        bcs_at(str(tmp_path), [10.5])


def test_other_load_series_are_rejected(tmp_path):
    with pytest.raises(_lib.S4GError, match="interpolationScheme step is not built"):
        _series_case(tmp_path, """{ type solidTraction; pressure uniform 0;
            tractionSeries { file "$FOAM_CASE/constant/timeVsTraction"; interpolationScheme step; } }""")
    with pytest.raises(_lib.S4GError, match="cannot open"):
        _series_case(tmp_path, """{ type solidTraction; pressure uniform 0;
            tractionSeries { file "$FOAM_CASE/constant/missing"; } }""")


def _controls_case(tmp_path, solid=None, mech=None, fvs=None):
    head = "FoamFile { version 2.0; format ascii; class dictionary; object x; }\n"
    (tmp_path / "constant").mkdir(exist_ok=True)
    (tmp_path / "system").mkdir(exist_ok=True)
    (tmp_path / "constant" / "solidProperties").write_text(head + (solid or """
solidModel     nonLinearGeometryTotalLagrangian;
"nonLinearGeometryTotalLagrangianCoeffs|nonLinearGeometryUpdatedLagrangianCoeffs"
{
    nCorrectors             20000;
    solutionTolerance       1e-08;
    alternativeTolerance    1e-09;
    infoFrequency           100;
    stabilisation { type RhieChow; scaleFactor 0.2; }
}
"""))
    (tmp_path / "constant" / "mechanicalProperties").write_text(head + (mech or """
planeStress     no;
mechanical
(
    rubber
    {
        type            neoHookeanElastic;
        rho             rho [1 -3 0 0 0 0 0] 1000;
        mu              mu [1 -1 -2 0 0 0 0] 3e+6;
        K               K [1 -1 -2 0 0 0 0] 2e+7;
    }
);
"""))
    (tmp_path / "system" / "fvSolution").write_text(head + (fvs or """
solvers
{
    "D|DD" { solver PCG; preconditioner FDIC; tolerance 1e-09; relTol 0.05; maxIter 500; }
}
"""))
    return str(tmp_path)


def test_case_controls(tmp_path):
    """solidProperties (coefficients under a regular-expression key),
    mechanicalProperties (dimensioned entries) and fvSolution map onto the
    model, law, solver and outer-loop arguments; unset entries keep the
    reference defaults."""
    from solids4foam_gb300.foam_case import read_controls
    c = read_controls(_controls_case(tmp_path))
    assert c["model"] == "nonLinearGeometryTotalLagrangian"
    assert c["law"] == dict(type="neoHookeanElastic", mu=3e6, K=2e7)
    assert c["solver"] == dict(preconditioner="DIC", tolerance=1e-9, relTol=0.05, maxIter=500)
    o = c["outer"]
    assert (o["nCorrectors"], o["solutionTolerance"], o["alternativeTolerance"]) == (20000, 1e-8, 1e-9)
    assert o["materialTolerance"] == 1e-5 and o["stabilisation"]["scaleFactor"] == 0.2
    c = read_controls(_controls_case(tmp_path, solid="solidModel linearGeometryTotalDisplacement;\n",
                                     mech="planeStress no; mechanical ( steel { type linearElastic; "
                                          "E E [1 -1 -2 0 0 0 0] 200e+9; nu 0.3; } );\n"))
    assert c["model"] == "linearGeometryTotalDisplacement"
    assert c["law"] == dict(type="linearElastic", E=200e9, nu=0.3)
    assert c["outer"]["nCorrectors"] == 10000 and c["outer"]["stabilisation"]["scaleFactor"] == 0.1


@pytest.mark.parametrize("part,text,match", [
    ("solid", "solidModel nonLinearGeometryUpdatedLagrangian;\n", "solidModel nonLinearGeometryUpdatedLagrangian is not built"),
    ("mech", "planeStress yes; mechanical ( s { type linearElastic; E 1e9; nu 0.3; } );\n", "planeStress yes"),
    ("mech", "planeStress no; mechanical ( a { type linearElastic; E 1e9; nu 0.3; } "
             "b { type linearElastic; E 2e9; nu 0.3; } );\n", "2 laws; one law is built"),
    ("mech", "planeStress no; mechanical ( s { type neoHookeanElastic; E 1e9; nu 0.3; mu 1; K 2; } );\n",
     "give E and nu, or mu and K"),
    ("mech", "planeStress no; mechanical ( s { type StVenantKirchhoffElastic; E 1e9; nu 0.3; } );\n",
     "law type StVenantKirchhoffElastic is not built"),
    ("fvs", "solvers { \"D|DD\" { solver GAMG; smoother GaussSeidel; tolerance 1e-9; relTol 0.1; } }\n",
     "solver GAMG is not built"),
    ("fvs", "solvers { \"D|DD\" { solver PCG; preconditioner GAMG; tolerance 1e-9; relTol 0.1; } }\n",
     "preconditioner GAMG is not built"),
])
def test_case_controls_refusals(tmp_path, part, text, match):
    from solids4foam_gb300.foam_case import read_controls
    with pytest.raises(_lib.S4GError, match=match):
        read_controls(_controls_case(tmp_path, **{part: text}))


def test_corrupt_case_files_are_errors(tmp_path):
    """Truncated or corrupted case files (seeded) end in S4GError or in a
    valid read, never in a crash; a uniform list with an absurd count is
    refused before it is expanded."""
    import random
    import shutil
    rng = random.Random(11)
    files = ("constant/polyMesh/points", "constant/polyMesh/faces", "constant/polyMesh/owner",
             "constant/polyMesh/neighbour", "constant/polyMesh/boundary", "0/D")
    for k in range(120):
        rel = files[k % len(files)]
        d = tmp_path / f"c{k}"
        shutil.copytree(PRISMS, d)
        text = (d / rel).read_text()
        if k % 2:
            text = text[:rng.randrange(len(text))]
        else:
            chars = list(text)
            for _ in range(rng.randint(1, 4)):
                chars[rng.randrange(len(chars))] = rng.choice('(){};0123456789-e. \n"/*')
            text = "".join(chars)
        (d / rel).write_text(text)
        try:
            read_case(str(d))
        except _lib.S4GError:
            pass
    d = tmp_path / "huge"
    shutil.copytree(PRISMS, d)
    (d / "constant" / "polyMesh" / "neighbour").write_text("2000000000{1}\n")
    with pytest.raises(_lib.S4GError, match="too long"):
        read_case(str(d))


def test_two_d_case(tmp_path):
    """A 2-D case (the cooksMembrane tutorial's set-up with frontAndBack of
    type empty) reads into the mesh without the empty faces -- bit for bit
    the mesh the 2-D tests build by hand -- with empty direction 3; the
    empty patch needs no boundary condition, the writers list it as empty,
    and the driver plans it as 2-D."""
    import json
    import subprocess
    from cases2d import cooks_membrane, cooks_membrane_case
    from solids4foam_gb300 import build as b
    from solids4foam_gb300.foam_case import load_case, write_results
    case = cooks_membrane_case(tmp_path / "case", 20)
    c = load_case(case)
    m = c["mesh"]
    _, ref = cooks_membrane(tmp_path / "ref", 20)
    for k in ("owner", "neighbour", "C", "V", "Cf", "Sf", "patch_start", "patch_size"):
        assert np.array_equal(m[k], ref[k]), k
    assert m["patch_names"] == ["left", "right", "topAndBottom"] and m["empty_direction"] == 3
    assert sorted(c["bcs"]) == ["left", "right", "topAndBottom"]
    assert c["model"] == "linearGeometryTotalDisplacement" and c["solver"]["maxIter"] == 200
    n = len(m["V"])
    write_results(case, "1", np.zeros((n, 3)), np.zeros((n, 6)), np.zeros((n, 9)))
    text = (tmp_path / "case" / "1" / "D").read_text()
    assert "frontAndBack\n    {\n        type            empty;" in text
    out = json.loads(subprocess.run([b.build_driver(), case, "--plan-only"], capture_output=True,
                                    text=True, check=True).stdout)
    assert out["empty_direction"] == 3 and out["cells"] == 400
    # the tutorial's extendedLeastSquares selects the full boundary delta
    assert c["ls_boundary_delta"] == 1 and out["ls_boundary_delta"] == 1
    with pytest.raises(_lib.S4GError, match="not normal to x, y or z"):
        read_case(cooks_membrane_case(tmp_path / "tilted", 4, rotate_deg=30.0))


def test_grad_scheme(tmp_path):
    """gradSchemes: leastSquares gives the patch-normal boundary delta (0),
    extendedLeastSquares the full face-centre delta (1); grad(D) before
    default; other schemes are refused by name."""
    import ctypes as ct
    head = "FoamFile { version 2.0; format ascii; class dictionary; object fvSchemes; }\n"
    f = tmp_path / "fvSchemes"
    L = _lib.lib()

    def read(text, field="D"):
        f.write_text(head + text)
        v = ct.c_int(-1)
        _lib.check(L.s4g_foam_read_grad_scheme(str(f).encode(), field.encode(), ct.byref(v)),
                   "s4g_foam_read_grad_scheme")
        return v.value
    assert read("gradSchemes { default leastSquares; }") == 0
    assert read("gradSchemes { default none; grad(D) extendedLeastSquares 0; }") == 1
    assert read("gradSchemes { default extendedLeastSquares 0; grad(D) leastSquares; }") == 0
    assert read("gradSchemes { default leastSquares; grad(D) extendedLeastSquares 0; }", "DD") == 0
    with pytest.raises(_lib.S4GError, match="Gauss is not built"):
        read("gradSchemes { default Gauss linear; }")
    with pytest.raises(_lib.S4GError, match="no scheme"):
        read("gradSchemes { default none; }")
