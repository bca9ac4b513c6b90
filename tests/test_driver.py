"""The standalone C++ driver (solids4foam_gb300/driver/s4g_solve_case.cpp)
built beside libs4g.so: host-side planning of a case read from disk, and
its failure modes.  The full solve needs a GPU."""
import json
import os
import subprocess

import pytest

from solids4foam_gb300 import build as b
from solids4foam_gb300.foam_case import box_polymesh, write_box_case

HERE = os.path.dirname(os.path.abspath(__file__))
PRISMS = os.path.join(HERE, "golden", "foam_prisms")


def run(*args):
    exe = b.build_driver()
    return subprocess.run([exe, *args], capture_output=True, text=True, timeout=120)


def test_plan_only_reads_the_case():
    r = run(PRISMS, "--plan-only")
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout)
    assert (out["cells"], out["faces"], out["points"], out["patches"]) == (2, 9, 8, 3)


def test_plan_only_box_case(tmp_path):
    write_box_case(str(tmp_path / "constant" / "polyMesh"), box_polymesh(10, 8, 6, jitter=0.2, seed=3))
    r = run(str(tmp_path), "--plan-only", "--renumber", "RCM", "--part-size", "64")
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout)
    assert out["cells"] == 480 and out["parts"] > 1


def test_errors_are_loud(tmp_path):
    r = run(str(tmp_path), "--plan-only")              # no polyMesh there
    assert r.returncode == 2 and "cannot open" in r.stderr
    r = run(PRISMS, "--model", "nonsense")
    assert r.returncode == 1 and "usage" in r.stderr


def test_no_device_is_an_error():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = run(PRISMS)
    assert r.returncode == 2 and "NO_DEVICE" in r.stderr


def _ramp_case(tmp_path, xmin_traction="0 0 0"):
    write_box_case(str(tmp_path / "constant" / "polyMesh"), box_polymesh(3, 3, 3))
    (tmp_path / "constant" / "timeVsTraction").write_text("((0 (0 0 0)) (10 (0 0 -1e5)))")
    (tmp_path / "system").mkdir()
    (tmp_path / "system" / "controlDict").write_text(
        "FoamFile { version 2.0; format ascii; class dictionary; object controlDict; }\n"
        "application solids4Foam;\nstartTime 0;\nendTime 10;\ndeltaT 0.5;\n")
    (tmp_path / "0").mkdir()
    free = "{ type solidTraction; traction uniform (0 0 0); pressure uniform 0; }"
    (tmp_path / "0" / "D").write_text(
        "FoamFile { version 2.0; format ascii; class volVectorField; object D; }\n"
        "boundaryField {\n"
        f"  xmin {{ type solidTraction; traction uniform ({xmin_traction}); pressure uniform 0; }}\n"
        f"  xmax {free} ymin {free} ymax {free}\n"
        "  zmin { type fixedDisplacement; value uniform (0 0 0); }\n"
        "  zmax { type solidTraction; pressure uniform 0;\n"
        "         tractionSeries { file \"$FOAM_CASE/constant/timeVsTraction\"; outOfBounds clamp; } }\n"
        "}\n")
    return str(tmp_path)


def test_load_ramp_sets_the_increments(tmp_path):
    """A total Lagrangian case whose load is a series ramping from zero runs
    one increment per time step of its controlDict (10 / 0.5 = 20)."""
    case = _ramp_case(tmp_path)
    r = run(case, "--plan-only", "--model", "nonLinearGeometryTotalLagrangian")
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout)
    assert out["load_ramp_end"] == 10 and out["increments"] == 20
    out = json.loads(run(case, "--plan-only", "--model", "nonLinearGeometryTotalLagrangian",
                         "--increments", "4").stdout)
    assert out["increments"] == 4
    out = json.loads(run(case, "--plan-only").stdout)   # linear geometry: one solve
    assert out["increments"] == 1


def test_load_tables_run_time_steps(tmp_path):
    """A load table that is not a ramp from zero (load, then unload) runs
    one evolve() per controlDict time step (s4g_solve_step), its series
    evaluated at each step's time; --time-steps asks the same of a ramp."""
    case = _ramp_case(tmp_path)
    (tmp_path / "constant" / "timeVsTraction").write_text(
        "((0 (0 0 0)) (5 (0 0 -1e5)) (10 (0 0 -2e4)))")
    for model in ("linearGeometryTotalDisplacement", "nonLinearGeometryTotalLagrangian"):
        r = run(case, "--plan-only", "--model", model)
        assert r.returncode == 0, r.stderr
        out = json.loads(r.stdout)
        assert out["load_series"] == 2 and out["time_steps"] == 20 and out["load_ramp_end"] == 0
    (tmp_path / "constant" / "timeVsTraction").write_text("((0 (0 0 0)) (10 (0 0 -1e5)))")
    out = json.loads(run(case, "--plan-only").stdout)
    assert out["load_series"] == 1 and out["time_steps"] == 0
    out = json.loads(run(case, "--plan-only", "--time-steps").stdout)
    assert out["time_steps"] == 20


def test_constant_load_beside_a_ramp_is_refused_for_tl(tmp_path):
    case = _ramp_case(tmp_path, xmin_traction="1e5 0 0")
    r = run(case, "--plan-only", "--model", "nonLinearGeometryTotalLagrangianTotalDisplacement")
    assert r.returncode == 2 and "constant loads beside load series" in r.stderr


def test_relaxation_factors(tmp_path):
    """Field relaxation of the solved field is built and read from the
    case (in either fvSolution form; a factor for another field is
    ignored); equation relaxation is not built and is refused by name."""
    case = _ramp_case(tmp_path)
    fvs = tmp_path / "system" / "fvSolution"
    head = "FoamFile { version 2.0; format ascii; class dictionary; object fvSolution; }\n"
    fvs.write_text(head + 'relaxationFactors { fields { "D|DD" 0.9; } equations { U 0.5; } }\n')
    r = run(case, "--plan-only")
    assert r.returncode == 0, r.stderr
    assert json.loads(r.stdout)["fieldRelaxation"] == 0.9
    fvs.write_text(head + "relaxationFactors { equations { DD 0.99; } }\n")
    r = run(case, "--plan-only", "--model", "nonLinearGeometryTotalLagrangian")
    assert r.returncode == 2 and "equation relaxationFactors for DD (0.99)" in r.stderr
    fvs.write_text(head + "relaxationFactors { D 0.7; }\n")          # the older flat form
    assert json.loads(run(case, "--plan-only").stdout)["fieldRelaxation"] == 0.7
    fvs.write_text(head + "relaxationFactors { fields { p 0.3; } }\n")
    assert json.loads(run(case, "--plan-only").stdout)["fieldRelaxation"] == 1


def test_time_window_other_than_the_series_is_refused(tmp_path):
    """Load series are applied up to their end value, which is the
    reference's load at endTime only for a run from 0 to the series' end:
    a run that stops before it, or starts later, is refused (exit 2), by
    the driver and by foam_case.load_case alike."""
    from solids4foam_gb300.foam_case import load_case
    case = _ramp_case(tmp_path)
    cd = tmp_path / "system" / "controlDict"
    head = "FoamFile { version 2.0; format ascii; class dictionary; object controlDict; }\n"
    (tmp_path / "system" / "fvSolution").write_text(
        head + 'solvers { "D|DD" { solver PCG; preconditioner DIC; } }\n')
    (tmp_path / "constant" / "solidProperties").write_text(
        head + "solidModel linearGeometryTotalDisplacement;\n")
    (tmp_path / "constant" / "mechanicalProperties").write_text(
        head + "planeStress no;\nmechanical ( r { type linearElastic; E 2e11; nu 0.3; } );\n")
    for window in ("startTime 0;\nendTime 5;\ndeltaT 0.5;\n", "startTime 2;\nendTime 10;\ndeltaT 0.5;\n"):
        cd.write_text(head + window)
        for model in ("linearGeometryTotalDisplacement", "nonLinearGeometryTotalLagrangian"):
            r = run(case, "--plan-only", "--model", model)
            assert r.returncode == 2 and "only a run from 0 to the series' end" in r.stderr
        with pytest.raises(ValueError, match="only a run from 0 to the series' end"):
            load_case(case)


def test_controls_come_from_the_case(tmp_path):
    """Without options the driver takes model, law and controls from the
    case's dictionaries; options override them."""
    case = _ramp_case(tmp_path)
    head = "FoamFile { version 2.0; format ascii; class dictionary; object x; }\n"
    (tmp_path / "constant" / "solidProperties").write_text(
        head + "solidModel nonLinearGeometryTotalLagrangianTotalDisplacement;\n"
        "nonLinearGeometryTotalLagrangianTotalDisplacementCoeffs { nCorrectors 777; }\n")
    (tmp_path / "constant" / "mechanicalProperties").write_text(
        head + "planeStress no;\nmechanical ( r { type neoHookeanElastic; mu 2e6; K 3e7; } );\n")
    (tmp_path / "system" / "fvSolution").write_text(
        head + 'solvers { "D|DD" { solver PCG; preconditioner FDIC; tolerance 1e-8; relTol 0.2; } }\n')
    out = json.loads(run(case, "--plan-only").stdout)
    assert out["model"] == "nonLinearGeometryTotalLagrangianTotalDisplacement"
    assert (out["law"], out["mu"], out["K"], out["use_mu_K"]) == ("neoHookeanElastic", 2e6, 3e7, 1)
    assert (out["nCorrectors"], out["tolerance"], out["relTol"]) == (777, 1e-8, 0.2)
    assert out["increments"] == 20                 # the traction ramp over 10 / 0.5
    out = json.loads(run(case, "--plan-only", "--nCorrectors", "50", "--mu", "1e6").stdout)
    assert (out["nCorrectors"], out["mu"]) == (50, 1e6)


def test_python_load_case_matches_the_driver(tmp_path):
    """foam_case.load_case resolves a case as the C++ driver does."""
    from solids4foam_gb300.foam_case import load_case
    case = _ramp_case(tmp_path)
    head = "FoamFile { version 2.0; format ascii; class dictionary; object x; }\n"
    (tmp_path / "constant" / "solidProperties").write_text(
        head + "solidModel nonLinearGeometryTotalLagrangian;\n")
    (tmp_path / "constant" / "mechanicalProperties").write_text(
        head + "planeStress no;\nmechanical ( r { type neoHookeanElastic; mu 2e6; K 3e7; } );\n")
    (tmp_path / "system" / "fvSolution").write_text(
        head + 'solvers { "D|DD" { solver PCG; preconditioner DIC; tolerance 1e-8; relTol 0.2; } }\n')
    c = load_case(case)
    drv = json.loads(run(case, "--plan-only").stdout)
    assert c["model"] == drv["model"] and c["n_increments"] == drv["increments"] == 20
    assert c["law"] == dict(type="neoHookeanElastic", mu=2e6, K=3e7)
    assert c["bcs"]["zmax"][0] == "solidTraction" and list(c["bcs"]["zmax"][1][0]) == [0, 0, -1e5]
    (tmp_path / "system" / "fvSolution").write_text(
        head + 'solvers { "D|DD" { solver PCG; preconditioner DIC; } }\n'
        'relaxationFactors { fields { DD 0.8; } }\n')
    assert load_case(case)["outer"]["fieldRelaxation"] == 0.8
    (tmp_path / "system" / "fvSolution").write_text(
        head + 'solvers { "D|DD" { solver PCG; preconditioner DIC; } }\n'
        'relaxationFactors { equations { DD 0.8; } }\n')
    with pytest.raises(ValueError, match="equation relaxationFactors for DD"):
        load_case(case)
