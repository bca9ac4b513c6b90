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
