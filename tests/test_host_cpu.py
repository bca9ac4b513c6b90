"""CPU tests of the C ABI library: it loads, exports every declared symbol,
and its host-side logic (mesh generation, validation, DIC ordering and
scheduling) is correct.  No compute call needs a GPU here."""
import ctypes as ct
import os
import re

import numpy as np
import pytest

import solids4foam_gb300 as sg
from solids4foam_gb300 import _lib
from solids4foam_gb300.solid_model import _desc, plan

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "s4g.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(s4g_[A-Za-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(built):
    L = _lib.lib()
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(_lib.declared_symbols())
    assert L.s4g_abi_version() == 7
    assert L.s4g_status_str(_lib.NOT_CONVERGED) == b"NOT_CONVERGED"


def test_box_mesh_geometry(built):
    m = sg.box_mesh(7, 5, 4, 1.4, 1.0, 0.8, 0.2, 3)
    nC = m["V"].shape[0]
    assert np.isclose(m["V"].sum(), 1.4 * 1.0 * 0.8, rtol=1e-12)
    # closed cells: outward areas sum to zero
    acc = np.zeros((nC, 3))
    ni = m["neighbour"].shape[0]
    np.add.at(acc, m["owner"], m["Sf"])
    np.add.at(acc, m["neighbour"], -m["Sf"][:ni])
    assert np.abs(acc).max() < 1e-14
    # upper-triangular face order
    own = m["owner"][:ni]
    assert np.all(own < m["neighbour"])
    key = own.astype(np.int64) * nC + m["neighbour"]
    assert np.all(np.diff(key) > 0)
    # boundary patches planar and outward
    for k, (ax, side) in enumerate([(0, 0), (0, 1), (1, 0), (1, 1), (2, 0), (2, 1)]):
        s, n = m["patch_start"][k], m["patch_size"][k]
        nrm = m["Sf"][s:s + n] / np.linalg.norm(m["Sf"][s:s + n], axis=1)[:, None]
        assert np.allclose(nrm[:, ax], 1.0 if side else -1.0)
    # jitter is seeded and stays inside +-0.2 h
    m2 = sg.box_mesh(7, 5, 4, 1.4, 1.0, 0.8, 0.2, 3)
    assert np.array_equal(m["C"], m2["C"])
    m3 = sg.box_mesh(7, 5, 4, 1.4, 1.0, 0.8, 0.2, 4)
    assert not np.array_equal(m["C"], m3["C"])


@pytest.mark.parametrize("renumber", ["none", "RCM", "tiled"])
@pytest.mark.parametrize("shape", [(8, 8, 8), (20, 3, 5), (1, 1, 40)])
def test_plan_is_a_permutation_with_topological_parts(built, renumber, shape):
    m = sg.box_mesh(*shape, 1.0, 1.0, 1.0, 0.1, 1)
    n = m["V"].shape[0]
    perm, info = plan(m, renumber, part_size=64)
    assert sorted(perm.tolist()) == list(range(n))
    assert info["n_cells"] == n
    assert 1 <= info["part_depth"] <= info["n_parts"]
    assert info["n_levels_global"] >= 1
    if renumber == "none":
        assert np.array_equal(perm, np.arange(n))


def test_tiled_order_has_shallow_part_dag(built):
    m = sg.box_mesh(32, 32, 32, 1.0, 1.0, 1.0, 0.2, 1)
    _, tiled = plan(m, "tiled", part_size=512)
    _, natural = plan(m, "none", part_size=512)
    assert tiled["part_depth"] <= 10
    assert natural["part_depth"] > 5 * tiled["part_depth"]


def test_rcm_reduces_bandwidth(built):
    m = sg.box_mesh(12, 12, 12, 1.0, 1.0, 1.0, 0.0, 1)
    rng = np.random.default_rng(2)
    shuffle = rng.permutation(m["V"].shape[0])
    from oracle.pyoracle import renumber_mesh
    ms = renumber_mesh(m, shuffle)
    perm, _ = plan(ms, "RCM")
    inv = np.empty_like(perm)
    inv[perm] = np.arange(perm.shape[0])
    bw_rcm = np.abs(inv[ms["owner"][:ms["neighbour"].shape[0]]] - inv[ms["neighbour"]]).max()
    bw_shuffled = np.abs(ms["owner"][:ms["neighbour"].shape[0]] - ms["neighbour"]).max()
    assert bw_rcm < bw_shuffled / 4


def test_invalid_meshes_are_rejected(built):
    L = _lib.lib()
    m = sg.box_mesh(3, 3, 3, 1.0, 1.0, 1.0, 0.0, 1)
    bad = dict(m)
    bad["neighbour"] = m["neighbour"].copy()
    bad["neighbour"][0] = 999
    keep = []
    d = _desc(bad, keep)
    assert L.s4g_mesh_plan(ct.byref(d), None, None, None) == _lib.BAD_ARG
    assert b"neighbour" in L.s4g_last_error()
    bad = dict(m)
    bad["V"] = m["V"].copy()
    bad["V"][3] = -1.0
    d = _desc(bad, keep)
    assert L.s4g_mesh_plan(ct.byref(d), None, None, None) == _lib.BAD_ARG
    bad = dict(m)
    bad["C"] = m["C"].copy()
    bad["C"][0, 0] = np.nan
    d = _desc(bad, keep)
    assert L.s4g_mesh_plan(ct.byref(d), None, None, None) == _lib.BAD_ARG
    bad = dict(m)
    bad["patch_size"] = m["patch_size"].copy()
    bad["patch_size"][2] += 1
    d = _desc(bad, keep)
    assert L.s4g_mesh_plan(ct.byref(d), None, None, None) == _lib.BAD_ARG
    # box generator refuses inverting jitter and bad sizes
    assert L.s4g_box_mesh_build(2, 2, 2, 1.0, 1.0, 1.0, 0.7, 1, *([None] * 9)) == _lib.BAD_ARG


def test_no_device_is_reported_without_gpu(built):
    """Without a GPU the context refuses to start: no CPU fallback."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(sg.S4GError) as e:
        sg.Context(0)
    assert e.value.status == _lib.NO_DEVICE


def test_ctypes_structs_match_the_c_header(tmp_path):
    """Every ctypes mirror has the size and field offsets of its C struct
    (compiled against include/s4g.h with the host C compiler, as strict
    C99)."""
    import ctypes as ct
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    pairs = {"s4g_ctx_opts": _lib.CtxOpts, "s4g_mesh_desc": _lib.MeshDesc,
             "s4g_mesh_opts": _lib.MeshOpts, "s4g_mesh_info": _lib.MeshInfo,
             "s4g_law": _lib.Law, "s4g_lin_solver": _lib.LinSolver, "s4g_outer": _lib.Outer,
             "s4g_perf": _lib.Perf, "s4g_server_opts": _lib.ServerOpts,
             "s4g_server_stats": _lib.ServerStats, "s4g_request": _lib.Request}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "s4g.h"', "int main(void) {"]
    for cname, py in pairs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    # the header is plain C: strict C99 with every warning an error
    subprocess.run([cc, "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I",
                    os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for ln in out.splitlines():
        c, f, v = ln.split()
        got[(c, f)] = int(v)
    for cname, py in pairs.items():
        assert got[(cname, "size")] == ct.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def _wait_for(srv, cond, timeout=10.0):
    """Polls the server's statistics until cond(stats) holds."""
    import time
    t0 = time.perf_counter()
    while True:
        st = srv.stats()
        if cond(st) or time.perf_counter() - t0 > timeout:
            return st
        time.sleep(0.001)


def test_server_scheduler_dry_run(built):
    """The serving scheduler without a GPU (dry run): rejection of what can
    never fit, cancellation of a queued request, first-fit admission by
    footprint (small requests pass a large one that waits for memory), the
    memory budget never exceeded, and the latency statistics.  The dry run
    holds a slot 10 ms per thousand cells (640 ms for the large request),
    and the test polls for each state rather than sleeping."""
    m_small = sg.box_mesh(6, 6, 6, 1.0, 1.0, 1.0, 0.1, 1)
    m_big = sg.box_mesh(40, 40, 40, 1.0, 1.0, 1.0, 0.1, 1)
    law = dict(type="linearElastic", E=70e9, nu=0.33)
    bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", [0, 0, -1e5], None)}
    # one slot: a queued request can be cancelled; an oversized one is rejected
    srv = sg.Server(max_slots=1, memory_budget=1 << 30, dry_run=True, dry_run_us_per_kcell=10000)
    with pytest.raises(_lib.S4GError, match="ADMISSION_REJECTED"):
        srv.submit(sg.box_mesh(160, 160, 160, 1.0, 1.0, 1.0, 0.1, 1), law, bcs)
    big = srv.submit(m_big, law, bcs)
    big_bytes = _wait_for(srv, lambda st: st["running"] == 1)["bytes_in_use"]
    assert big_bytes > 0
    queued = srv.submit(m_small, law, bcs)
    srv.cancel(queued)
    assert srv.result(queued)[0] == _lib.CANCELLED
    assert srv.result(big)[0] == _lib.OK
    st = srv.stats()
    assert st["rejected"] == 1 and st["cancelled"] == 1 and st["completed"] == 1
    srv.close()
    # two slots, memory for one large request: small ones pass the second large one
    srv = sg.Server(max_slots=2, memory_budget=int(1.5 * big_bytes), dry_run=True,
                    dry_run_us_per_kcell=10000)
    b1 = srv.submit(m_big, law, bcs)
    b2 = srv.submit(m_big, law, bcs)
    smalls = [srv.submit(m_small, law, bcs) for _ in range(4)]
    st = _wait_for(srv, lambda st: st["completed"] >= 4)
    # the four small ones ran beside the first large one; the second waits
    assert st["completed"] == 4 and st["running"] == 1 and st["queued"] == 1
    assert st["bytes_in_use"] <= st["memory_budget"]
    for rid in smalls + [b1, b2]:
        status, D, sig, perf = srv.result(rid)
        assert status == _lib.OK and D.shape == (sig.shape[0], 3)
    st = srv.stats()
    assert st["completed"] == 6
    assert 0 < st["p50_ms"] <= st["p99_ms"] and st["solves_per_s"] > 0
    # the second large request finished last: the small ones did not wait for it
    assert st["p99_ms"] > 1000
    srv.close()


def test_server_footprint_of_the_models(built):
    """Dry run: both total Lagrangian forms are admitted and sized above the
    linear-geometry model (their extra fields); a traction relaxation
    factor, which requests cannot carry, is refused."""
    m = sg.box_mesh(12, 12, 12, 1.0, 1.0, 1.0, 0.1, 1)
    bcs = {"zmin": ("fixedDisplacement", None, None), "zmax": ("solidTraction", [0, 0, -1e5], None)}
    lin = dict(type="linearElastic", E=70e9, nu=0.33)
    neo = dict(type="neoHookeanElastic", mu=1e6, K=2e7)
    used = {}
    for model, law in (("linearGeometryTotalDisplacement", lin),
                       ("nonLinearGeometryTotalLagrangian", neo),
                       ("nonLinearGeometryTotalLagrangianTotalDisplacement", neo)):
        # the dry run holds its slot for 1728 cells x 0.3 s/kcell, long enough
        # to be seen running on a loaded machine
        srv = sg.Server(max_slots=1, memory_budget=1 << 32, dry_run=True, dry_run_us_per_kcell=300000)
        rid = srv.submit(m, law, bcs, model=model)
        used[model] = _wait_for(srv, lambda st: st["running"] == 1)["bytes_in_use"]
        assert srv.result(rid)[0] == _lib.OK
        srv.close()
    assert used["nonLinearGeometryTotalLagrangian"] > used["linearGeometryTotalDisplacement"] > 0
    assert (used["nonLinearGeometryTotalLagrangianTotalDisplacement"]
            == used["nonLinearGeometryTotalLagrangian"])
    # a solidTraction relaxationFactor travels with the request; one outside
    # (0, 1] is refused at submit
    srv = sg.Server(max_slots=1, dry_run=True)
    rid = srv.submit(m, lin, {"zmax": ("solidTraction", [0, 0, -1e5], None, 0.5)})
    assert srv.result(rid)[0] == _lib.OK
    with pytest.raises(_lib.S4GError, match="BAD_ARG"):
        srv.submit(m, lin, {"zmax": ("solidTraction", [0, 0, -1e5], None, 1.5)})
    srv.close()


def test_caller_decomposition_plan(built):
    """s4g_mesh_opts.part_of_cell: the caller's subdomains become the
    processor-local DIC's parts (in the caller's cell order); it needs the
    caller's numbering and the processor-local DIC, and ids must be dense."""
    from oracle.box_mesh import block_parts
    m = sg.box_mesh(16, 8, 8, 1.0, 1.0, 1.0, 0.2, 3)
    parts = block_parts(16, 8, 8, 4)
    perm, info = plan(m, renumber="none", dic_subdomains=True, parts=parts)
    assert info["n_parts"] == 16 and np.array_equal(perm, np.arange(16 * 8 * 8))
    # in-part levels of a 4^3 block in lexicographic order: i + j + k
    assert info["max_local_levels"] == 10
    # lexicographic blocks: at most three lower and three upper neighbours
    # per row, so the fixed-slot tables; a shuffled cell order within the
    # parts needs the generic tables
    assert info["local_slots"] == 1
    from oracle.pyoracle import renumber_mesh
    shuffle = np.random.default_rng(1).permutation(16 * 8 * 8)
    _, info2 = plan(renumber_mesh(m, shuffle), renumber="none", dic_subdomains=True,
                    parts=parts[shuffle])
    assert info2["n_parts"] == 16 and info2["local_slots"] == 0
    for kw in (dict(renumber="tiled", dic_subdomains=True), dict(renumber="none")):
        with pytest.raises(_lib.S4GError, match="part_of_cell"):
            plan(m, parts=parts, **kw)
    gap = parts.copy()
    gap[gap == 3] = 2
    with pytest.raises(_lib.S4GError, match="every id used"):
        plan(m, renumber="none", dic_subdomains=True, parts=gap)


def test_time_step_and_series_entry_points_check_their_arguments(built):
    """s4g_solve_step, s4g_state_reset and the series entry points refuse
    null handles with S4G_BAD_ARG (no device is touched)."""
    L = _lib.lib()
    perf = _lib.Perf()
    assert L.s4g_solve_step(None, 0, None, None, ct.byref(perf)) == _lib.BAD_ARG
    assert L.s4g_state_reset(None) == _lib.BAD_ARG
    kind = ct.c_int()
    assert L.s4g_foam_series_kind(None, ct.byref(kind)) == _lib.BAD_ARG
    t = ct.c_int()
    assert L.s4g_foam_bc_at(None, 0, 0.0, ct.byref(t), None, None, None) == _lib.BAD_ARG
    assert L.s4g_foam_apply_bcs_at(None, None, 0.0) == _lib.BAD_ARG
