#!/usr/bin/env python
"""Benchmark of the segregated finite-volume solid solve on GB300.

One step is one full solve of the benchmark case: the 128^3 jittered unit
cube (2,097,152 hex cells, interior vertices jittered +-0.2 h, seed 1),
linear elastic E = 70 GPa, nu = 0.33, bottom fixed, top pressure 10 MPa,
sides traction-free, linearGeometryTotalDisplacement with PCG+DIC (tol 1e-9,
relTol 0.1) and outer tolerance 1e-6 / 2000 correctors -- run to
convergence through the library's public API.  By default the inner solves
run in FP32 with FP64 refinement, and the DIC is processor-local over
8^3-cell blocks given as the caller's decomposition (the preconditioner of a
decomposed run with 4096 processors); one plain FP64 solve of the same case
is timed beside it.  Inputs are synthetic (generated from the seed); the
working set (about 1.7 GB) is far larger than L2, so no L2 flush is needed
between steps.  The timed steps run the production path (CUDA graphs, no
per-kernel events); the per-kernel breakdown and the roofline come from one
more solve with CUDA events on every launch.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
                  [--precision FP32_REFINE|FP64] [--n 128] [--dic blocks|library|exact]
                  [--no-fp64] [--no-cpu] [--no-batched] [--no-served] [--e2e-steps 1]

--impl reference runs one full FP64 CPU solve of the same case by the oracle
(the restatement of the reference's solve; the reference itself needs an
OpenFOAM installation that is not available) on all host cores, with the
same DIC subdomains and inputs from the oracle's own mesh generator, and
reports the same metric.  It leaves its result where a GPU arm run after it
on the same machine finds it and reports its error against it.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("solves/s + p50/p99 latency (FP32+refine batched vs plain FP64), 1 GB300, "
          "err≤1e-6")
# Correctors the 128^3 benchmark case takes to converge (solutionTolerance
# 1e-6), measured with the GPU path; the CPU sample is scaled to a full solve
# with it when the GPU run is not in the same process.
FULL_SOLVE_CORRECTORS_128 = 799


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_bytes(kind, n_cells, n_faces, n_bfaces, v, n_loc=0, split=False, slots=False):
    """Minimal DRAM bytes of one launch of a kernel kind (k = 3 columns,
    v = value bytes, 4-byte indices); the formulas follow the solve's
    scope table: SpMV nnz(v+i) + 4(N+1) + 2Nvk; one DIC sweep
    nnz_L(v+i) + 4(N+1) + Nv + 2Nvk (+ Nvk for the backward w.r sums).
    Fused processor-local iteration: loc_precond reads r and q and writes r
    and w (4Nvk) plus rD (Nv), the in-part table (n_loc entries of v + 2
    bytes) and, with generic tables, 4 bytes of row metadata per row;
    loc_spmv reads w, p_old and x, writes p_new, q and x (the pending
    iteration's x += alpha p: 6Nvk), plus the matrix nnz(v+i) + Nv +
    4(N+1); its split form (p-update pass with x, then SpMV on p_new) moves
    7Nvk."""
    N, F, B, k = n_cells, n_faces, n_bfaces, 3
    nnz_l = F
    if kind == "loc_precond":
        return 4 * N * v * k + N * v + n_loc * (v + 2) + (0 if slots else 4 * N)
    if kind == "loc_spmv":
        return (7 if split else 6) * N * v * k + 2 * F * (v + 4) + N * v + 4 * (N + 1)
    if kind == "sweep_fwd":
        return nnz_l * (v + 4) + 4 * (N + 1) + N * v + 2 * N * v * k
    if kind == "sweep_bwd":
        return nnz_l * (v + 4) + 4 * (N + 1) + N * v + 3 * N * v * k
    if kind == "spmv":
        return 2 * F * (v + 4) + N * v + 4 * (N + 1) + 2 * N * v * k
    if kind == "update":
        return 5 * N * v * k          # read x, p, q, r; write x, r (x, r in place)
    if kind == "p_update":
        return 3 * N * v * k
    if kind == "rhs":                  # FP64 fields: D, grad, sigma, face data, r, x
        return N * 8 * (3 + 9 + 6 + 3) + F * 8 * 6 + 2 * F * 8 + N * v * 6 + B * 8 * 10
    if kind == "post":
        return N * 8 * (3 + 3 + 6 + 9 + 6) + 2 * F * 4 + N * v * 3 + B * 8 * 30
    return None


def iteration_roofline(tot_ms, tot_n, n_cells, n_faces, n_bfaces, v, n_loc, split, slots, peak):
    """The fused PCG iteration as a whole: the algorithmic bytes of its two
    kernels (loc_precond, loc_spmv) over their summed average launch time,
    or None when the solve did not run them."""
    kinds = ("loc_precond", "loc_spmv")
    if not all(tot_n.get(k) for k in kinds):
        return None
    nbytes = sum(algorithmic_bytes(k, n_cells, n_faces, n_bfaces, v, n_loc, split, slots)
                 for k in kinds)
    us = sum(1000.0 * tot_ms[k] / tot_n[k] for k in kinds)
    achieved = nbytes / (us * 1e-6) / 1e9
    return {"kernels": list(kinds), "algorithmic_bytes": nbytes, "us": us,
            "achieved": achieved, "unit": "GB/s", "frac": achieved / peak if peak else None}


def load_traffic(workload):
    """Per-launch DRAM traffic from the committed ncu summary, if it covers
    this workload: lines '<kind> <bytes_per_launch> <workload>'."""
    path = os.path.join(ROOT, "profiles", "kernel_traffic.txt")
    out = {}
    try:
        with open(path) as f:
            for ln in f:
                parts = ln.split()
                if len(parts) >= 3 and not ln.startswith("#") and parts[2] == workload:
                    out[parts[0]] = float(parts[1])
    except OSError:
        pass
    return out


def build_case(n):
    from solids4foam_gb300.cases import cube_case
    return cube_case(n)


def cache_path(n):
    """Where the reference arm leaves its oracle result, for the GPU arm of
    the same run on the same machine to measure its error against."""
    d = os.environ.get("S4G_BENCH_CACHE") or os.path.join(tempfile.gettempdir(), "s4g_bench")
    return os.path.join(d, f"oracle_cube{n}_seed1_jitter0.2_blocks8.npz")


def oracle_case(n):
    """The benchmark case built by the oracle's own code (oracle/box_mesh.py:
    the same mesh, bit for bit, as the library's generator) with the same
    8^3-block decomposition: nothing of the product computes the CPU
    baseline's inputs."""
    from oracle.box_mesh import block_parts, box_mesh
    mesh = box_mesh(n, n, n, 1.0, 1.0, 1.0, 0.2, 1)
    top = int(mesh["patch_size"][5])
    bcs = [(1, None, None)] * 4 + [(0, None, None), (1, None, np.full(top, 10e6))]
    return mesh, bcs, block_parts(n, n, n, 8)


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as td
        td.init_process_group("gloo")
        dist = td
    return world, rank, local, dist


def barrier(dist):
    if dist:
        dist.barrier()


def whole_job_rate(dist, world, step_ms):
    """Replicas (weak scaling): every rank solves the same case, so the
    job's solves/s is world solves per the slowest rank's mean step.
    Returns (solves/s of the whole job, that step time in ms)."""
    ms_step = allmax(dist, statistics.mean(step_ms))
    return world * 1000.0 / ms_step, ms_step


def allmax(dist, x):
    if not dist:
        return x
    import torch
    t = torch.tensor([float(x)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def host_threads():
    return len(os.sched_getaffinity(0)) or 1


def cpu_sample(n, sample_s=20.0, threads=None):
    """The CPU oracle on the first correctors of the benchmark case, all host
    threads, the same decomposition as the GPU arm: (seconds per corrector,
    details).  A bounded sample, for a quick figure beside the GPU line."""
    from oracle import pyoracle
    threads = threads or host_threads()
    mesh, bcs, parts = oracle_case(n)
    _, _, _, pm = pyoracle.solve(mesh, bcs, dic_domain=parts, E=70e9, nu=0.33,
                                 n_threads=threads, max_seconds=sample_s, n_correctors=2000)
    return pm["seconds"] / pm["n_correctors"], {
        "cores": threads,
        "sample": (f"first {pm['n_correctors']} correctors of the same case ({pm['seconds']:.1f} s, "
                   f"{pm['total_lin_iters']} PCG iterations, DIC over the same 8^3-cell blocks)")}


def run_reference(args):
    """The reference arm: one full FP64 CPU solve of the benchmark case by the
    oracle (the restatement of the reference's solve; the reference needs an
    OpenFOAM installation that is not available), on all host threads, with
    the GPU arm's decomposition (DIC restricted to the same 8^3-cell
    blocks).  Its inputs come from the oracle's own generator.  One solve
    takes about 25 minutes on 16 Arm cores (about 800 correctors), so one
    step is timed, whatever --steps asks; a
    solve that passes --ref-max-s is reported as an estimate, marked so."""
    world, rank, local, dist = dist_init()
    if rank != 0:
        return
    from oracle import pyoracle
    threads = host_threads()
    mesh, bcs, parts = oracle_case(args.n)
    D, sig, _, pm = pyoracle.solve(mesh, bcs, dic_domain=parts, E=70e9, nu=0.33,
                                   n_threads=threads, n_correctors=2000,
                                   max_seconds=args.ref_max_s)
    complete = pm["converged"] == 1 or pm["n_correctors"] >= 2000
    if complete:
        secs = pm["seconds"]
        sample = (f"one full solve: {pm['n_correctors']} correctors, {pm['total_lin_iters']} PCG "
                  f"iterations, converged {pm['converged']}, DIC over the same 8^3-cell blocks")
    else:
        secs = pm["seconds"] / pm["n_correctors"] * args.full_correctors
        sample = (f"ESTIMATE: stopped after {pm['n_correctors']} correctors ({pm['seconds']:.0f} s), "
                  f"scaled to {args.full_correctors} correctors")
    try:
        os.makedirs(os.path.dirname(cache_path(args.n)), exist_ok=True)
        if complete:
            np.savez(cache_path(args.n), D=D, sigma=sig, n_correctors=pm["n_correctors"],
                     pcg=pm["total_lin_iters"], seconds=pm["seconds"], threads=threads)
    except OSError:
        pass
    value = 1.0 / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
        "n_gpus": 1, "steps": 1, "warmup": 0, "steps_requested": args.steps,
        "ms_per_step": 1000.0 * secs, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"cube{args.n}_jittered_linear_elastic", "cells": args.n ** 3,
                   "model": "linearGeometryTotalDisplacement", "precision": "FP64",
                   "dic": "blocks8 (4096 subdomains at 128^3)", "complete_solve": complete,
                   "same_config_as_gpu_arm": "same mesh, loads, controls and DIC subdomains; "
                   "FP64 throughout (the GPU headline runs FP32+refine, its plain_fp64 leg FP64)",
                   "note": "CPU FP64 oracle (restatement of the reference's solve; the reference "
                           "itself needs OpenFOAM, which is not installed); inputs from the "
                           "oracle's own mesh generator"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def leg(run):
    """An optional leg beside the headline: a failure is reported in its
    place in the JSON line (with the library's message) instead of ending
    the run."""
    try:
        return run()
    except Exception as e:
        return {"error": f"{type(e).__name__}: {e}"}


class Budget:
    """Wall-clock guard of the optional legs, so that a run stays inside
    the time it is given."""

    def __init__(self, seconds):
        self.t0 = time.perf_counter()
        self.seconds = seconds

    def left(self):
        return self.seconds - (time.perf_counter() - self.t0)


def oracle_check_small(args, threads):
    """The headline case's form at 32^3 against the oracle in this process:
    FP32+refine and plain FP64 on the GPU, the oracle with the same blocks.
    Stands in for the 128^3 comparison when the reference arm's result is
    not on this machine."""
    import solids4foam_gb300 as sg
    from oracle import pyoracle
    mesh, bcs_o, parts = oracle_case(32)
    Do, so, _, po = pyoracle.solve(mesh, bcs_o, dic_domain=parts, E=70e9, nu=0.33,
                                   n_threads=threads, n_correctors=2000)
    c = build_case(32)
    ctx = sg.Context(0)
    out = {"workload": "cube32 (same form, same 8^3 blocks)", "oracle_correctors": po["n_correctors"]}
    for prec in ("FP32_REFINE", "FP64"):
        m = sg.SolidModel(ctx, c["mesh"], c["law"], c["bcs"], solver=c["solver"], outer=c["outer"],
                          precision=prec, parts=c["parts"])
        D, sig, p = m.evolve()
        m.close()
        out[prec] = {"rel_l2_D": rel_l2(D, Do), "rel_l2_sigma": rel_l2(sig, so),
                     "correctors": p["n_correctors"]}
    ctx.close()
    return out


def run_batched(args, ctx, budget):
    """Batched load cases (one 64^3 mesh, 64 cases, FP32+refine, one
    s4g_solve_cases call) against plain FP64 single solves of the same cases
    one after another; both over the same 8^3-cell blocks.  Case 0 is also
    checked against the oracle."""
    import solids4foam_gb300 as sg
    from solids4foam_gb300.cases import load_cases
    lc = load_cases(args.batch_n, args.batch_cases)
    cases = lc["cases"]
    kw = dict(solver=lc["solver"], outer=lc["outer"], parts=lc["parts"])
    model = sg.SolidModel(ctx, lc["mesh"], lc["law"], cases[0], precision="FP32_REFINE", **kw)
    model.evolve_cases(cases[:2])  # warm-up: tuning, FP32 copies
    t0 = time.perf_counter()
    Db, sb, perfs = model.evolve_cases(cases)
    wall = time.perf_counter() - t0
    model.close()
    dev_s = perfs[0]["solve_ms"] / 1e3
    n64 = min(args.batch_fp64_cases, len(cases))
    m64 = sg.SolidModel(ctx, lc["mesh"], lc["law"], cases[0], precision="FP64", **kw)
    m64.evolve()  # warm-up
    t64, errD, errS = [], [], []
    for c in range(n64):
        for name, spec in cases[c].items():
            m64.set_bc(["xmin", "xmax", "ymin", "ymax", "zmin", "zmax"].index(name), *spec)
        t1 = time.perf_counter()
        D64, s64, p64 = m64.evolve()
        t64.append(time.perf_counter() - t1)
        errD.append(rel_l2(Db[c], D64))
        errS.append(rel_l2(sb[c], s64))
    m64.close()
    fp64_rate = 1.0 / statistics.mean(t64)
    rate = len(cases) / wall
    out = {"workload": f"cube{args.batch_n}_x{len(cases)}_load_cases", "cases": len(cases),
           "cells": int(lc["mesh"]["V"].shape[0]), "dic": "blocks8", "solves_per_s": rate,
           "wall_s": wall, "device_s": dev_s,
           "correctors_min_max": [min(p["n_correctors"] for p in perfs),
                                  max(p["n_correctors"] for p in perfs)],
           "all_converged": all(p["converged"] == 1 for p in perfs),
           "plain_fp64_solves_per_s": fp64_rate, "plain_fp64_cases_timed": n64,
           "speedup_vs_plain_fp64": rate / fp64_rate,
           "max_rel_l2_D_vs_fp64": max(errD), "max_rel_l2_sigma_vs_fp64": max(errS)}
    if args.batch_oracle_cases > 0 and budget.left() > 400:
        from oracle import pyoracle
        from oracle.box_mesh import block_parts, box_mesh
        n = args.batch_n
        mo = box_mesh(n, n, n, 1.0, 1.0, 1.0, 0.2, 2)
        top = int(mo["patch_size"][5])
        errs = []
        for c in range(min(args.batch_oracle_cases, len(cases))):
            bo = [(1, None, None)] * 4 + [(0, None, None),
                                          (1, np.tile(lc["loads"][c], (top, 1)), None)]
            Do, so, _, po = pyoracle.solve(mo, bo, dic_domain=block_parts(n, n, n, 8), E=200e9,
                                           nu=0.3, n_threads=host_threads(), n_correctors=2000)
            errs.append((rel_l2(Db[c], Do), rel_l2(sb[c], so)))
        out["oracle_cases_checked"] = len(errs)
        out["max_rel_l2_D_vs_oracle"] = max(e[0] for e in errs)
        out["max_rel_l2_sigma_vs_oracle"] = max(e[1] for e in errs)
    return out


def run_served(args, budget):
    """The served stream of config form 4 (Poisson arrivals; 80% linear
    elastic, 20% neoHookean total Lagrangian over 10 increments; jittered
    boxes of 8^3-96^3 cells; FP32+refine over 8^3-cell blocks) through the
    server, against the same requests solved one after another in plain
    FP64.  Requests of up to --serve-oracle-cells cells are also checked
    against the oracle."""
    import solids4foam_gb300 as sg
    from solids4foam_gb300.cases import oracle_bcs, served_stream
    stream = served_stream(args.serve_n, tl_fraction=args.serve_tl_fraction)
    srv = sg.Server(max_slots=args.serve_slots)
    t0 = time.perf_counter()
    ids = []
    for arrival, req in stream:
        wait = arrival - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        kw = dict(req)
        kw["precision"] = "FP32_REFINE"
        ids.append(srv.submit(**kw))
    results = [srv.result(i) for i in ids]
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    n = len(stream)
    out = {"workload": f"stream{n}_poisson_boxes_8^3-96^3",
           "neoHookean_fraction": args.serve_tl_fraction,
           "neoHookean_requests": sum(1 for _, r in stream if "model" in r),
           "requests": n, "slots": args.serve_slots, "solves_per_s": n / wall,
           "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"],
           "all_converged": all(r[0] == 0 for r in results),
           "statuses": [int(r[0]) for r in results]}
    # plain FP64, one request after another
    if budget.left() > 2.5 * wall + 60:
        ctx = sg.Context(0)
        seq, errs = 0.0, []
        for (arrival, req), res in zip(stream, results):
            kw = dict(req)
            n_inc = kw.pop("n_increments", 1)
            m = sg.SolidModel(ctx, kw.pop("mesh"), kw.pop("law"), kw.pop("bcs"), precision="FP64",
                              **kw)
            t1 = time.perf_counter()
            D, sig, perf = m.evolve(n_increments=n_inc)
            seq += time.perf_counter() - t1
            m.close()
            errs.append(rel_l2(res[1], D))
        ctx.close()
        out.update({"plain_fp64_sequential_solves_per_s": n / seq,
                    "speedup_vs_plain_fp64_sequential": (n / wall) / (n / seq),
                    "max_rel_l2_D_vs_fp64": max(errs)})
    else:
        out["plain_fp64_sequential"] = "skipped: not enough of the run's time budget left"
    if args.serve_oracle_cells > 0 and budget.left() > 120:
        from oracle import pyoracle
        errs = []
        for (arrival, req), res in zip(stream, results):
            m = req["mesh"]
            if m["V"].shape[0] > args.serve_oracle_cells:
                continue
            law, o = req["law"], req["outer"]
            kw = dict(n_correctors=o["nCorrectors"], field_relaxation=o.get("fieldRelaxation", 1.0),
                      solution_tol=o.get("solutionTolerance", 1e-6),
                      alternative_tol=o.get("alternativeTolerance", 1e-7),
                      n_threads=host_threads(), dic_domain=req["parts"])
            if law["type"] == "linearElastic":
                kw.update(E=law["E"], nu=law["nu"])
            else:
                kw.update(model=1, law=1, use_mu_K=1, mu=law["mu"], K=law["K"],
                          n_increments=req["n_increments"])
            Do, so, _, po = pyoracle.solve(m, oracle_bcs(m, req["bcs"]), **kw)
            errs.append((rel_l2(res[1], Do), rel_l2(res[2], so)))
        if errs:
            out["oracle_requests_checked"] = len(errs)
            out["max_rel_l2_D_vs_oracle"] = max(e[0] for e in errs)
            out["max_rel_l2_sigma_vs_oracle"] = max(e[1] for e in errs)
    return out


def run_mesh_batch(args, budget):
    """Many meshes in one launch (config form 3b): --mbatch-n jittered boxes
    of 10-48 cells per edge with near-cubic cells and aspect ratios 1-2 (the
    segregated loop runs away on more slender boxes), E and nu drawn per mesh,
    FP32+refine over 8^3-cell blocks, all advanced by one s4g_solve_batch
    call (one CUDA-graph launch).  Against plain FP64 single solves of the
    first --mbatch-fp64 meshes one after another, and the smallest mesh
    against the oracle."""
    import solids4foam_gb300 as sg
    from solids4foam_gb300.cases import mesh_batch, oracle_bcs
    cases = mesh_batch(args.mbatch_n)
    ctx = sg.Context(0)
    models = [sg.SolidModel(ctx, c["mesh"], c["law"], c["bcs"], outer=c["outer"],
                            precision="FP32_REFINE", parts=c["parts"]) for c in cases]
    sg.solve_batch(models)  # warm-up: tuning, FP32 copies, graph set-up
    t0 = time.perf_counter()
    res = sg.solve_batch(models)
    wall = time.perf_counter() - t0
    for m in models:
        m.close()
    n = len(cases)
    out = {"workload": f"batch{n}_boxes_10-48_per_edge", "meshes": n,
           "cells": int(sum(c["mesh"]["V"].shape[0] for c in cases)),
           "solves_per_s": n / wall, "wall_s": wall, "device_s": res[0][2]["solve_ms"] / 1e3,
           "all_converged": all(r[2]["converged"] == 1 for r in res),
           "correctors_min_max": [min(r[2]["n_correctors"] for r in res),
                                  max(r[2]["n_correctors"] for r in res)]}
    k = min(args.mbatch_fp64, n)
    if k and budget.left() > 200:
        seq, errs = 0.0, []
        for i in range(k):
            c = cases[i]
            m = sg.SolidModel(ctx, c["mesh"], c["law"], c["bcs"], outer=c["outer"], precision="FP64",
                              parts=c["parts"])
            t1 = time.perf_counter()
            D, sig, p = m.evolve()
            seq += time.perf_counter() - t1
            m.close()
            errs.append(rel_l2(res[i][0], D))
        out.update({"plain_fp64_sequential_solves_per_s": k / seq, "plain_fp64_meshes_timed": k,
                    "speedup_vs_plain_fp64_sequential": (n / wall) / (k / seq),
                    "max_rel_l2_D_vs_fp64": max(errs)})
    if budget.left() > 120:
        from oracle import pyoracle
        i = min(range(n), key=lambda j: cases[j]["mesh"]["V"].shape[0])
        c = cases[i]
        Do, so, _, po = pyoracle.solve(c["mesh"], oracle_bcs(c["mesh"], c["bcs"]),
                                       dic_domain=c["parts"], E=c["law"]["E"], nu=c["law"]["nu"],
                                       n_correctors=c["outer"]["nCorrectors"],
                                       field_relaxation=c["outer"].get("fieldRelaxation", 1.0),
                                       solution_tol=c["outer"].get("solutionTolerance", 1e-6),
                                       alternative_tol=c["outer"].get("alternativeTolerance", 1e-7),
                                       n_threads=host_threads())
        out["oracle_mesh_checked"] = {"cells": int(c["mesh"]["V"].shape[0]),
                                      "rel_l2_D": rel_l2(res[i][0], Do),
                                      "rel_l2_sigma": rel_l2(res[i][1], so)}
    ctx.close()
    return out


def model_kwargs(case, args):
    kw = dict(solver=case["solver"], outer=case["outer"], precision=args.precision)
    if args.dic == "blocks":
        kw["parts"] = case["parts"]
    elif args.dic == "library":
        kw["dic_subdomains"] = True
    return kw


def run_gb300(args):
    import solids4foam_gb300 as sg
    budget = Budget(args.budget_s)
    world, rank, local, dist = dist_init()
    case = build_case(args.n)
    mesh = case["mesh"]
    kw = model_kwargs(case, args)
    # the production path: CUDA graphs on, no per-kernel events
    ctx = sg.Context(local, graphs=not args.no_graphs)
    model = sg.SolidModel(ctx, mesh, case["law"], case["bcs"], **kw)
    for _ in range(args.warmup):
        model.evolve()
    sampler = ClockSampler(local)
    sampler.start()
    barrier(dist)
    perfs = []
    tw0 = time.perf_counter()
    for _ in range(args.steps):
        D, sig, perf = model.evolve()
        perfs.append(perf)
    wall_steps = time.perf_counter() - tw0
    barrier(dist)
    clocks = sampler.stop()
    ms = [p["solve_ms"] for p in perfs]
    value, ms_step = whole_job_rate(dist, world, ms)

    # end to end through the C ABI with host buffers: upload, solve, download
    e2e_ms = []
    h2d = sum(np.asarray(mesh[k]).nbytes for k in ("owner", "neighbour", "C", "V", "Cf", "Sf",
                                                     "patch_start", "patch_size"))
    h2d += sum(np.asarray(v).nbytes for _, v, p in case["bcs"].values() if v is not None)
    h2d += sum(np.asarray(p).nbytes for _, v, p in case["bcs"].values() if p is not None)
    if "parts" in kw:
        h2d += kw["parts"].nbytes
    d2h = mesh["V"].shape[0] * 8 * (3 + 6)
    for _ in range(args.e2e_steps):
        barrier(dist)
        t0 = time.perf_counter()
        m2 = sg.SolidModel(ctx, mesh, case["law"], case["bcs"], **kw)
        m2.evolve()
        m2.close()
        e2e_ms.append(1000.0 * (time.perf_counter() - t0))
    e2e_step = whole_job_rate(dist, world, e2e_ms)[1] if e2e_ms else None

    # per-kernel CUDA events of one more solve, launched kernel by kernel
    ctxp = sg.Context(local, profile=True)
    mp = sg.SolidModel(ctxp, mesh, case["law"], case["bcs"], **kw)
    _, _, pp = mp.evolve()
    v = 8 if args.precision == "FP64" else 4
    nC, nI = mesh["V"].shape[0], mesh["neighbour"].shape[0]
    nB = mesh["owner"].shape[0] - nI
    tot_ms, tot_n = pp["kernel_ms"], pp["kernel_launches_by"]
    dom = max(tot_ms, key=lambda k: tot_ms[k])
    peak, peak_kind = peaks()
    avg_ms = tot_ms[dom] / max(1, tot_n[dom])
    n_loc = mp.info()["n_local_entries"]
    slots = bool(mp.info()["local_slots"])
    split = pp["spmv_unroll"] == 0 and pp["part_threads"] > 0
    mp.close()
    ctxp.close()
    ab = algorithmic_bytes(dom, nC, nI, nB, v, n_loc, split, slots)
    achieved = ab / (avg_ms * 1e-3) / 1e9 if ab else None
    workload = f"cube{args.n}_{args.precision.lower()}_{args.dic}"
    traffic = load_traffic(workload).get(dom)
    kernels = {k: {"launches": tot_n[k], "ms_total": round(tot_ms[k], 3),
                   "share": round(tot_ms[k] / max(1e-9, sum(tot_ms.values())), 4),
                   "avg_us": round(1000 * tot_ms[k] / max(1, tot_n[k]), 2),
                   "gbs": (round(algorithmic_bytes(k, nC, nI, nB, v, n_loc, split, slots) /
                                 (tot_ms[k] / max(1, tot_n[k]) * 1e-3) / 1e9, 1)
                           if tot_n[k] and algorithmic_bytes(k, nC, nI, nB, v, n_loc, split, slots)
                           else None)}
               for k in tot_ms if tot_n[k]}

    # plain FP64 solve of the same case, for the FP32+refine comparison
    fp64 = None
    D64 = s64 = None
    if args.precision != "FP64" and not args.no_fp64:
        kw64 = dict(kw, precision="FP64")
        m64 = sg.SolidModel(ctx, mesh, case["law"], case["bcs"], **kw64)
        D64, s64, p64 = m64.evolve()
        m64.close()
        fp64 = {"solves_per_s": 1000.0 / p64["solve_ms"], "ms_per_solve": p64["solve_ms"],
                "n_correctors": p64["n_correctors"], "pcg_iterations": p64["total_lin_iters"],
                "speedup_of_fp32_refine": p64["solve_ms"] / ms_step,
                "rel_l2_D_fp32_vs_fp64": rel_l2(D, D64), "rel_l2_sigma_fp32_vs_fp64": rel_l2(sig, s64)}

    # error against the FP64 oracle: the reference arm's full solve when it
    # ran on this machine before this arm, else the same form at 32^3
    parity = None
    if rank == 0:
        cp = cache_path(args.n)
        if os.path.exists(cp):
            ref = np.load(cp)
            parity = {"against": "the reference arm's full oracle solve of this case",
                      "oracle_correctors": int(ref["n_correctors"]),
                      "rel_l2_D": rel_l2(D, ref["D"]), "rel_l2_sigma": rel_l2(sig, ref["sigma"])}
            if D64 is not None:
                parity["plain_fp64"] = {"rel_l2_D": rel_l2(D64, ref["D"]),
                                        "rel_l2_sigma": rel_l2(s64, ref["sigma"])}
        elif not args.no_cpu and budget.left() > 300:
            parity = oracle_check_small(args, host_threads())

    # the legs in the order the metric names them: batched load cases, the
    # served stream (its p50/p99 latency), then the many-mesh batch
    batched = (leg(lambda: run_batched(args, ctx, budget))
               if (rank == 0 and not args.no_batched and budget.left() > 300) else None)
    served = (leg(lambda: run_served(args, budget))
              if (rank == 0 and not args.no_served and budget.left() > 300) else None)
    mbatch = (leg(lambda: run_mesh_batch(args, budget))
              if (rank == 0 and not args.no_mbatch and budget.left() > 300) else None)

    n_parts = int(model.info()["n_parts"])
    cpu = None
    if rank == 0 and not args.no_cpu:
        cp = cache_path(args.n)
        if os.path.exists(cp):
            ref = np.load(cp)
            cpu = {"value": 1.0 / float(ref["seconds"]), "unit": "solves/s",
                   "cores": int(ref["threads"]), "kind": "port",
                   "sample": f"the reference arm's full solve in this run ({int(ref['n_correctors'])} "
                             f"correctors, DIC over the same 8^3-cell blocks)"}
        else:
            spc, info = cpu_sample(args.n, sample_s=args.cpu_sample_s)
            cpu = {"value": 1.0 / (spc * perfs[0]["n_correctors"]), "unit": "solves/s",
                   "cores": info["cores"], "kind": "port",
                   "sample": info["sample"] + f", scaled to this solve's "
                             f"{perfs[0]['n_correctors']} correctors (estimate)"}
    ctx.close()
    if rank != 0:
        return
    p0 = perfs[0]
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "FP64" else "f32+f64",
        "data": "synthetic",
        "config": {"workload": workload, "cells": nC, "internal_faces": nI,
                   "model": "linearGeometryTotalDisplacement", "law": "linearElastic",
                   "solver": "PCG+DIC tol 1e-9 relTol 0.1", "outer": "solutionTolerance 1e-6, "
                   "nCorrectors 2000", "precision": args.precision, "dic": args.dic,
                   "dic_subdomains": n_parts if args.dic != "exact" else 1,
                   "parallelism": f"replicas{world}", "path": "production (CUDA graphs, no "
                   "per-kernel events); kernels/roofline from one profiled solve in this run",
                   "l2": "working set ~1.7 GB >> 129 MB L2 (no flush needed)",
                   "n_correctors": p0["n_correctors"], "converged": p0["converged"],
                   "autotuned": {"part_threads": p0["part_threads"],
                                 "spmv": ("split" if p0["spmv_unroll"] == 0 else
                                          f"fused, unroll {p0['spmv_unroll']}")},
                   "pcg_iterations": p0["total_lin_iters"],
                   "wall_s_of_timed_steps": wall_steps},
        "e2e": {"value": (world * 1000.0 / e2e_step) if e2e_step else None, "unit": "solves/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(sum(p["kernel_launches"] for p in perfs)),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                     "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_launch": ab, "avg_launch_us": avg_ms * 1000,
                     "pcg_iteration": iteration_roofline(tot_ms, tot_n, nC, nI, nB, v, n_loc,
                                                         split, slots, peak)},
        "kernels": kernels,
        "error_vs_oracle": parity,
        "plain_fp64": fp64,
        "batched": batched,
        "mesh_batch": mbatch,
        "served": served,
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    model.close()
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="FP32_REFINE", choices=["FP64", "FP32_REFINE"])
    ap.add_argument("--dic", default="blocks", choices=["blocks", "library", "exact"],
                    help="DIC subdomains: 8^3-cell blocks (a decomposed run's processors), "
                         "the library's own parts, or the exact global DIC")
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the plain-FP64 comparison solve")
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--cpu-sample-s", type=float, default=20.0)
    ap.add_argument("--full-correctors", type=int, default=FULL_SOLVE_CORRECTORS_128)
    ap.add_argument("--ref-max-s", type=float, default=1700.0,
                    help="reference arm: wall time after which the CPU solve stops and is "
                         "reported as an estimate")
    ap.add_argument("--budget-s", type=float, default=1500.0,
                    help="wall time the optional legs of the GPU arm may take in all")
    ap.add_argument("--no-graphs", action="store_true",
                    help="host-driven corrector loop, kernel by kernel (for profilers)")
    ap.add_argument("--no-profiled-solve", action="store_true",
                    help="skip the solve with per-kernel events (no kernels/roofline)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched load cases")
    ap.add_argument("--batch-n", type=int, default=64)
    ap.add_argument("--batch-cases", type=int, default=64)
    ap.add_argument("--batch-fp64-cases", type=int, default=3,
                    help="plain FP64 single solves timed for the batched comparison")
    ap.add_argument("--batch-oracle-cases", type=int, default=1,
                    help="batched cases also checked against the oracle")
    ap.add_argument("--no-mbatch", action="store_true", help="skip the many-mesh batch")
    ap.add_argument("--mbatch-n", type=int, default=256)
    ap.add_argument("--mbatch-fp64", type=int, default=16,
                    help="meshes of the batch solved one by one in plain FP64 for the comparison")
    ap.add_argument("--no-served", action="store_true", help="skip the served stream")
    ap.add_argument("--serve-n", type=int, default=24)
    ap.add_argument("--serve-slots", type=int, default=8)
    ap.add_argument("--serve-tl-fraction", type=float, default=0.2,
                    help="share of neoHookean total Lagrangian requests in the stream")
    ap.add_argument("--serve-oracle-cells", type=int, default=25000,
                    help="served requests up to this many cells are checked against the oracle")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
