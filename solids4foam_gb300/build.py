"""Builds libs4g.so in-tree (solids4foam_gb300/_build/) with nvcc for sm_103a,
and the standalone C++ driver s4g_solve_case linked against it.

Translation units compile in parallel; the CUDA runtime is linked
statically, so the library only needs the NVIDIA driver at run time.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libs4g.so")
DRIVER_SRC = os.path.join(HERE, "driver", "s4g_solve_case.cpp")
DRIVER = os.path.join(OUT, "s4g_solve_case")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code rounds every double operation on its own (no fused multiply-add
# contraction), so host results are the same on x86-64 and aarch64.
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", os.path.join(ROOT, "include"), "-I", SRC]
CU_FLAGS = ARCH + ["-lineinfo", "--expt-relaxed-constexpr"] + COMMON
CXX_FLAGS = COMMON


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(SRC) if f.endswith((".cu", ".cpp")))


def _compile(nvcc: str, src: str, extra: list[str]) -> str:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    flags = CU_FLAGS if src.endswith(".cu") else CXX_FLAGS
    cmd = [nvcc] + flags + extra + ["-c", os.path.join(SRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)]
    deps.append(os.path.join(ROOT, "include", "s4g.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build_driver(force: bool = False) -> str:
    """The standalone driver, linked to libs4g.so with an $ORIGIN rpath."""
    if (not force and os.path.exists(DRIVER)
            and all(os.path.getmtime(DRIVER) >= os.path.getmtime(d)
                    for d in (DRIVER_SRC, LIB, os.path.join(ROOT, "include", "s4g.h")))):
        return DRIVER
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("no C++ compiler for the driver")
    cmd = [cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), DRIVER_SRC,
           "-L", OUT, "-ls4g", "-Wl,-rpath,$ORIGIN", "-o", DRIVER + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(DRIVER + ".tmp", DRIVER)
    return DRIVER


def _try_driver(force: bool) -> None:
    """The driver is an extra beside the library: a failure to build it is
    reported, not raised (its own tests then fail)."""
    try:
        build_driver(force=force)
    except (RuntimeError, OSError) as e:
        print(f"warning: s4g_solve_case not built: {e}", file=sys.stderr)


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    if not force and not _stale():
        _try_driver(False)
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, extra), sources()))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    _try_driver(True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
