"""ctypes binding of the CPU FP64 oracle (oracle/s4g_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by the tests, the smoke check and the CPU
baseline leg of the benchmark, never by the product package.

A mesh is a dict of numpy arrays with the keys of ``s4g_mesh_desc``:
owner, neighbour, C, V, Cf, Sf, patch_start, patch_size (and n_cells,
n_internal_faces).  Boundary conditions are a list, one entry per patch:
``(type, value[size,3] or None, pressure[size] or None)`` with type 0 =
fixedDisplacement, 1 = solidTraction.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libs4g_oracle.so")

FIXED_DISPLACEMENT = 0
SOLID_TRACTION = 1
LINEAR_ELASTIC = 0
NEO_HOOKEAN = 1
LIN_GEOM_TOTAL_DISP = 0
NONLIN_GEOM_TOTAL_LAG = 1
DIC = 0
DIAGONAL = 1


class MeshDesc(ct.Structure):
    _fields_ = [
        ("n_cells", ct.c_int), ("n_faces", ct.c_int), ("n_internal_faces", ct.c_int),
        ("owner", ct.c_void_p), ("neighbour", ct.c_void_p),
        ("C", ct.c_void_p), ("V", ct.c_void_p), ("Cf", ct.c_void_p), ("Sf", ct.c_void_p),
        ("n_patches", ct.c_int), ("patch_start", ct.c_void_p), ("patch_size", ct.c_void_p),
    ]


class Bc(ct.Structure):
    _fields_ = [("type", ct.c_int), ("value", ct.c_void_p), ("pressure", ct.c_void_p),
                ("relaxation_factor", ct.c_double)]


class Settings(ct.Structure):
    _fields_ = [
        ("model", ct.c_int), ("law", ct.c_int),
        ("E", ct.c_double), ("nu", ct.c_double), ("mu", ct.c_double), ("K", ct.c_double),
        ("use_mu_K", ct.c_int), ("preconditioner", ct.c_int),
        ("tolerance", ct.c_double), ("rel_tol", ct.c_double), ("max_iter", ct.c_int),
        ("n_correctors", ct.c_int),
        ("solution_tol", ct.c_double), ("alternative_tol", ct.c_double),
        ("material_tol", ct.c_double), ("stab_scale", ct.c_double),
        ("ls_boundary_delta", ct.c_int), ("n_increments", ct.c_int),
        ("n_threads", ct.c_int), ("max_correctors_run", ct.c_int),
        ("dic_domain", ct.c_void_p), ("max_seconds", ct.c_double),
        ("empty_direction", ct.c_int), ("field_relaxation", ct.c_double),
        ("relaxation_method", ct.c_int),
    ]


class Perf(ct.Structure):
    _fields_ = [
        ("n_correctors", ct.c_int), ("converged", ct.c_int),
        ("total_lin_iters", ct.c_longlong), ("initial_residual", ct.c_double),
        ("rel_residual", ct.c_double), ("seconds", ct.c_double),
        ("enforce_linear", ct.c_int), ("nan_detected", ct.c_int),
    ]


_lib = None


def build(force: bool = False) -> str:
    """Compiles the oracle with its Makefile (gcc, a few seconds)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ct.CDLL(_LIB_PATH)
        _lib.orc_solve.restype = ct.c_int
        _lib.orc_solve.argtypes = [ct.POINTER(MeshDesc), ct.POINTER(Bc), ct.POINTER(Settings),
                                   ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                   ct.POINTER(Perf)]
        _lib.orc_default_settings.argtypes = [ct.POINTER(Settings)]
        for fn in ("orc_amul", "orc_dic_precondition"):
            getattr(_lib, fn).restype = ct.c_int
        _lib.orc_assemble_matrix.argtypes = [ct.POINTER(MeshDesc), ct.POINTER(Bc), ct.c_double,
                                             ct.c_void_p, ct.c_void_p]
        _lib.orc_amul.argtypes = [ct.POINTER(MeshDesc)] + [ct.c_void_p] * 4
        _lib.orc_dic_precondition.argtypes = [ct.POINTER(MeshDesc)] + [ct.c_void_p] * 4
        _lib.orc_ls_grad.argtypes = [ct.POINTER(MeshDesc), ct.c_int] + [ct.c_void_p] * 5
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def _desc(mesh, keep):
    arrs = {}
    for k, dt in (("owner", np.int32), ("neighbour", np.int32), ("C", np.float64),
                  ("V", np.float64), ("Cf", np.float64), ("Sf", np.float64),
                  ("patch_start", np.int32), ("patch_size", np.int32)):
        arrs[k] = np.ascontiguousarray(mesh[k], dtype=dt)
    keep.append(arrs)
    d = MeshDesc()
    d.n_cells = int(arrs["V"].shape[0])
    d.n_faces = int(arrs["owner"].shape[0])
    d.n_internal_faces = int(arrs["neighbour"].shape[0])
    d.n_patches = int(arrs["patch_start"].shape[0])
    for k in arrs:
        setattr(d, k, _ptr(arrs[k]))
    return d


def _bcs(bcs, mesh, keep):
    arr = (Bc * len(bcs))()
    for i, (t, v, p, *rest) in enumerate(bcs):
        v2 = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        p2 = None if p is None else np.ascontiguousarray(p, dtype=np.float64)
        keep.append((v2, p2))
        arr[i].type = int(t)
        arr[i].value = _ptr(v2)
        arr[i].pressure = _ptr(p2)
        arr[i].relaxation_factor = float(rest[0]) if rest else 1.0
    return arr


def default_settings(**kw) -> Settings:
    s = Settings()
    lib().orc_default_settings(ct.byref(s))
    for k, v in kw.items():
        if not hasattr(s, k):
            raise KeyError(k)
        setattr(s, k, v)
    return s


def solve(mesh, bcs, settings: Settings | None = None, perm=None, dic_domain=None, **kw):
    """Full oracle solve.  Returns (D [n,3], sigma [n,6], gradD [n,9], perf dict).
    dic_domain (optional, caller cell order): DIC restricted to subdomains."""
    s = settings if settings is not None else default_settings(**kw)
    keep = []
    if dic_domain is not None:
        dd = np.ascontiguousarray(dic_domain, dtype=np.int32)
        keep.append(dd)
        s.dic_domain = dd.ctypes.data
    d = _desc(mesh, keep)
    b = _bcs(bcs, mesh, keep)
    n = d.n_cells
    D = np.zeros((n, 3))
    sig = np.zeros((n, 6))
    G = np.zeros((n, 9))
    perm_a = None if perm is None else np.ascontiguousarray(perm, dtype=np.int32)
    perf = Perf()
    rc = lib().orc_solve(ct.byref(d), b, ct.byref(s), _ptr(perm_a), _ptr(D), _ptr(sig),
                         _ptr(G), ct.byref(perf))
    if rc != 0:
        raise RuntimeError(f"orc_solve failed with code {rc}")
    pd = {f[0]: getattr(perf, f[0]) for f in Perf._fields_}
    return D, sig, G, pd


def matrix(mesh, bcs, impK):
    keep = []
    d = _desc(mesh, keep)
    b = _bcs(bcs, mesh, keep)
    diag = np.zeros(d.n_cells)
    upper = np.zeros(d.n_internal_faces)
    rc = lib().orc_assemble_matrix(ct.byref(d), b, float(impK), _ptr(diag), _ptr(upper))
    if rc != 0:
        raise RuntimeError(rc)
    return diag, upper


def amul(mesh, diag, upper, x):
    keep = []
    d = _desc(mesh, keep)
    diag = np.ascontiguousarray(diag, dtype=np.float64)
    upper = np.ascontiguousarray(upper, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    lib().orc_amul(ct.byref(d), _ptr(diag), _ptr(upper), _ptr(x), _ptr(y))
    return y


def dic(mesh, diag, upper, r):
    keep = []
    d = _desc(mesh, keep)
    diag = np.ascontiguousarray(diag, dtype=np.float64)
    upper = np.ascontiguousarray(upper, dtype=np.float64)
    r = np.ascontiguousarray(r, dtype=np.float64)
    w = np.zeros_like(r)
    lib().orc_dic_precondition(ct.byref(d), _ptr(diag), _ptr(upper), _ptr(r), _ptr(w))
    return w


def ls_grad(mesh, D, Db, snGradB, ls_boundary_delta=0):
    keep = []
    d = _desc(mesh, keep)
    D = np.ascontiguousarray(D, dtype=np.float64)
    Db = np.ascontiguousarray(Db, dtype=np.float64)
    sg = np.ascontiguousarray(snGradB, dtype=np.float64)
    G = np.zeros((d.n_cells, 9))
    Gb = np.zeros((Db.shape[0], 9))
    lib().orc_ls_grad(ct.byref(d), int(ls_boundary_delta), _ptr(D), _ptr(Db), _ptr(sg),
                      _ptr(G), _ptr(Gb))
    return G, Gb


def renumber_mesh(mesh, perm):
    """Mesh in the solver numbering given by perm (new cell i = old perm[i]),
    faces re-sorted upper-triangular like OpenFOAM's renumberMesh."""
    perm = np.asarray(perm)
    n = perm.shape[0]
    new_of = np.empty(n, dtype=np.int64)
    new_of[perm] = np.arange(n)
    ni = mesh["neighbour"].shape[0]
    own = new_of[mesh["owner"]]
    nei = new_of[mesh["neighbour"]]
    o_i, n_i = own[:ni].copy(), nei.copy()
    flip = o_i > n_i
    lo = np.where(flip, n_i, o_i)
    hi = np.where(flip, o_i, n_i)
    sf = mesh["Sf"].copy()
    sf[:ni][flip] *= -1.0
    order = np.lexsort((hi, lo))
    out = dict(mesh)
    out["owner"] = np.concatenate([lo[order], own[ni:]]).astype(np.int32)
    out["neighbour"] = hi[order].astype(np.int32)
    out["Sf"] = np.concatenate([sf[:ni][order], sf[ni:]])
    out["Cf"] = np.concatenate([mesh["Cf"][:ni][order], mesh["Cf"][ni:]])
    out["C"] = mesh["C"][perm]
    out["V"] = mesh["V"][perm]
    out["face_order"] = order
    out["face_flip"] = flip[order]
    return out
