"""Host-side mirror of the reference's solidModel / mechanicalLaw interface.

A ``SolidModel`` is built from the same vocabulary as a solids4foam case:
the ``solidModel`` type name of constant/solidProperties
(``linearGeometryTotalDisplacement``, ``nonLinearGeometryTotalLagrangian`` or
``nonLinearGeometryTotalLagrangianTotalDisplacement``), a ``mechanical`` law
entry of constant/mechanicalProperties (``linearElastic`` with E/nu,
``neoHookeanElastic`` with E/nu or mu/K), the ``0/D`` patch types
``fixedDisplacement`` / ``solidTraction`` as ``(type, value or traction,
pressure[, relaxationFactor])`` tuples, the ``solvers { "D|DD" {...} }``
entry of system/fvSolution and the ``<model>Coeffs`` keys of
solidProperties.  A meshed OpenFOAM case reads into these arguments with
``foam_case.read_case``.  ``evolve()`` runs the model's
outer-corrector loop on the GPU through the C ABI (include/s4g.h), as
solidModel::evolve does in the reference (solidModel.H:759).

Errors raise S4GError, the counterpart of the reference's FatalError; a run
that reaches nCorrectors without converging returns its result and sets
``perf["converged"] = 0`` (the reference prints "Max iterations reached").
"""
from __future__ import annotations

import ctypes as ct
import weakref

import numpy as np

from . import _lib
from .cases import PATCHES

MODELS = {
    "linearGeometryTotalDisplacement": _lib.LIN_GEOM_TOTAL_DISP,
    "nonLinearGeometryTotalLagrangian": _lib.NONLIN_GEOM_TOTAL_LAG,
    "nonLinearGeometryTotalLagrangianTotalDisplacement": _lib.NONLIN_GEOM_TOTAL_LAG_TOTAL_DISP,
}
PRECONDITIONERS = {"DIC": _lib.PRECOND_DIC, "FDIC": _lib.PRECOND_DIC,
                   "diagonal": _lib.PRECOND_DIAGONAL}
RENUMBER = {"none": _lib.RENUMBER_NONE, "RCM": _lib.RENUMBER_RCM, "tiled": _lib.RENUMBER_TILED}


class Context:
    """One GPU (s4g_ctx)."""

    def __init__(self, device: int = 0, verbose: bool = False, profile: bool = False,
                 graphs: bool = True, spin_limit: int = 0):
        """spin_limit: polls a bounded device wait makes before it gives up
        and the solve returns S4G_TIMEOUT (0: the library's default)."""
        self.L = _lib.lib()
        h = ct.c_void_p()
        opts = _lib.CtxOpts(device, 1 if verbose else 0, 1 if profile else 0, 0 if graphs else 1,
                            int(spin_limit))
        _lib.check(self.L.s4g_ctx_create(ct.byref(h), ct.byref(opts)), "s4g_ctx_create")
        self.h = h
        self.models = weakref.WeakSet()

    def close(self):
        """Destroys the context; the library frees meshes still alive, and
        the Python models of those meshes are marked closed first."""
        if self.h:
            for m in list(self.models):
                m.h = None
            self.L.s4g_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _desc(mesh, keep):
    arrs = {}
    for k, dt in (("owner", np.int32), ("neighbour", np.int32), ("C", np.float64),
                  ("V", np.float64), ("Cf", np.float64), ("Sf", np.float64),
                  ("patch_start", np.int32), ("patch_size", np.int32)):
        arrs[k] = np.ascontiguousarray(mesh[k], dtype=dt)
    keep.append(arrs)
    d = _lib.MeshDesc()
    d.n_cells = arrs["V"].shape[0]
    d.n_faces = arrs["owner"].shape[0]
    d.n_internal_faces = arrs["neighbour"].shape[0]
    d.n_patches = arrs["patch_start"].shape[0]
    for k, a in arrs.items():
        setattr(d, k, a.ctypes.data)
    return d


def _law_struct(law: dict):
    """constant/mechanicalProperties: one linearElastic or neoHookeanElastic law."""
    t = law.get("type", "linearElastic")
    if t not in ("linearElastic", "neoHookeanElastic"):
        raise ValueError(f"unknown mechanical law {t!r}")
    use_muK = "mu" in law and "K" in law
    return _lib.Law(_lib.LINEAR_ELASTIC if t == "linearElastic" else _lib.NEO_HOOKEAN,
                    1 if use_muK else 0, float(law.get("E", 0.0)), float(law.get("nu", 0.0)),
                    float(law.get("mu", 0.0)), float(law.get("K", 0.0)),
                    float(law.get("rho", 1000.0)))


def _control_structs(L, solver: dict, outer: dict, precision: str = "FP64"):
    """system/fvSolution solvers { D } and solidProperties <model>Coeffs."""
    lin, out = _lib.LinSolver(), _lib.Outer()
    L.s4g_default_controls(ct.byref(lin), ct.byref(out))
    if "preconditioner" in solver:
        lin.preconditioner = PRECONDITIONERS[solver["preconditioner"]]
    lin.tolerance = solver.get("tolerance", lin.tolerance)
    lin.rel_tol = solver.get("relTol", lin.rel_tol)
    lin.max_iter = solver.get("maxIter", lin.max_iter)
    out.n_correctors = outer.get("nCorrectors", out.n_correctors)
    out.solution_tol = outer.get("solutionTolerance", out.solution_tol)
    out.alternative_tol = outer.get("alternativeTolerance", out.alternative_tol)
    out.material_tol = outer.get("materialTolerance", out.material_tol)
    out.info_frequency = outer.get("infoFrequency", out.info_frequency)
    # relaxationFactors { fields { D f; } } of fvSolution, and the
    # <model>Coeffs relaxationMethod
    out.field_relaxation = outer.get("fieldRelaxation", 1.0)
    method = outer.get("relaxationMethod", "fixed")
    if method not in ("fixed", "Aitken"):
        raise ValueError(f"unknown relaxationMethod {method!r}")
    out.relaxation_method = 0 if method == "fixed" else 1
    stab = outer.get("stabilisation", {"type": "RhieChow", "scaleFactor": 0.1})
    if stab.get("type", "RhieChow") != "RhieChow":
        raise ValueError("only RhieChow stabilisation is built")
    out.stab_scale = stab.get("scaleFactor", 0.1)
    prec = {"FP64": _lib.FP64, "FP32_REFINE": _lib.FP32_REFINE}[precision]
    return lin, out, prec


class SolidModel:
    """GPU drop-in for one solid region's outer-corrector loop."""

    def __init__(self, ctx: Context, mesh, law: dict, bcs: dict, model: str =
                 "linearGeometryTotalDisplacement", solver: dict | None = None,
                 outer: dict | None = None, precision: str = "FP64", renumber: str = "tiled",
                 part_size: int = 512, ls_boundary_delta: int = 0, dic_subdomains: bool = False,
                 autotune: bool = True, empty_direction: int = 0, parts=None):
        """empty_direction: 1, 2 or 3 for a 2-D case whose empty patches'
        faces the mesh leaves out (x, y or z empty; plane strain); 0: 3-D.
        parts: the caller's decomposition into DIC subdomains (cell ->
        subdomain id, decomposePar's cellDecomposition); implies
        renumber="none" and dic_subdomains=True.  outer may hold
        fieldRelaxation (fvSolution relaxationFactors fields factor) and
        relaxationMethod ("fixed" or "Aitken")."""
        self.time_steps = None
        if model not in MODELS:
            raise ValueError(f"unknown solidModel {model!r}; valid: {list(MODELS)}")
        self.ctx = ctx
        self.L = ctx.L
        self.model = model
        self.mesh = mesh
        self.n_cells = int(np.asarray(mesh["V"]).shape[0])
        keep = []
        d = _desc(mesh, keep)
        if parts is not None:
            parts = np.ascontiguousarray(parts, dtype=np.int32)
            keep.append(parts)
            renumber, dic_subdomains = "none", True
        opts = _lib.MeshOpts(RENUMBER[renumber], part_size, ls_boundary_delta,
                             1 if dic_subdomains else 0, 0 if autotune else 1, empty_direction,
                             None if parts is None else parts.ctypes.data)
        h = ct.c_void_p()
        _lib.check(self.L.s4g_mesh_upload(ctx.h, ct.byref(d), ct.byref(opts), ct.byref(h)),
                   "s4g_mesh_upload")
        self.h = h
        ctx.models.add(self)
        self.set_law(law)
        names = list(mesh.get("patch_names", PATCHES))
        for name, spec in bcs.items():
            self.set_bc(names.index(name), *spec)
        self.set_controls(solver or {}, outer or {}, precision)

    @classmethod
    def from_case(cls, ctx: "Context", case_dir: str, **kw):
        """A model of a meshed OpenFOAM case directory (foam_case.load_case):
        returns (model, n_increments) for model.evolve(n_increments).  A
        case with load tables other than ramps from zero keeps its time
        steps in model.time_steps (for model.run_time_steps()).  Keyword
        arguments (precision, renumber, part_size, ...) are passed on to the
        constructor."""
        from .foam_case import load_case
        c = load_case(case_dir)
        kw.setdefault("empty_direction", c["mesh"].get("empty_direction", 0))
        kw.setdefault("ls_boundary_delta", c["ls_boundary_delta"])
        model = cls(ctx, c["mesh"], c["law"], c["bcs"], model=c["model"], solver=c["solver"],
                    outer=c["outer"], **kw)
        model.time_steps = c["time_steps"]
        return model, c["n_increments"]

    def close(self):
        if self.h and self.ctx.h:
            self.L.s4g_mesh_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- constant/mechanicalProperties
    def set_law(self, law: dict):
        lw = _law_struct(law)
        _lib.check(self.L.s4g_material_set(self.h, ct.byref(lw)), "s4g_material_set")

    # -- 0/D boundaryField
    def set_bc(self, patch: int, bc_type: str, value=None, pressure=None,
               relaxation: float | None = None):
        """relaxation: the solidTraction relaxationFactor (default 1)."""
        t = {"fixedDisplacement": _lib.FIXED_DISPLACEMENT,
             "solidTraction": _lib.SOLID_TRACTION,
             "solidTractionFree": _lib.SOLID_TRACTION}[bc_type]
        size = int(self.mesh["patch_size"][patch])
        v = None if value is None else np.ascontiguousarray(
            np.broadcast_to(np.asarray(value, dtype=np.float64), (size, 3)))
        p = None if pressure is None else np.ascontiguousarray(
            np.broadcast_to(np.asarray(pressure, dtype=np.float64), (size,)))
        _lib.check(self.L.s4g_bc_set(self.h, patch, t, None if v is None else v.ctypes.data,
                                     None if p is None else p.ctypes.data), "s4g_bc_set")
        if relaxation is not None:
            _lib.check(self.L.s4g_bc_set_relaxation(self.h, patch, float(relaxation)),
                       "s4g_bc_set_relaxation")

    # -- system/fvSolution and solidProperties <model>Coeffs
    def set_controls(self, solver: dict, outer: dict, precision: str = "FP64"):
        lin, out, prec = _control_structs(self.L, solver, outer, precision)
        _lib.check(self.L.s4g_solver_set(self.h, ct.byref(lin), ct.byref(out), prec),
                   "s4g_solver_set")

    def evolve(self, n_increments: int = 1):
        """Runs the outer-corrector loop; returns (D [n,3], sigma [n,6], perf)."""
        D = np.zeros((self.n_cells, 3))
        sig = np.zeros((self.n_cells, 6))
        perf = _lib.Perf()
        st = self.L.s4g_solve(self.h, MODELS[self.model], int(n_increments), D.ctypes.data,
                              sig.ctypes.data, ct.byref(perf))
        _lib.check(st, "s4g_solve", allow=(_lib.OK, _lib.NOT_CONVERGED))
        return D, sig, perf.as_dict()

    def step(self, bcs: dict | None = None):
        """One time step (s4g_solve_step): evolve() once with the boundary
        values as they are, continuing from the previous step's state.
        bcs (optional): {patch name: (type, value, pressure[, relaxation])}
        set first, e.g. a load series evaluated at the step's time.
        Returns (D [n,3], sigma [n,6], perf of this step)."""
        if bcs:
            names = list(self.mesh.get("patch_names", PATCHES))
            for name, spec in bcs.items():
                self.set_bc(names.index(name), spec[0], spec[1] if len(spec) > 1 else None,
                            spec[2] if len(spec) > 2 else None,
                            spec[3] if len(spec) > 3 else None)
        D = np.zeros((self.n_cells, 3))
        sig = np.zeros((self.n_cells, 6))
        perf = _lib.Perf()
        st = self.L.s4g_solve_step(self.h, MODELS[self.model], D.ctypes.data, sig.ctypes.data,
                                   ct.byref(perf))
        _lib.check(st, "s4g_solve_step", allow=(_lib.OK, _lib.NOT_CONVERGED))
        return D, sig, perf.as_dict()

    def run_time_steps(self, steps=None):
        """Steps through [(time, bcs), ...] -- by default the case's own
        time_steps (from_case) -- one s4g_solve_step each.  Returns (D,
        sigma) of the last step and the perf of every step."""
        steps = self.time_steps if steps is None else steps
        if not steps:
            raise ValueError("no time steps to run")
        perfs = []
        for _, bcs in steps:
            D, sig, perf = self.step(bcs)
            perfs.append(perf)
        return D, sig, perfs

    def reset_state(self):
        """The next step starts from zero (s4g_state_reset)."""
        _lib.check(self.L.s4g_state_reset(self.h), "s4g_state_reset")

    def evolve_cases(self, case_bcs: list):
        """Batched load cases (s4g_solve_cases): case_bcs is a list of
        dicts {patch name: (type, value, pressure)} like the constructor's
        bcs, one per case, with the model's boundary-condition types.
        Returns (D [C,n,3], sigma [C,n,6], [perf per case])."""
        C = len(case_bcs)
        nI = int(np.asarray(self.mesh["neighbour"]).shape[0])
        nB = int(np.asarray(self.mesh["owner"]).shape[0]) - nI
        names = list(self.mesh.get("patch_names", PATCHES))
        starts = np.asarray(self.mesh["patch_start"]) - nI
        sizes = np.asarray(self.mesh["patch_size"])
        bval = np.zeros((C, nB, 3))
        bpress = np.zeros((C, nB))
        for c, bcs in enumerate(case_bcs):
            for name, spec in bcs.items():
                i = names.index(name)
                lo, hi = int(starts[i]), int(starts[i] + sizes[i])
                value = spec[1] if len(spec) > 1 else None
                pressure = spec[2] if len(spec) > 2 else None
                if value is not None:
                    bval[c, lo:hi] = np.broadcast_to(np.asarray(value, np.float64), (hi - lo, 3))
                if pressure is not None:
                    bpress[c, lo:hi] = np.broadcast_to(np.asarray(pressure, np.float64), (hi - lo,))
        D = np.zeros((C, self.n_cells, 3))
        sig = np.zeros((C, self.n_cells, 6))
        perfs = (_lib.Perf * C)()
        st = self.L.s4g_solve_cases(self.h, C, bval.ctypes.data, bpress.ctypes.data, D.ctypes.data,
                                    sig.ctypes.data, ct.cast(perfs, ct.c_void_p))
        _lib.check(st, "s4g_solve_cases", allow=(_lib.OK, _lib.NOT_CONVERGED))
        return D, sig, [p.as_dict() for p in perfs]

    def gradD(self):
        G = np.zeros((self.n_cells, 9))
        _lib.check(self.L.s4g_get_gradD(self.h, G.ctypes.data), "s4g_get_gradD")
        return G

    def set_points(self, points, point_cell_start, point_cells):
        """The mesh's points and the cells of each point (s4g_point_cells)
        for point_displacement_device."""
        pts = np.ascontiguousarray(points, dtype=np.float64)
        pcs = np.ascontiguousarray(point_cell_start, dtype=np.int32)
        pcc = np.ascontiguousarray(point_cells, dtype=np.int32)
        _lib.check(self.L.s4g_mesh_set_points(self.h, int(pts.shape[0]), pts.ctypes.data,
                                              pcs.ctypes.data, pcc.ctypes.data),
                   "s4g_mesh_set_points")
        self.n_points = int(pts.shape[0])

    def point_displacement_device(self):
        """pointD of the last solve, interpolated on the device (s4g_get_pointD)."""
        out = np.zeros((self.n_points, 3))
        _lib.check(self.L.s4g_get_pointD(self.h, out.ctypes.data), "s4g_get_pointD")
        return out

    def permutation(self):
        perm = np.zeros(self.n_cells, np.int32)
        _lib.check(self.L.s4g_mesh_get_permutation(self.h, perm.ctypes.data),
                   "s4g_mesh_get_permutation")
        return perm

    def parts(self):
        """Scheduling part (DIC subdomain with dic_subdomains) of each cell."""
        part = np.zeros(self.n_cells, np.int32)
        _lib.check(self.L.s4g_mesh_get_parts(self.h, part.ctypes.data), "s4g_mesh_get_parts")
        return part

    def info(self):
        inf = _lib.MeshInfo()
        _lib.check(self.L.s4g_mesh_get_info(self.h, ct.byref(inf)), "s4g_mesh_get_info")
        return {f[0]: getattr(inf, f[0]) for f in inf._fields_}

    # operator-level access (parity tests)
    def op_matrix(self):
        diag = np.zeros(self.n_cells)
        upper = np.zeros(int(np.asarray(self.mesh["neighbour"]).shape[0]))
        _lib.check(self.L.s4g_op_matrix(self.h, diag.ctypes.data, upper.ctypes.data),
                   "s4g_op_matrix")
        return diag, upper

    def op_amul(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        k = 1 if x.ndim == 1 else x.shape[1]
        y = np.zeros_like(x)
        _lib.check(self.L.s4g_op_amul(self.h, k, x.ctypes.data, y.ctypes.data), "s4g_op_amul")
        return y

    def op_amul_dot_noalloc(self, x):
        """y = A x and the column products x.Ax through the entry point that
        allocates nothing (meshes of at most 262,144 cells, matrix assembled)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        k = 1 if x.ndim == 1 else x.shape[1]
        y = np.zeros_like(x)
        xax = np.zeros(k)
        _lib.check(self.L.s4g_op_amul_dot_noalloc(self.h, k, x.ctypes.data, y.ctypes.data,
                                                   xax.ctypes.data), "s4g_op_amul_dot_noalloc")
        return y, xax

    def op_precondition(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        k = 1 if r.ndim == 1 else r.shape[1]
        w = np.zeros_like(r)
        _lib.check(self.L.s4g_op_precondition(self.h, k, r.ctypes.data, w.ctypes.data),
                   "s4g_op_precondition")
        return w


def solve_batch(models):
    """s4g_solve_batch: the linear-geometry solves of several models (one
    context, one CUDA-graph launch for all).  Returns a list of (D, sigma,
    perf) in the order of `models`."""
    n = len(models)
    if n == 0:
        return []
    L = models[0].L
    hs = (ct.c_void_p * n)(*[m.h.value if isinstance(m.h, ct.c_void_p) else m.h for m in models])
    Ds = [np.zeros((m.n_cells, 3)) for m in models]
    Ss = [np.zeros((m.n_cells, 6)) for m in models]
    dp = (ct.c_void_p * n)(*[d.ctypes.data for d in Ds])
    sp = (ct.c_void_p * n)(*[x.ctypes.data for x in Ss])
    perfs = (_lib.Perf * n)()
    st = L.s4g_solve_batch(ct.cast(hs, ct.c_void_p), n, ct.cast(dp, ct.c_void_p),
                           ct.cast(sp, ct.c_void_p), ct.cast(perfs, ct.c_void_p))
    _lib.check(st, "s4g_solve_batch", allow=(_lib.OK, _lib.NOT_CONVERGED))
    return [(Ds[i], Ss[i], perfs[i].as_dict()) for i in range(n)]


def plan(mesh, renumber: str = "tiled", part_size: int = 512, dic_subdomains: bool = False,
         parts=None):
    """Host-only DIC order and scheduling figures (no GPU): (perm, info).
    parts: a caller decomposition, as for SolidModel (renumber and
    dic_subdomains are then passed as given, so that the library's checks
    on them can be seen)."""
    L = _lib.lib()
    keep = []
    d = _desc(mesh, keep)
    if parts is not None:
        parts = np.ascontiguousarray(parts, dtype=np.int32)
        keep.append(parts)
    opts = _lib.MeshOpts(RENUMBER[renumber], part_size, 0, 1 if dic_subdomains else 0, 0, 0,
                         None if parts is None else parts.ctypes.data)
    n = d.n_cells
    perm = np.zeros(n, np.int32)
    inf = _lib.MeshInfo()
    _lib.check(L.s4g_mesh_plan(ct.byref(d), ct.byref(opts), perm.ctypes.data, ct.byref(inf)),
               "s4g_mesh_plan")
    return perm, {f[0]: getattr(inf, f[0]) for f in inf._fields_}


BC_TYPES = {"fixedDisplacement": _lib.FIXED_DISPLACEMENT, "solidTraction": _lib.SOLID_TRACTION,
            "solidTractionFree": _lib.SOLID_TRACTION}


class Server:
    """Continuous admission of solves onto one GPU (s4g_server_*): submit
    requests from any thread, poll their results; p50/p99 latency and
    throughput from stats()."""

    def __init__(self, device: int = 0, max_slots: int = 8, memory_budget: int = 0,
                 dry_run: bool = False, dry_run_us_per_kcell: float = 50.0):
        self.L = _lib.lib()
        o = _lib.ServerOpts(device, max_slots, int(memory_budget), 1 if dry_run else 0,
                            float(dry_run_us_per_kcell))
        h = ct.c_void_p()
        _lib.check(self.L.s4g_server_create(ct.byref(o), ct.byref(h)), "s4g_server_create")
        self.h = h
        self.n_cells = {}

    def submit(self, mesh, law: dict, bcs: dict, model: str = "linearGeometryTotalDisplacement",
               solver: dict | None = None, outer: dict | None = None, precision: str = "FP64",
               n_increments: int = 1, renumber: str = "tiled", part_size: int = 512,
               dic_subdomains: bool = False, parts=None):
        """bcs entries are (type, value, pressure[, relaxationFactor]);
        parts as for SolidModel."""
        keep = []
        d = _desc(mesh, keep)
        names = list(mesh.get("patch_names", PATCHES))
        patches, types, vecs, press, relax = [], [], [], [], []
        for name, spec in bcs.items():
            i = names.index(name)
            size = int(np.asarray(mesh["patch_size"])[i])
            patches.append(i)
            types.append(BC_TYPES[spec[0]])
            v = spec[1] if len(spec) > 1 else None
            p = spec[2] if len(spec) > 2 else None
            relax.append(1.0 if len(spec) < 4 or spec[3] is None else float(spec[3]))
            va = None if v is None else np.ascontiguousarray(
                np.broadcast_to(np.asarray(v, np.float64), (size, 3)))
            pa = None if p is None else np.ascontiguousarray(
                np.broadcast_to(np.asarray(p, np.float64), (size,)))
            keep += [va, pa]
            vecs.append(None if va is None else va.ctypes.data)
            press.append(None if pa is None else pa.ctypes.data)
        nb = len(patches)
        pa_ = (ct.c_int * max(nb, 1))(*patches)
        ta_ = (ct.c_int * max(nb, 1))(*types)
        va_ = (ct.c_void_p * max(nb, 1))(*vecs)
        pr_ = (ct.c_void_p * max(nb, 1))(*press)
        rl_ = (ct.c_double * max(nb, 1))(*relax)
        lin, out, prec = _control_structs(self.L, solver or {}, outer or {}, precision)
        rq = _lib.Request()
        rq.mesh = ct.cast(ct.pointer(d), ct.c_void_p)
        if parts is not None:
            parts = np.ascontiguousarray(parts, dtype=np.int32)
            keep.append(parts)
            renumber, dic_subdomains = "none", True
        rq.mesh_opts = _lib.MeshOpts(RENUMBER[renumber], part_size, 0,
                                     1 if dic_subdomains else 0, 0, 0,
                                     None if parts is None else parts.ctypes.data)
        rq.law = _law_struct(law)
        rq.n_bc = nb
        rq.bc_patch = ct.cast(pa_, ct.c_void_p)
        rq.bc_type = ct.cast(ta_, ct.c_void_p)
        rq.bc_vec3 = ct.cast(va_, ct.c_void_p)
        rq.bc_pressure = ct.cast(pr_, ct.c_void_p)
        rq.lin, rq.outer, rq.precision = lin, out, prec
        rq.model = MODELS[model]
        rq.n_increments = int(n_increments)
        rq.bc_relaxation = ct.cast(rl_, ct.c_void_p)
        rid = ct.c_uint64()
        _lib.check(self.L.s4g_server_submit(self.h, ct.byref(rq), ct.byref(rid)),
                   "s4g_server_submit")
        self.n_cells[rid.value] = d.n_cells
        return rid.value

    def result(self, rid: int, wait: bool = True):
        """(status, D, sigma, perf); None while pending (wait=False)."""
        n = self.n_cells[rid]
        D = np.zeros((n, 3))
        sig = np.zeros((n, 6))
        perf = _lib.Perf()
        st = self.L.s4g_server_poll(self.h, rid, 1 if wait else 0, D.ctypes.data, sig.ctypes.data,
                                    ct.byref(perf))
        if st == _lib.PENDING:
            return None
        del self.n_cells[rid]
        return st, D, sig, perf.as_dict()

    def cancel(self, rid: int):
        _lib.check(self.L.s4g_server_cancel(self.h, rid), "s4g_server_cancel")

    def stats(self):
        st = _lib.ServerStats()
        _lib.check(self.L.s4g_server_get_stats(self.h, ct.byref(st)), "s4g_server_get_stats")
        return {f[0]: getattr(st, f[0]) for f in st._fields_}

    def close(self):
        if self.h:
            self.L.s4g_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
