"""OpenFOAM case files on the host (s4g_foam_* in libs4g): read a meshed
case's constant/polyMesh and 0/D into the mesh and boundary-condition
dictionaries SolidModel takes, and write meshes as ASCII polyMesh.

The mesh dictionary has the keys of box_mesh (owner, neighbour, C, V, Cf,
Sf, patch_start, patch_size, patch_names) plus patch_types, points,
face_start and face_points; with a D file also load_ramp_end (the end time
of its load series, which are linear ramps from zero, or None) and
constant_loads_beside_ramp.  The boundary conditions are
{patch name: (type, value or traction [n,3], pressure [n] or None,
relaxationFactor)}."""
import ctypes as ct
import os

import numpy as np

from . import _lib
from .cases import box_mesh

BC_NAMES = {_lib.FIXED_DISPLACEMENT: "fixedDisplacement", _lib.SOLID_TRACTION: "solidTraction"}


def _arr(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype)
    ctype = {np.float64: ct.c_double, np.int32: ct.c_int}[dtype]
    return np.ctypeslib.as_array(ct.cast(ptr, ct.POINTER(ctype)), shape=(n,)).copy()


def read_case(case_dir: str, d_file: str | None = "0/D", polymesh: str = "constant/polyMesh"):
    """Reads <case_dir>/<polymesh> and, unless d_file is None, the
    boundaryField of <case_dir>/<d_file>.  Returns (mesh, bcs); bcs is None
    when no D file is read."""
    L = _lib.lib()
    h = ct.c_void_p()
    _lib.check(L.s4g_foam_read_mesh(os.path.join(case_dir, polymesh).encode(), ct.byref(h)),
               "s4g_foam_read_mesh")
    try:
        d = _lib.MeshDesc()
        npts = ct.c_int()
        _lib.check(L.s4g_foam_mesh_desc(h, ct.byref(d), ct.byref(npts)), "s4g_foam_mesh_desc")
        nc, nf, ni, npch = d.n_cells, d.n_faces, d.n_internal_faces, d.n_patches
        mesh = dict(owner=_arr(d.owner, nf, np.int32), neighbour=_arr(d.neighbour, ni, np.int32),
                    C=_arr(d.C, 3 * nc, np.float64).reshape(nc, 3), V=_arr(d.V, nc, np.float64),
                    Cf=_arr(d.Cf, 3 * nf, np.float64).reshape(nf, 3),
                    Sf=_arr(d.Sf, 3 * nf, np.float64).reshape(nf, 3),
                    patch_start=_arr(d.patch_start, npch, np.int32),
                    patch_size=_arr(d.patch_size, npch, np.int32))
        pp, fs, fp = ct.c_void_p(), ct.c_void_p(), ct.c_void_p()
        _lib.check(L.s4g_foam_mesh_points(h, ct.byref(pp), ct.byref(fs), ct.byref(fp)),
                   "s4g_foam_mesh_points")
        mesh["points"] = _arr(pp.value, 3 * npts.value, np.float64).reshape(-1, 3)
        mesh["face_start"] = _arr(fs.value, nf + 1, np.int32)
        mesh["face_points"] = _arr(fp.value, int(mesh["face_start"][-1]), np.int32)
        mesh["patch_names"] = [L.s4g_foam_patch_name(h, p).decode() for p in range(npch)]
        mesh["empty_direction"] = L.s4g_foam_empty_direction(h)
        mesh["patch_types"] = [L.s4g_foam_patch_type(h, p).decode() for p in range(npch)]
        bcs = None
        if d_file is not None:
            _lib.check(L.s4g_foam_read_d(h, os.path.join(case_dir, d_file).encode()),
                       "s4g_foam_read_d")
            bcs = {}
            for p, name in enumerate(mesh["patch_names"]):
                t, v, pr, rf = ct.c_int(), ct.c_void_p(), ct.c_void_p(), ct.c_double()
                _lib.check(L.s4g_foam_bc(h, p, ct.byref(t), ct.byref(v), ct.byref(pr), ct.byref(rf)),
                           "s4g_foam_bc")
                n = int(mesh["patch_size"][p])
                vec = _arr(v.value, 3 * n, np.float64).reshape(n, 3)
                press = None if not pr.value else _arr(pr.value, n, np.float64)
                bcs[name] = (BC_NAMES[t.value], vec, press, rf.value)
            end, mixed = ct.c_double(), ct.c_int()
            _lib.check(L.s4g_foam_load_ramp(h, ct.byref(end), ct.byref(mixed)),
                       "s4g_foam_load_ramp")
            mesh["load_ramp_end"] = end.value or None
            mesh["constant_loads_beside_ramp"] = bool(mixed.value)
            kind = ct.c_int()
            _lib.check(L.s4g_foam_series_kind(h, ct.byref(kind)), "s4g_foam_series_kind")
            mesh["load_series"] = kind.value
        return mesh, bcs
    finally:
        L.s4g_foam_free(h)


def bcs_at(case_dir: str, times, d_file: str = "0/D", polymesh: str = "constant/polyMesh"):
    """The D boundary conditions at each of `times` (s4g_foam_bc_at): the
    load series evaluated at the time, as the reference's conditions
    evaluate them at a time step, constant values as read.  One bcs dict
    per time, in read_case's form."""
    L = _lib.lib()
    h = ct.c_void_p()
    _lib.check(L.s4g_foam_read_mesh(os.path.join(case_dir, polymesh).encode(), ct.byref(h)),
               "s4g_foam_read_mesh")
    try:
        _lib.check(L.s4g_foam_read_d(h, os.path.join(case_dir, d_file).encode()), "s4g_foam_read_d")
        d = _lib.MeshDesc()
        npts = ct.c_int()
        _lib.check(L.s4g_foam_mesh_desc(h, ct.byref(d), ct.byref(npts)), "s4g_foam_mesh_desc")
        sizes = _arr(d.patch_size, d.n_patches, np.int32)
        names = [L.s4g_foam_patch_name(h, p).decode() for p in range(d.n_patches)]
        out = []
        for t in times:
            bcs = {}
            for p, name in enumerate(names):
                n = int(sizes[p])
                vec, press = np.zeros((n, 3)), np.zeros(n)
                ty, rf = ct.c_int(), ct.c_double()
                _lib.check(L.s4g_foam_bc_at(h, p, float(t), ct.byref(ty), vec.ctypes.data,
                                            press.ctypes.data, ct.byref(rf)), "s4g_foam_bc_at")
                bcs[name] = (BC_NAMES[ty.value], vec,
                             press if ty.value == _lib.SOLID_TRACTION else None, rf.value)
            out.append(bcs)
        return out
    finally:
        L.s4g_foam_free(h)


def write_polymesh(polymesh_dir: str, points, face_start, face_points, owner, neighbour,
                   patch_names, patch_start, patch_size, patch_types=None):
    """Writes an ASCII polyMesh into polymesh_dir, which is created if
    needed; patch_types (default all "patch") may name e.g. "empty"."""
    os.makedirs(polymesh_dir, exist_ok=True)
    keep = [np.ascontiguousarray(points, np.float64), np.ascontiguousarray(face_start, np.int32),
            np.ascontiguousarray(face_points, np.int32), np.ascontiguousarray(owner, np.int32),
            np.ascontiguousarray(neighbour, np.int32), np.ascontiguousarray(patch_start, np.int32),
            np.ascontiguousarray(patch_size, np.int32)]
    names = (ct.c_char_p * len(patch_names))(*[n.encode() for n in patch_names])
    types = None if patch_types is None else (ct.c_char_p * len(patch_types))(
        *[t.encode() for t in patch_types])
    pts, fs, fp, own, nei, ps, pz = keep
    _lib.check(_lib.lib().s4g_foam_write_mesh(
        polymesh_dir.encode(), pts.shape[0], pts.ctypes.data, fs.shape[0] - 1, fs.ctypes.data,
        fp.ctypes.data, nei.shape[0], own.ctypes.data, nei.ctypes.data, len(patch_names), names,
        ps.ctypes.data, pz.ctypes.data, types), "s4g_foam_write_mesh")


def box_polymesh(nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, jitter=0.0, seed=1):
    """box_mesh with its points and faces (four point ids per face)."""
    m = box_mesh(nx, ny, nz, lx, ly, lz, jitter, seed, points=True)
    nf = m["owner"].shape[0]
    fp = np.zeros((nf, 4), np.int32)
    _lib.check(_lib.lib().s4g_box_mesh_faces(nx, ny, nz, fp.ctypes.data), "s4g_box_mesh_faces")
    m["face_points"] = fp.reshape(-1)
    m["face_start"] = np.arange(0, 4 * nf + 1, 4, dtype=np.int32)
    return m


def write_box_case(polymesh_dir: str, mesh):
    """Writes a box_polymesh mesh as an ASCII polyMesh."""
    write_polymesh(polymesh_dir, mesh["points"], mesh["face_start"], mesh["face_points"],
                   mesh["owner"], mesh["neighbour"], list(mesh["patch_names"]),
                   mesh["patch_start"], mesh["patch_size"])


def polymesh_from_cells(points, cells, patch_of, patch_names):
    """An OpenFOAM polyMesh from cells given as lists of faces (point-id
    lists, any orientation): shared faces become internal faces (owner the
    lower cell, sorted by owner then neighbour), each face oriented out of
    its owner (by its area vector against the cell's point average; convex
    cells); every other face goes to patch patch_of(face centre).  Returns
    the arguments of write_polymesh."""
    points = np.asarray(points, np.float64)
    faces = {}  # sorted point ids -> [(cell, ids oriented out of that cell)]
    for cell, cell_faces in enumerate(cells):
        cc = points[sorted({i for f in cell_faces for i in f})].mean(axis=0)
        for f in cell_faces:
            q = points[f]
            area = 0.5 * sum(np.cross(q[e] - q[0], q[e + 1] - q[0]) for e in range(1, len(f) - 1))
            if np.dot(area, q.mean(axis=0) - cc) < 0:
                f = f[::-1]
            faces.setdefault(tuple(sorted(f)), []).append((cell, list(f)))
    internal, boundary = [], [[] for _ in patch_names]
    for users in faces.values():
        if len(users) == 2:
            (a, fa), (b, _) = sorted(users, key=lambda u: u[0])
            internal.append((a, b, fa))
        elif len(users) == 1:
            (a, fa), = users
            boundary[patch_of(points[fa].mean(axis=0))].append((a, fa))
        else:
            raise RuntimeError("a face shared by more than two cells")
    internal.sort(key=lambda t: (t[0], t[1]))
    for b in boundary:
        b.sort(key=lambda t: t[0])
    owner = [a for a, _, _ in internal] + [a for b in boundary for a, _ in b]
    flist = [f for _, _, f in internal] + [f for b in boundary for _, f in b]
    sizes = [len(b) for b in boundary]
    return dict(points=points,
                face_start=np.cumsum([0] + [len(f) for f in flist]).astype(np.int32),
                face_points=np.concatenate([np.asarray(f) for f in flist]).astype(np.int32),
                owner=np.asarray(owner, np.int32),
                neighbour=np.asarray([b for _, b, _ in internal], np.int32),
                patch_names=list(patch_names),
                patch_start=np.asarray(np.cumsum([len(internal)] + sizes[:-1]), np.int32),
                patch_size=np.asarray(sizes, np.int32))


def _box_patch(lx, ly, lz):
    def patch_of(c):
        for p, (axis, val) in enumerate(((0, 0.0), (0, lx), (1, 0.0), (1, ly), (2, 0.0), (2, lz))):
            if abs(c[axis] - val) < 1e-12 * max(lx, ly, lz):
                return p
        raise RuntimeError("boundary face off the box")
    return patch_of


def prism_box_polymesh(nx, ny, nz, lx=1.0, ly=1.0, lz=1.0):
    """An nx x ny x nz box whose hexahedra are each split along their x = y
    diagonal into two triangular prisms (cells 2h and 2h+1 of hex h), with
    the patches xmin, xmax, ymin, ymax, zmin, zmax.  Returns the arguments
    of write_polymesh."""
    px, py = nx + 1, ny + 1
    pid = lambda i, j, k: i + px * (j + py * k)
    g = np.meshgrid(np.arange(px) * (lx / nx), np.arange(py) * (ly / ny),
                    np.arange(nz + 1) * (lz / nz), indexing="ij")
    points = np.stack([a.transpose(2, 1, 0).reshape(-1) for a in g], axis=1)
    cells = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                for tri in (((i, j), (i + 1, j), (i + 1, j + 1)), ((i, j), (i + 1, j + 1), (i, j + 1))):
                    lo = [pid(a, b, k) for a, b in tri]
                    hi = [pid(a, b, k + 1) for a, b in tri]
                    cells.append([lo, hi] + [[lo[e], lo[(e + 1) % 3], hi[(e + 1) % 3], hi[e]]
                                             for e in range(3)])
    return polymesh_from_cells(points, cells, _box_patch(lx, ly, lz),
                               ["xmin", "xmax", "ymin", "ymax", "zmin", "zmax"])


def annulus_polymesh(nr, nt, nz, a, b, h):
    """A thick-walled cylinder a <= r <= b, 0 <= z <= h, of nr x nt x nz
    hexahedra (radial, circumferential, axial), closed around the axis, with
    the patches inner, outer, front (z = 0), back (z = h).  Returns the
    arguments of write_polymesh."""
    r = np.linspace(a, b, nr + 1)
    t = np.linspace(0.0, 2.0 * np.pi, nt + 1)[:-1]
    z = np.linspace(0.0, h, nz + 1)
    pid = lambda i, j, k: i + (nr + 1) * ((j % nt) + nt * k)
    points = np.array([[ri * np.cos(tj), ri * np.sin(tj), zk] for zk in z for tj in t for ri in r])
    cells = []
    for k in range(nz):
        for j in range(nt):
            for i in range(nr):
                v = [pid(i, j, k), pid(i + 1, j, k), pid(i + 1, j + 1, k), pid(i, j + 1, k)]
                w = [pid(i, j, k + 1), pid(i + 1, j, k + 1), pid(i + 1, j + 1, k + 1), pid(i, j + 1, k + 1)]
                cells.append([v, w] + [[v[e], v[(e + 1) % 4], w[(e + 1) % 4], w[e]] for e in range(4)])

    def patch_of(c):
        rc = np.hypot(c[0], c[1])
        if abs(c[2]) < 1e-12 * h:
            return 2
        if abs(c[2] - h) < 1e-12 * h:
            return 3
        return 0 if rc < 0.5 * (a + b) else 1
    return polymesh_from_cells(points, cells, patch_of, ["inner", "outer", "front", "back"])


def read_relaxation(case_dir: str, field: str = "D"):
    """(field factor, equation factor) of system/fvSolution's
    relaxationFactors for the solved field ("D", or "DD" for the incremental
    total Lagrangian model); 1.0 where none is set.  The field factor is
    built (read_controls returns it as outer["fieldRelaxation"]); equation
    relaxation is not, and a case that sets it below 1 must be refused."""
    ff, ef = ct.c_double(), ct.c_double()
    _lib.check(_lib.lib().s4g_foam_read_relaxation(
        os.path.join(case_dir, "system", "fvSolution").encode(), field.encode(), ct.byref(ff),
        ct.byref(ef)), "s4g_foam_read_relaxation")
    return ff.value, ef.value


MODEL_NAMES = {_lib.LIN_GEOM_TOTAL_DISP: "linearGeometryTotalDisplacement",
               _lib.NONLIN_GEOM_TOTAL_LAG: "nonLinearGeometryTotalLagrangian",
               _lib.NONLIN_GEOM_TOTAL_LAG_TOTAL_DISP:
                   "nonLinearGeometryTotalLagrangianTotalDisplacement"}


def read_controls(case_dir: str):
    """The case's model, law and controls (constant/solidProperties,
    constant/mechanicalProperties, system/fvSolution) as the keyword
    arguments of SolidModel: dict(model=..., law=..., solver=..., outer=...).
    Unset entries keep the reference defaults; anything not built raises."""
    model, law = ct.c_int(), _lib.Law()
    lin, out = _lib.LinSolver(), _lib.Outer()
    _lib.check(_lib.lib().s4g_foam_read_controls(case_dir.encode(), ct.byref(model), ct.byref(law),
                                                 ct.byref(lin), ct.byref(out)),
               "s4g_foam_read_controls")
    if law.type == _lib.LINEAR_ELASTIC:
        lw = dict(type="linearElastic")
    else:
        lw = dict(type="neoHookeanElastic")
    if law.use_mu_K:
        lw.update(mu=law.mu, K=law.K)
    else:
        lw.update(E=law.E, nu=law.nu)
    return dict(model=MODEL_NAMES[model.value], law=lw,
                solver=dict(preconditioner="DIC" if lin.preconditioner == _lib.PRECOND_DIC
                            else "diagonal",
                            tolerance=lin.tolerance, relTol=lin.rel_tol, maxIter=lin.max_iter),
                outer=dict(nCorrectors=out.n_correctors, solutionTolerance=out.solution_tol,
                           alternativeTolerance=out.alternative_tol,
                           materialTolerance=out.material_tol, infoFrequency=out.info_frequency,
                           stabilisation=dict(type="RhieChow", scaleFactor=out.stab_scale),
                           fieldRelaxation=out.field_relaxation,
                           relaxationMethod="fixed" if out.relaxation_method == 0 else "Aitken"))


def write_results(case_dir: str, time: str, D, sigma, gradD, polymesh: str = "constant/polyMesh",
                  d_file: str = "0/D"):
    """Writes D, sigma and sigmaEq into <case_dir>/<time>/ as ASCII vol
    fields: cell values, and on the patches the prescribed displacement
    (fixedDisplacement) or the gradient-extrapolated one for D, the adjacent
    cell's value for sigma and sigmaEq."""
    from .post import derived_fields
    L = _lib.lib()
    h = ct.c_void_p()
    _lib.check(L.s4g_foam_read_mesh(os.path.join(case_dir, polymesh).encode(), ct.byref(h)),
               "s4g_foam_read_mesh")
    try:
        _lib.check(L.s4g_foam_read_d(h, os.path.join(case_dir, d_file).encode()), "s4g_foam_read_d")
        D = np.ascontiguousarray(D, np.float64)
        sig = np.ascontiguousarray(sigma, np.float64)
        G = np.ascontiguousarray(gradD, np.float64).reshape(-1, 9)
        seq, _, _ = derived_fields(sig)
        d = _lib.MeshDesc()
        _lib.check(L.s4g_foam_mesh_desc(h, ct.byref(d), None), "s4g_foam_mesh_desc")
        Db = np.zeros((d.n_faces - d.n_internal_faces, 3))
        _lib.check(L.s4g_foam_boundary_D(h, D.ctypes.data, G.ctypes.data, Db.ctypes.data),
                   "s4g_foam_boundary_D")
        out = os.path.join(case_dir, time)
        os.makedirs(out, exist_ok=True)
        for name, width, dims, cells, bnd in (("D", 3, "[0 1 0 0 0 0 0]", D, Db),
                                              ("sigma", 6, "[1 -1 -2 0 0 0 0]", sig, None),
                                              ("sigmaEq", 1, "[1 -1 -2 0 0 0 0]", seq, None)):
            _lib.check(L.s4g_foam_write_field(h, out.encode(), name.encode(), width, dims.encode(),
                                              cells.ctypes.data,
                                              None if bnd is None else bnd.ctypes.data),
                       "s4g_foam_write_field")
    finally:
        L.s4g_foam_free(h)


def read_time(case_dir: str):
    """(startTime, endTime, deltaT) of system/controlDict."""
    t0, t1, dt = ct.c_double(), ct.c_double(), ct.c_double()
    _lib.check(_lib.lib().s4g_foam_read_time(
        os.path.join(case_dir, "system", "controlDict").encode(), ct.byref(t0), ct.byref(t1),
        ct.byref(dt)), "s4g_foam_read_time")
    return t0.value, t1.value, dt.value


def load_case(case_dir: str):
    """Everything a solve of a meshed case needs, resolved as the C++ driver
    resolves it: dict(mesh, bcs, model, law, solver, outer, n_increments,
    ls_boundary_delta).
    The model, law and controls come from the case's dictionaries; a total
    Lagrangian case whose loads ramp from zero runs one increment per
    controlDict time step; a case with other load tables gets time_steps,
    [(time, bcs at that time)] for SolidModel.run_time_steps (None
    otherwise).  Raises for what is not built: equation
    relaxation of the solved field, constant loads beside a ramp (total
    Lagrangian), load series whose end is not the controlDict endTime (or a
    startTime other than 0), and everything the readers refuse."""
    mesh, bcs = read_case(case_dir)
    c = read_controls(case_dir)
    tl = c["model"] != "linearGeometryTotalDisplacement"
    if os.path.exists(os.path.join(case_dir, "system", "fvSolution")):
        field = "DD" if c["model"] == "nonLinearGeometryTotalLagrangian" else "D"
        ff, ef = read_relaxation(case_dir, field)
        if ef != 1.0:
            raise ValueError(f"equation relaxationFactors for {field} ({ef:g}) are not built on "
                             "the GPU path")
    n_inc = 1
    steps = None
    if mesh.get("load_series") == 2:
        # tables other than ramps from zero: one s4g_solve_step per
        # controlDict time step, the series evaluated at its time
        cd = os.path.join(case_dir, "system", "controlDict")
        if not os.path.exists(cd):
            raise ValueError("load series that are not ramps from zero are stepped through "
                             "system/controlDict's time steps, and the case has none")
        t0, t1, dt = read_time(case_dir)
        n = max(1, int(round((t1 - t0) / dt)))
        times = [t0 + k * dt for k in range(1, n + 1)]
        steps = list(zip(times, bcs_at(case_dir, times)))
    ramp = mesh.get("load_ramp_end")
    if ramp:
        if tl and mesh.get("constant_loads_beside_ramp"):
            raise ValueError("constant loads beside load series are not built for the total "
                             "Lagrangian models")
        if os.path.exists(os.path.join(case_dir, "system", "controlDict")):
            t0, t1, dt = read_time(case_dir)
            # the series are applied up to their end value, which is the
            # reference's load at endTime only when the two coincide
            if t0 != 0.0 or abs(t1 - ramp) > 1e-9 * ramp:
                raise ValueError(f"load series end at {ramp:g} but the run goes from {t0:g} to "
                                 f"{t1:g}: only a run from 0 to the series' end is built")
            if tl:
                n_inc = max(1, int(round((t1 - t0) / dt)))
    # the leastSquares boundary delta the case's gradSchemes select
    lsd = 0
    fvs = os.path.join(case_dir, "system", "fvSchemes")
    if os.path.exists(fvs):
        field = "DD" if c["model"] == "nonLinearGeometryTotalLagrangian" else "D"
        v = ct.c_int()
        _lib.check(_lib.lib().s4g_foam_read_grad_scheme(fvs.encode(), field.encode(), ct.byref(v)),
                   "s4g_foam_read_grad_scheme")
        lsd = v.value
    return dict(mesh=mesh, bcs=bcs, n_increments=n_inc, ls_boundary_delta=lsd, time_steps=steps,
                **c)
