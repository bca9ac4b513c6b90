"""The steps after the outer-corrector loop (host, libs4g): pointD by the
reference's gradient-extrapolated inverse-distance interpolation, and the
derived fields of writeFields (sigmaEq, epsilon, epsilonEq).  The mesh
dictionary needs points, face_start and face_points (box_polymesh,
prism_box_polymesh + read_case, or read_case's own keys)."""
import numpy as np

from . import _lib


def point_cells(mesh):
    """(point_cell_start [n_points+1], point_cells): the cells of every
    point in increasing order."""
    L = _lib.lib()
    pts = np.asarray(mesh["points"])
    fs = np.ascontiguousarray(mesh["face_start"], np.int32)
    fp = np.ascontiguousarray(mesh["face_points"], np.int32)
    own = np.ascontiguousarray(mesh["owner"], np.int32)
    nei = np.ascontiguousarray(mesh["neighbour"], np.int32)
    start = np.zeros(pts.shape[0] + 1, np.int32)
    args = (pts.shape[0], fs.shape[0] - 1, fs.ctypes.data, fp.ctypes.data, nei.shape[0],
            own.ctypes.data, nei.ctypes.data, start.ctypes.data)
    _lib.check(L.s4g_point_cells(*args, None), "s4g_point_cells")
    cells = np.zeros(int(start[-1]), np.int32)
    _lib.check(L.s4g_point_cells(*args, cells.ctypes.data), "s4g_point_cells")
    return start, cells


def point_displacement(mesh, D, gradD, pc=None):
    """pointD [n_points, 3] from the cell values D [n, 3] and gradD [n, 9]
    (SolidModel.gradD())."""
    start, cells = point_cells(mesh) if pc is None else pc
    pts = np.ascontiguousarray(mesh["points"], np.float64)
    C = np.ascontiguousarray(mesh["C"], np.float64)
    D = np.ascontiguousarray(D, np.float64)
    G = np.ascontiguousarray(gradD, np.float64).reshape(-1, 9)
    out = np.zeros((pts.shape[0], 3))
    _lib.check(_lib.lib().s4g_point_interpolate(pts.shape[0], pts.ctypes.data, start.ctypes.data,
                                                cells.ctypes.data, C.shape[0], C.ctypes.data,
                                                D.ctypes.data, G.ctypes.data, out.ctypes.data),
               "s4g_point_interpolate")
    return out


def derived_fields(sigma, gradD=None):
    """(sigmaEq [n], epsilon [n, 6] or None, epsilonEq [n] or None)."""
    s = np.ascontiguousarray(sigma, np.float64).reshape(-1, 6)
    n = s.shape[0]
    seq = np.zeros(n)
    eps = epsEq = None
    g = None
    if gradD is not None:
        g = np.ascontiguousarray(gradD, np.float64).reshape(-1, 9)
        eps, epsEq = np.zeros((n, 6)), np.zeros(n)
    _lib.check(_lib.lib().s4g_derived_fields(n, s.ctypes.data, None if g is None else g.ctypes.data,
                                             seq.ctypes.data,
                                             None if eps is None else eps.ctypes.data,
                                             None if epsEq is None else epsEq.ctypes.data),
               "s4g_derived_fields")
    return seq, eps, epsEq
