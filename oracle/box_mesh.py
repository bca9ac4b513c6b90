"""Seeded hexahedral box meshes for the oracle, in numpy.

TEST INFRASTRUCTURE ONLY: the CPU baseline of the benchmark and the tests
build their meshes here, so that the oracle's inputs do not come from the
product library.

The mesh is the one the library's generator (s4g_box_mesh_build) defines:
a structured nx x ny x nz box in OpenFOAM polyMesh conventions whose
interior vertices move by a seeded uniform amount in [-jitter h, +jitter h]
per axis (a stand-in for the reference's perturbMeshPoints utility,
applications/utilities/perturbMeshPoints/perturbMeshPoints.C:244-330),
with OpenFOAM's primitiveMesh geometry:
  * face centre and area vector from a fan of triangles about the average
    of the face's points, the centre weighted by the triangles' areas;
  * cell centre and volume from pyramids on the cell's faces, apex at the
    average of the cell's face centres.
Conventions: cells i + nx (j + ny k); internal faces of each cell in cell
order, its +x, +y, +z faces (so sorted by owner, then neighbour); boundary
patches xmin, xmax, ymin, ymax, zmin, zmax; area vectors point out of the
owner.  Random numbers are a counter-based splitmix64 of (seed, 3 v + axis)
for vertex v.  Every floating-point operation is done in the order the
generator's definition gives, element by element, so the arrays are equal
bit for bit to the library's on any machine that rounds IEEE double
operations without fused multiply-adds.
"""
from __future__ import annotations

import numpy as np

PATCHES = ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x):
    x = x + np.uint64(0x9E3779B97F4A7C15)
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def _uniform01(seed, idx):
    with np.errstate(over="ignore"):
        s = _splitmix64(np.array([seed], dtype=np.uint64))[0]
        h = _splitmix64(s ^ (idx.astype(np.uint64) * np.uint64(0xD1B54A32D192ED03)))
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _points(nx, ny, nz, lx, ly, lz, jitter, seed):
    hx, hy, hz = lx / nx, ly / ny, lz / nz
    k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    P = np.stack([i * hx, j * hy, k * hz], axis=1)
    if jitter > 0:
        inner = (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)
        v = np.nonzero(inner)[0].astype(np.uint64)
        for ax, h in enumerate((hx, hy, hz)):
            u = _uniform01(seed, np.uint64(3) * v + np.uint64(ax))
            P[inner, ax] = P[inner, ax] + ((2.0 * u - 1.0) * jitter) * h
    return P


def _faces(nx, ny, nz):
    """Owner, neighbour (-1 on the boundary) and the four point ids of every
    face in storage order, with the patch starts and sizes."""
    px, py = nx + 1, ny + 1
    pid = lambda i, j, k: i + px * (j + py * k)
    cid = lambda i, j, k: i + nx * (j + ny * k)

    def quad(axis, i, j, k):
        if axis == 0:
            return np.stack([pid(i, j, k), pid(i, j + 1, k), pid(i, j + 1, k + 1), pid(i, j, k + 1)], -1)
        if axis == 1:
            return np.stack([pid(i, j, k), pid(i, j, k + 1), pid(i + 1, j, k + 1), pid(i + 1, j, k)], -1)
        return np.stack([pid(i, j, k), pid(i + 1, j, k), pid(i + 1, j + 1, k), pid(i, j + 1, k)], -1)

    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    c = cid(i, j, k)
    n = c.shape[0]
    # per cell in order: +x, +y, +z internal faces where they exist
    own = np.repeat(c, 3)
    nei = np.stack([cid(i + 1, j, k), cid(i, j + 1, k), cid(i, j, k + 1)], 1).ravel()
    ok = np.stack([i + 1 < nx, j + 1 < ny, k + 1 < nz], 1).ravel()
    q = np.stack([quad(0, i + 1, j, k), quad(1, i, j + 1, k), quad(2, i, j, k + 1)], 1).reshape(3 * n, 4)
    owner, neighbour, fq = [own[ok]], [nei[ok]], [q[ok]]
    starts, sizes = [], []
    nf = int(ok.sum())

    def flip(qq):
        return qq[:, [0, 3, 2, 1]]

    def patch(cells, qq, flipped):
        nonlocal nf
        starts.append(nf)
        sizes.append(cells.shape[0])
        owner.append(cells)
        neighbour.append(np.full(cells.shape[0], -1))
        fq.append(flip(qq) if flipped else qq)
        nf += cells.shape[0]

    kk, jj = np.meshgrid(np.arange(nz), np.arange(ny), indexing="ij")
    kk, jj = kk.ravel(), jj.ravel()
    patch(cid(0, jj, kk), quad(0, 0 * jj, jj, kk), True)
    patch(cid(nx - 1, jj, kk), quad(0, nx + 0 * jj, jj, kk), False)
    kk, ii = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")
    kk, ii = kk.ravel(), ii.ravel()
    patch(cid(ii, 0, kk), quad(1, ii, 0 * ii, kk), True)
    patch(cid(ii, ny - 1, kk), quad(1, ii, ny + 0 * ii, kk), False)
    jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    jj, ii = jj.ravel(), ii.ravel()
    patch(cid(ii, jj, 0), quad(2, ii, jj, 0 * ii), True)
    patch(cid(ii, jj, nz - 1), quad(2, ii, jj, nz + 0 * ii), False)
    return (np.concatenate(owner), np.concatenate(neighbour), np.concatenate(fq),
            np.array(starts), np.array(sizes))


def _add(a, b):
    return a + b


def _cross(a, b):
    return np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                     a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], 1)


def _dot(a, b):
    return (a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1]) + a[:, 2] * b[:, 2]


def _face_geometry(P, fq):
    """Triangle fan about the point average: centre and area vector."""
    pts = [P[fq[:, m]] for m in range(4)]
    fc = ((pts[0] + pts[1]) + pts[2]) + pts[3]
    fc = (1.0 / 4) * fc
    sumN = np.zeros_like(fc)
    sumAc = np.zeros_like(fc)
    sumA = np.zeros(fc.shape[0])
    for m in range(4):
        a, b = pts[m], pts[(m + 1) % 4]
        c = (a + b) + fc
        nn = _cross(b - a, fc - a)
        mg = np.sqrt(_dot(nn, nn))
        sumN = sumN + nn
        sumA = sumA + mg
        sumAc = sumAc + mg[:, None] * c
    ctr = (1.0 / (3.0 * sumA))[:, None] * sumAc
    area = 0.5 * sumN
    return ctr, area


def _cell_geometry(n_cells, owner, neighbour, n_int, Cf, Sf):
    """Pyramids about the average face centre; each cell's faces are taken
    in increasing face order (a face adds to its owner, then its
    neighbour)."""
    nf = owner.shape[0]
    fidx = np.arange(nf)
    cells = np.concatenate([owner, neighbour[:n_int]])
    faces = np.concatenate([fidx, fidx[:n_int]])
    isown = np.concatenate([np.ones(nf, bool), np.zeros(n_int, bool)])
    order = np.lexsort((faces, cells))   # by cell, then face
    cells, faces, isown = cells[order], faces[order], isown[order]
    per = np.bincount(cells, minlength=n_cells)
    if np.any(per == 0) or np.any(per != per[0]):
        raise ValueError("every cell of a box mesh has the same number of faces")
    k = int(per[0])
    F = faces.reshape(n_cells, k)
    O = isown.reshape(n_cells, k)
    est = np.zeros((n_cells, 3))
    for m in range(k):
        est = est + Cf[F[:, m]]
    est = (1.0 / k) * est
    cc = np.zeros((n_cells, 3))
    vv = np.zeros(n_cells)
    for m in range(k):
        fc, fa = Cf[F[:, m]], Sf[F[:, m]]
        v3 = np.where(O[:, m], _dot(fa, fc - est), _dot(fa, est - fc))
        pc = 0.75 * fc + 0.25 * est
        cc = cc + v3[:, None] * pc
        vv = vv + v3
    if not np.all(vv > 0):
        raise ValueError("inverted cell: the jitter is too large")
    C = (1.0 / vv)[:, None] * cc
    V = vv / 3.0
    return C, V


def box_mesh(nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, jitter=0.0, seed=1, points=False):
    """The mesh dict of a seeded box (owner, neighbour, C, V, Cf, Sf,
    patch_start, patch_size, shape, patch_names[, points])."""
    if not (0 <= jitter < 0.5):
        raise ValueError("jitter must be in [0, 0.5)")
    P = _points(nx, ny, nz, lx, ly, lz, jitter, seed)
    owner, nei, fq, starts, sizes = _faces(nx, ny, nz)
    n_int = int(starts[0])
    Cf, Sf = _face_geometry(P, fq)
    C, V = _cell_geometry(nx * ny * nz, owner, nei, n_int, Cf, Sf)
    m = dict(owner=owner.astype(np.int32), neighbour=nei[:n_int].astype(np.int32), C=C, V=V,
             Cf=Cf, Sf=Sf, patch_start=starts.astype(np.int32), patch_size=sizes.astype(np.int32),
             shape=(nx, ny, nz), patch_names=PATCHES)
    if points:
        m["points"] = P
    return m


def block_parts(nx, ny, nz, bx, by=None, bz=None):
    """A decomposition of the box into bx x by x bz blocks of cells (the
    last block of an axis takes the remainder), numbered block i fastest:
    cell i + nx (j + ny k) -> block (i // bx) + nbx ((j // by) + nby (k // bz)),
    like a decomposePar 'simple' decomposition into regular blocks."""
    by = by or bx
    bz = bz or bx
    nbx, nby = -(-nx // bx), -(-ny // by)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return ((i // bx) + nbx * ((j // by) + nby * (k // bz))).ravel().astype(np.int32)
