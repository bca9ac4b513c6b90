// Seeded hexahedral box-mesh generator in OpenFOAM polyMesh conventions.
//
// This is the case generator of the standalone driver: it stands in for
// `blockMesh` (structured hex box) followed by the reference's
// `perturbMeshPoints` utility (applications/utilities/perturbMeshPoints/
// perturbMeshPoints.C:244-330, seeded random vertex jitter) and OpenFOAM's
// primitiveMesh geometry (face centres/areas by triangle decomposition about
// the face-point average; cell centres/volumes by pyramid decomposition about
// the average of the face centres).  It is input generation, not part of the
// solve: a real OpenFOAM case hands the same arrays (owner, neighbour, C, V,
// Cf, Sf, patch table) straight to s4g_mesh_upload.
//
// Conventions (OpenFOAM polyMesh):
//  * cells numbered i + nx*(j + ny*k);
//  * internal faces first, upper-triangular: sorted by owner, then by
//    neighbour, owner < neighbour, area vector pointing owner -> neighbour;
//  * boundary faces grouped by patch in the order xmin, xmax, ymin, ymax,
//    zmin, zmax, area vectors pointing out of the domain.
// Jitter: every vertex that is not on the boundary of the box moves by an
// independent uniform amount in [-jitter*h, +jitter*h] per axis, h being the
// cell size along that axis.  Boundary vertices do not move, so patches stay
// planar.  The random stream is a counter-based splitmix64 of
// (seed, vertex, axis), so the mesh does not depend on generation order.

#include "s4g.h"
#include "host_geometry.hpp"

#include <cstdint>
#include <cstring>
#include <vector>

namespace {

using namespace s4g_host;

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Uniform double in [0,1) from (seed, stream index).
inline double uniform01(uint64_t seed, uint64_t idx) {
  uint64_t h = splitmix64(splitmix64(seed) ^ (idx * 0xD1B54A32D192ED03ull));
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// Faces of the nx x ny x nz box in storage order: visit(face, owner,
// neighbour or -1 on the boundary, four point ids ordered so that the area
// vector points out of the owner); fills the patch starts and sizes.
template <class Visit>
void boxFaces(int nx, int ny, int nz, int* patch_start, int* patch_size, Visit visit) {
  const int px = nx + 1, py = ny + 1;
  auto pid = [&](int i, int j, int k) { return i + px * (j + py * k); };
  auto cid = [&](int i, int j, int k) { return i + nx * (j + ny * k); };
  // Quads with their normal along +x, +y, +z (right-hand rule).
  int q[4];
  auto quadX = [&](int i, int j, int k) {
    q[0] = pid(i, j, k); q[1] = pid(i, j + 1, k); q[2] = pid(i, j + 1, k + 1); q[3] = pid(i, j, k + 1);
  };
  auto quadY = [&](int i, int j, int k) {
    q[0] = pid(i, j, k); q[1] = pid(i, j, k + 1); q[2] = pid(i + 1, j, k + 1); q[3] = pid(i + 1, j, k);
  };
  auto quadZ = [&](int i, int j, int k) {
    q[0] = pid(i, j, k); q[1] = pid(i + 1, j, k); q[2] = pid(i + 1, j + 1, k); q[3] = pid(i, j + 1, k);
  };
  int f = 0;
  auto emit = [&](int own, int nei, bool flip) {
    if (flip) { int t = q[1]; q[1] = q[3]; q[3] = t; }
    visit(f, own, nei, q);
    ++f;
  };
  // Internal faces: for each cell in order, its +x, +y, +z faces, which is
  // already sorted by (owner, neighbour) since c+1 < c+nx < c+nx*ny.
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        int c = cid(i, j, k);
        if (i + 1 < nx) { quadX(i + 1, j, k); emit(c, cid(i + 1, j, k), false); }
        if (j + 1 < ny) { quadY(i, j + 1, k); emit(c, cid(i, j + 1, k), false); }
        if (k + 1 < nz) { quadZ(i, j, k + 1); emit(c, cid(i, j, k + 1), false); }
      }
  // Boundary patches xmin, xmax, ymin, ymax, zmin, zmax.
  int p = 0;
  patch_start[0] = f;
  auto close = [&]() { patch_size[p] = f - patch_start[p]; if (++p < 6) patch_start[p] = f; };
  for (int k = 0; k < nz; ++k) for (int j = 0; j < ny; ++j) { quadX(0, j, k); emit(cid(0, j, k), -1, true); }
  close();
  for (int k = 0; k < nz; ++k) for (int j = 0; j < ny; ++j) { quadX(nx, j, k); emit(cid(nx - 1, j, k), -1, false); }
  close();
  for (int k = 0; k < nz; ++k) for (int i = 0; i < nx; ++i) { quadY(i, 0, k); emit(cid(i, 0, k), -1, true); }
  close();
  for (int k = 0; k < nz; ++k) for (int i = 0; i < nx; ++i) { quadY(i, ny, k); emit(cid(i, ny - 1, k), -1, false); }
  close();
  for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i) { quadZ(i, j, 0); emit(cid(i, j, 0), -1, true); }
  close();
  for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i) { quadZ(i, j, nz); emit(cid(i, j, nz - 1), -1, false); }
  close();
}

}  // namespace

extern "C" {

s4g_status s4g_box_mesh_sizes(int nx, int ny, int nz, int* n_cells,
                              int* n_faces, int* n_internal_faces,
                              int* n_points) {
  if (nx < 1 || ny < 1 || nz < 1 || !n_cells || !n_faces || !n_internal_faces)
    return S4G_BAD_ARG;
  long long nc = (long long)nx * ny * nz;
  long long ni = (long long)(nx - 1) * ny * nz + (long long)nx * (ny - 1) * nz +
                 (long long)nx * ny * (nz - 1);
  long long nb = 2LL * (ny * nz + nx * nz + nx * ny);
  if (nc > 0x7fffffff || ni + nb > 0x7fffffff) return S4G_BAD_ARG;
  *n_cells = (int)nc;
  *n_internal_faces = (int)ni;
  *n_faces = (int)(ni + nb);
  if (n_points) *n_points = (nx + 1) * (ny + 1) * (nz + 1);
  return S4G_OK;
}

s4g_status s4g_box_mesh_build(int nx, int ny, int nz, double lx, double ly,
                              double lz, double jitter, uint64_t seed,
                              int* owner, int* neighbour, double* C, double* V,
                              double* Cf, double* Sf, int* patch_start,
                              int* patch_size, double* points) {
  int nCells, nFaces, nInt, nPts;
  s4g_status st = s4g_box_mesh_sizes(nx, ny, nz, &nCells, &nFaces, &nInt, &nPts);
  if (st != S4G_OK) return st;
  if (!owner || !neighbour || !C || !V || !Cf || !Sf || !patch_start ||
      !patch_size || !(lx > 0) || !(ly > 0) || !(lz > 0) || jitter < 0 ||
      jitter >= 0.5)
    return S4G_BAD_ARG;

  const double hx = lx / nx, hy = ly / ny, hz = lz / nz;
  const int px = nx + 1, py = ny + 1;
  auto pid = [&](int i, int j, int k) { return i + px * (j + py * k); };
  std::vector<P3> pts((size_t)nPts);
  for (int k = 0; k <= nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        P3 p = {i * hx, j * hy, k * hz};
        bool interior = i > 0 && i < nx && j > 0 && j < ny && k > 0 && k < nz;
        if (interior && jitter > 0) {
          uint64_t v = (uint64_t)pid(i, j, k);
          p.x += (2.0 * uniform01(seed, 3 * v + 0) - 1.0) * jitter * hx;
          p.y += (2.0 * uniform01(seed, 3 * v + 1) - 1.0) * jitter * hy;
          p.z += (2.0 * uniform01(seed, 3 * v + 2) - 1.0) * jitter * hz;
        }
        pts[(size_t)pid(i, j, k)] = p;
      }
  if (points) std::memcpy(points, pts.data(), sizeof(P3) * pts.size());

  boxFaces(nx, ny, nz, patch_start, patch_size, [&](int f, int own, int nei, const int* q) {
    owner[f] = own;
    if (nei >= 0) neighbour[f] = nei;
    P3 r[4] = {pts[(size_t)q[0]], pts[(size_t)q[1]], pts[(size_t)q[2]], pts[(size_t)q[3]]};
    P3 c, a;
    polygonGeometry(r, 4, c, a);
    Cf[3 * (size_t)f + 0] = c.x; Cf[3 * (size_t)f + 1] = c.y; Cf[3 * (size_t)f + 2] = c.z;
    Sf[3 * (size_t)f + 0] = a.x; Sf[3 * (size_t)f + 1] = a.y; Sf[3 * (size_t)f + 2] = a.z;
  });
  // Cell centres and volumes; an inverted cell means the jitter was too large.
  if (!cellGeometry(nCells, nFaces, nInt, owner, neighbour, Cf, Sf, C, V)) return S4G_BAD_ARG;
  return S4G_OK;
}

s4g_status s4g_box_mesh_faces(int nx, int ny, int nz, int* face_points) {
  int nCells, nFaces, nInt, nPts;
  s4g_status st = s4g_box_mesh_sizes(nx, ny, nz, &nCells, &nFaces, &nInt, &nPts);
  if (st != S4G_OK) return st;
  if (!face_points) return S4G_BAD_ARG;
  int ps[6], pz[6];
  boxFaces(nx, ny, nz, ps, pz, [&](int f, int, int, const int* q) {
    for (int k = 0; k < 4; ++k) face_points[4 * (size_t)f + k] = q[k];
  });
  return S4G_OK;
}

}  // extern "C"
