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

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

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

struct P3 { double x, y, z; };

inline P3 sub(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline P3 add(P3 a, P3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline P3 scl(double s, P3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline P3 cross(P3 a, P3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double dot(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double mag(P3 a) { return std::sqrt(dot(a, a)); }

// Face centre and area vector of a polygon: triangle fan about the point
// average, area-weighted triangle centroids (OpenFOAM primitiveMesh method).
void polygonGeometry(const P3* pts, int n, P3& ctr, P3& area) {
  P3 fc = {0, 0, 0};
  for (int i = 0; i < n; ++i) fc = add(fc, pts[i]);
  fc = scl(1.0 / n, fc);
  P3 sumN = {0, 0, 0}, sumAc = {0, 0, 0};
  double sumA = 0;
  for (int i = 0; i < n; ++i) {
    P3 a = pts[i], b = pts[(i + 1) % n];
    P3 c = add(add(a, b), fc);
    P3 nn = cross(sub(b, a), sub(fc, a));
    double m = mag(nn);
    sumN = add(sumN, nn);
    sumA += m;
    sumAc = add(sumAc, scl(m, c));
  }
  if (sumA < 1e-300) {
    ctr = fc;
    area = {0, 0, 0};
  } else {
    ctr = scl(1.0 / (3.0 * sumA), sumAc);
    area = scl(0.5, sumN);
  }
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

  auto cid = [&](int i, int j, int k) { return i + nx * (j + ny * k); };
  // Quads with their normal along +x, +y, +z (right-hand rule).
  auto quadX = [&](int i, int j, int k, P3* q) {
    q[0] = pts[pid(i, j, k)]; q[1] = pts[pid(i, j + 1, k)];
    q[2] = pts[pid(i, j + 1, k + 1)]; q[3] = pts[pid(i, j, k + 1)];
  };
  auto quadY = [&](int i, int j, int k, P3* q) {
    q[0] = pts[pid(i, j, k)]; q[1] = pts[pid(i, j, k + 1)];
    q[2] = pts[pid(i + 1, j, k + 1)]; q[3] = pts[pid(i + 1, j, k)];
  };
  auto quadZ = [&](int i, int j, int k, P3* q) {
    q[0] = pts[pid(i, j, k)]; q[1] = pts[pid(i + 1, j, k)];
    q[2] = pts[pid(i + 1, j + 1, k)]; q[3] = pts[pid(i, j + 1, k)];
  };
  auto emit = [&](int f, const P3* q, bool flip) {
    P3 r[4];
    if (flip) { r[0] = q[0]; r[1] = q[3]; r[2] = q[2]; r[3] = q[1]; }
    else { r[0] = q[0]; r[1] = q[1]; r[2] = q[2]; r[3] = q[3]; }
    P3 c, a;
    polygonGeometry(r, 4, c, a);
    Cf[3 * (size_t)f + 0] = c.x; Cf[3 * (size_t)f + 1] = c.y; Cf[3 * (size_t)f + 2] = c.z;
    Sf[3 * (size_t)f + 0] = a.x; Sf[3 * (size_t)f + 1] = a.y; Sf[3 * (size_t)f + 2] = a.z;
  };

  // Internal faces: for each cell in order, its +x, +y, +z faces, which is
  // already sorted by (owner, neighbour) since c+1 < c+nx < c+nx*ny.
  int f = 0;
  P3 q[4];
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        int c = cid(i, j, k);
        if (i + 1 < nx) { owner[f] = c; neighbour[f] = cid(i + 1, j, k); quadX(i + 1, j, k, q); emit(f, q, false); ++f; }
        if (j + 1 < ny) { owner[f] = c; neighbour[f] = cid(i, j + 1, k); quadY(i, j + 1, k, q); emit(f, q, false); ++f; }
        if (k + 1 < nz) { owner[f] = c; neighbour[f] = cid(i, j, k + 1); quadZ(i, j, k + 1, q); emit(f, q, false); ++f; }
      }
  // Boundary patches.
  int p = 0;
  patch_start[p] = f;
  for (int k = 0; k < nz; ++k) for (int j = 0; j < ny; ++j) { owner[f] = cid(0, j, k); quadX(0, j, k, q); emit(f, q, true); ++f; }
  patch_size[p] = f - patch_start[p]; ++p; patch_start[p] = f;
  for (int k = 0; k < nz; ++k) for (int j = 0; j < ny; ++j) { owner[f] = cid(nx - 1, j, k); quadX(nx, j, k, q); emit(f, q, false); ++f; }
  patch_size[p] = f - patch_start[p]; ++p; patch_start[p] = f;
  for (int k = 0; k < nz; ++k) for (int i = 0; i < nx; ++i) { owner[f] = cid(i, 0, k); quadY(i, 0, k, q); emit(f, q, true); ++f; }
  patch_size[p] = f - patch_start[p]; ++p; patch_start[p] = f;
  for (int k = 0; k < nz; ++k) for (int i = 0; i < nx; ++i) { owner[f] = cid(i, ny - 1, k); quadY(i, ny, k, q); emit(f, q, false); ++f; }
  patch_size[p] = f - patch_start[p]; ++p; patch_start[p] = f;
  for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i) { owner[f] = cid(i, j, 0); quadZ(i, j, 0, q); emit(f, q, true); ++f; }
  patch_size[p] = f - patch_start[p]; ++p; patch_start[p] = f;
  for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i) { owner[f] = cid(i, j, nz - 1); quadZ(i, j, nz, q); emit(f, q, false); ++f; }
  patch_size[p] = f - patch_start[p];

  // Cell centres and volumes: pyramids on each face with apex at the average
  // of the cell's face centres.
  std::vector<P3> cEst((size_t)nCells, P3{0, 0, 0});
  std::vector<int> nCellFaces((size_t)nCells, 0);
  for (int g = 0; g < nFaces; ++g) {
    P3 c = {Cf[3 * (size_t)g], Cf[3 * (size_t)g + 1], Cf[3 * (size_t)g + 2]};
    cEst[owner[g]] = add(cEst[owner[g]], c); nCellFaces[owner[g]]++;
    if (g < nInt) { cEst[neighbour[g]] = add(cEst[neighbour[g]], c); nCellFaces[neighbour[g]]++; }
  }
  for (int c = 0; c < nCells; ++c) cEst[c] = scl(1.0 / nCellFaces[c], cEst[c]);
  std::vector<P3> cc((size_t)nCells, P3{0, 0, 0});
  std::vector<double> vv((size_t)nCells, 0.0);
  auto pyr = [&](int cell, int g, bool own) {
    P3 fc = {Cf[3 * (size_t)g], Cf[3 * (size_t)g + 1], Cf[3 * (size_t)g + 2]};
    P3 fa = {Sf[3 * (size_t)g], Sf[3 * (size_t)g + 1], Sf[3 * (size_t)g + 2]};
    double v3 = own ? dot(fa, sub(fc, cEst[cell])) : dot(fa, sub(cEst[cell], fc));
    P3 pc = add(scl(0.75, fc), scl(0.25, cEst[cell]));
    cc[cell] = add(cc[cell], scl(v3, pc));
    vv[cell] += v3;
  };
  for (int g = 0; g < nFaces; ++g) {
    pyr(owner[g], g, true);
    if (g < nInt) pyr(neighbour[g], g, false);
  }
  for (int c = 0; c < nCells; ++c) {
    if (!(vv[c] > 0)) return S4G_BAD_ARG;  // inverted cell: jitter too large
    P3 ctr = scl(1.0 / vv[c], cc[c]);
    C[3 * (size_t)c + 0] = ctr.x; C[3 * (size_t)c + 1] = ctr.y; C[3 * (size_t)c + 2] = ctr.z;
    V[c] = vv[c] / 3.0;
  }
  return S4G_OK;
}

}  // extern "C"
