// Host-side mesh geometry in OpenFOAM's primitiveMesh conventions, shared by
// the box-mesh generator and the polyMesh reader:
//  * face centre and area vector by a triangle fan about the average of the
//    face's points, centre = area-weighted triangle centroids
//    (primitiveMeshFaceCentresAndAreas);
//  * cell centre and volume by pyramids on each face with their apex at the
//    average of the cell's face centres (primitiveMeshCellCentresAndVols).
// Faces are visited in face order and each adds to its owner, then to its
// neighbour, so a mesh handed in twice gives bit-identical geometry.
#pragma once

#include <cmath>
#include <cstddef>
#include <vector>

namespace s4g_host {

struct P3 { double x, y, z; };

inline P3 sub(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline P3 add(P3 a, P3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline P3 scl(double s, P3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline P3 cross(P3 a, P3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double dot(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double mag(P3 a) { return std::sqrt(dot(a, a)); }

// Face centre and area vector of a polygon of n >= 3 points.
inline void polygonGeometry(const P3* pts, int n, P3& ctr, P3& area) {
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

// Cell centres C [nCells][3] and volumes V [nCells] from the face centres
// Cf and area vectors Sf [nFaces][3] (area vectors point out of the owner).
// Returns false if a cell has a volume that is not positive.
inline bool cellGeometry(int nCells, int nFaces, int nInt, const int* owner,
                         const int* neighbour, const double* Cf, const double* Sf,
                         double* C, double* V) {
  std::vector<P3> cEst((size_t)nCells, P3{0, 0, 0});
  std::vector<int> nCellFaces((size_t)nCells, 0);
  for (int g = 0; g < nFaces; ++g) {
    P3 c = {Cf[3 * (size_t)g], Cf[3 * (size_t)g + 1], Cf[3 * (size_t)g + 2]};
    cEst[owner[g]] = add(cEst[owner[g]], c); nCellFaces[owner[g]]++;
    if (g < nInt) { cEst[neighbour[g]] = add(cEst[neighbour[g]], c); nCellFaces[neighbour[g]]++; }
  }
  for (int c = 0; c < nCells; ++c) {
    if (nCellFaces[c] == 0) return false;
    cEst[c] = scl(1.0 / nCellFaces[c], cEst[c]);
  }
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
    if (!(vv[c] > 0)) return false;
    P3 ctr = scl(1.0 / vv[c], cc[c]);
    C[3 * (size_t)c + 0] = ctr.x; C[3 * (size_t)c + 1] = ctr.y; C[3 * (size_t)c + 2] = ctr.z;
    V[c] = vv[c] / 3.0;
  }
  return true;
}

}  // namespace s4g_host
