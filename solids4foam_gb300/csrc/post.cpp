// The steps after the outer-corrector loop, on the host:
//  * pointD: the reference's enhancedVolPointInterpolation::interpolate(D,
//    gradD, pointD) (enhancedVolPointInterpolate.C:351-423, called from
//    mechanicalModel::interpolate, mechanicalModel.C:829-841, after each
//    evolve(), linGeomTotalDispSolid.C:212): every point takes the
//    inverse-distance-weighted average, over all its cells, of the value
//    extrapolated from the cell centre with the cell gradient,
//        pointD_p = sum_c w_pc (D_c + (x_p - C_c) . gradD_c) / sum_c w_pc,
//        w_pc = 1 / |x_p - C_c|;
//  * tractionBoundarySnGrad, for boundary evaluations outside evolve();
//  * the derived fields of solidModel::writeFields (solidModel.C:1936-1962):
//    epsilon = symm(gradD), epsilonEq = sqrt(2/3 |dev epsilon|^2),
//    sigmaEq = sqrt(3/2 |dev sigma|^2).
// Layouts: vector [n][3]; symmTensor [n][6] XX XY XZ YY YZ ZZ; tensor [n][9]
// row-major with gradD_ij = dD_j/dx_i.

#include "s4g.h"
#include "s4g_internal.hpp"

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

namespace {

// |dev(s)|^2 of a symmTensor (double contraction, off-diagonals twice).
double magSqrDev(const double* s) {
  const double tr3 = (s[0] + s[3] + s[5]) / 3.0;
  const double xx = s[0] - tr3, yy = s[3] - tr3, zz = s[5] - tr3;
  return xx * xx + yy * yy + zz * zz + 2.0 * (s[1] * s[1] + s[2] * s[2] + s[4] * s[4]);
}

s4g_status bad(const std::string& msg) {
  s4g::setLastError(msg);
  return S4G_BAD_ARG;
}

}  // namespace

extern "C" {

s4g_status s4g_point_cells(int n_points, int n_faces, const int* face_start,
                           const int* face_points, int n_internal_faces, const int* owner,
                           const int* neighbour, int* point_cell_start, int* point_cells) {
  if (n_points < 0 || n_faces < 0 || n_internal_faces < 0 || n_internal_faces > n_faces ||
      !face_start || !face_points || !owner || (n_internal_faces > 0 && !neighbour) ||
      !point_cell_start)
    return bad("s4g_point_cells: bad arguments");
  // cells of every point, from the faces; sorted and unique per point
  std::vector<std::vector<int>> pc((size_t)n_points);
  for (int f = 0; f < n_faces; ++f) {
    if (face_start[f + 1] < face_start[f]) return bad("s4g_point_cells: decreasing face_start");
    for (int k = face_start[f]; k < face_start[f + 1]; ++k) {
      const int p = face_points[k];
      if (p < 0 || p >= n_points) return bad("s4g_point_cells: face point out of range");
      pc[(size_t)p].push_back(owner[f]);
      if (f < n_internal_faces) pc[(size_t)p].push_back(neighbour[f]);
    }
  }
  point_cell_start[0] = 0;
  for (int p = 0; p < n_points; ++p) {
    std::vector<int>& v = pc[(size_t)p];
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    point_cell_start[p + 1] = point_cell_start[p] + (int)v.size();
    if (point_cells)
      for (size_t i = 0; i < v.size(); ++i) point_cells[point_cell_start[p] + (int)i] = v[i];
  }
  return S4G_OK;
}

s4g_status s4g_point_interpolate(int n_points, const double* points, const int* point_cell_start,
                                 const int* point_cells, int n_cells, const double* C,
                                 const double* D, const double* gradD, double* pointD) {
  if (n_points < 0 || n_cells < 0 || !points || !point_cell_start || !point_cells || !C || !D ||
      !gradD || !pointD)
    return bad("s4g_point_interpolate: bad arguments");
  for (int p = 0; p < n_points; ++p) {
    const double* x = points + 3 * (size_t)p;
    double acc[3] = {0, 0, 0}, sumW = 0;
    for (int k = point_cell_start[p]; k < point_cell_start[p + 1]; ++k) {
      const int c = point_cells[k];
      if (c < 0 || c >= n_cells) return bad("s4g_point_interpolate: cell out of range");
      const double* cc = C + 3 * (size_t)c;
      const double d[3] = {x[0] - cc[0], x[1] - cc[1], x[2] - cc[2]};
      const double w = 1.0 / std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      const double* g = gradD + 9 * (size_t)c;
      const double* u = D + 3 * (size_t)c;
      for (int j = 0; j < 3; ++j)  // (delta & gradD)_j = delta_i gradD_ij
        acc[j] += w * (u[j] + (d[0] * g[j] + d[1] * g[3 + j] + d[2] * g[6 + j]));
      sumW += w;
    }
    // normalised where the weight sum exceeds OpenFOAM's ROOTVSMALL
    for (int j = 0; j < 3; ++j) pointD[3 * (size_t)p + j] = sumW > 1e-150 ? acc[j] / sumW : acc[j];
  }
  return S4G_OK;
}

s4g_status s4g_traction_sngrad(int n_faces, const double* traction, const double* pressure,
                               const double* normal, const double* sigma_b, const double* gradD_b,
                               const double* Finv_b, double impK, double* g_out) {
  if (n_faces < 0 || !normal || !sigma_b || !gradD_b || !g_out || !(impK > 0))
    return bad("s4g_traction_sngrad: bad arguments");
  for (int f = 0; f < n_faces; ++f) {
    const double* n = normal + 3 * (size_t)f;
    const double* s = sigma_b + 6 * (size_t)f;
    const double* G = gradD_b + 9 * (size_t)f;
    double nc[3] = {n[0], n[1], n[2]};
    if (Finv_b) {  // deformed normal Finv^T & n, normalised
      const double* Fi = Finv_b + 9 * (size_t)f;
      for (int j = 0; j < 3; ++j) nc[j] = n[0] * Fi[j] + n[1] * Fi[3 + j] + n[2] * Fi[6 + j];
      const double m = std::sqrt(nc[0] * nc[0] + nc[1] * nc[1] + nc[2] * nc[2]);
      if (!(m > 0)) return bad("s4g_traction_sngrad: degenerate deformed normal");
      for (double& v : nc) v /= m;
    }
    const double S[3][3] = {{s[0], s[1], s[2]}, {s[1], s[3], s[4]}, {s[2], s[4], s[5]}};
    const double p = pressure ? pressure[f] : 0.0;
    for (int j = 0; j < 3; ++j) {
      const double t = traction ? traction[3 * (size_t)f + j] : 0.0;
      const double ncSig = nc[0] * S[0][j] + nc[1] * S[1][j] + nc[2] * S[2][j];
      const double nG = n[0] * G[j] + n[1] * G[3 + j] + n[2] * G[6 + j];
      g_out[3 * (size_t)f + j] = ((t - nc[j] * p) - ncSig + impK * nG) / impK;
    }
  }
  return S4G_OK;
}

s4g_status s4g_derived_fields(int n, const double* sigma, const double* gradD, double* sigmaEq,
                              double* epsilon, double* epsilonEq) {
  if (n < 0 || (sigmaEq && !sigma) || ((epsilon || epsilonEq) && !gradD))
    return bad("s4g_derived_fields: bad arguments");
  for (int c = 0; c < n; ++c) {
    if (sigmaEq) sigmaEq[c] = std::sqrt(1.5 * magSqrDev(sigma + 6 * (size_t)c));
    if (epsilon || epsilonEq) {
      const double* g = gradD + 9 * (size_t)c;
      const double e[6] = {g[0], 0.5 * (g[1] + g[3]), 0.5 * (g[2] + g[6]),
                           g[4], 0.5 * (g[5] + g[7]), g[8]};
      if (epsilon)
        for (int k = 0; k < 6; ++k) epsilon[6 * (size_t)c + k] = e[k];
      if (epsilonEq) epsilonEq[c] = std::sqrt((2.0 / 3.0) * magSqrDev(e));
    }
  }
  return S4G_OK;
}

}  // extern "C"
