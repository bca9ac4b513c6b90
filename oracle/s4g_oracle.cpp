// CPU FP64 oracle for the segregated finite-volume solid solve.
//
// TEST INFRASTRUCTURE ONLY: loaded by the tests, the smoke check and the CPU
// baseline leg of the benchmark, never by the product.
//
// Restated from the reference (paths relative to the solids4foam tree):
//  * outer loop:        src/solids4FoamModels/solidModels/linGeomTotalDispSolid/
//                       linGeomTotalDispSolid.C:111-232 (traction snGrad :235-271)
//  * TL outer loop:     .../nonLinGeomTotalLagSolid/nonLinGeomTotalLagSolid.C:125-260
//                       (traction snGrad :263-325)
//  * converged():       .../solidModel/solidModelTemplates.C:26-188
//  * checkEnforceLinear .../solidModel/solidModel.C:1894-1913
//  * RhieChow:          .../solidModel/momentumStabilisation/momentumStabilisation.C:79-217
//  * laws:              .../linearElastic/linearElastic.C:62-133,204-245,318-339;
//                       .../neoHookeanElastic/neoHookeanElastic.C:50-79,101-119,275-303;
//                       .../mechanicalLaw/mechanicalLaw.C:983-1001,1095-1159
//  * BCs:               .../solidTraction/solidTractionFvPatchVectorField.C:321-463;
//                       .../fixedDisplacement/fixedDisplacementFvPatchVectorField.C:258-356;
//                       numerics/patchCorrectionVectors/patchCorrectionVectors.C:24-36
// OpenFOAM operators (third-party, not in the tree; written from the published
// finite-volume formulation, with the conventions: linear weights
// |S.(C_N-C_f)|/(|S.(C_f-C_P)|+|S.(C_N-C_f)|), deltaCoeffs 1/max(n.d, 0.05|d|),
// boundary deltaCoeffs 1/(n.(C_f-C_P)), RhieChow gamma = 0 on boundary faces):
// fvm/fvc::laplacian Gauss linear corrected, fvc::div Gauss linear,
// leastSquares gradient with boundary snGrad correction, linear interpolation,
// PCG with DIC and OpenFOAM's residual normalisation.
//
// Face loops are written cell-centrically: every cell visits its faces in
// increasing face index, which reproduces the accumulation order of the
// face-ordered OpenFOAM loops (owner +flux, neighbour -flux) exactly.

#include "s4g_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double SMALL = 1e-15;
const double VSMALL = 1e-300;

struct V3 { double x, y, z; };
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3& operator+=(V3& a, V3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
inline V3& operator-=(V3& a, V3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double mag(V3 a) { return std::sqrt(dot(a, a)); }
inline double magSqr(V3 a) { return dot(a, a); }

// Full tensor, row-major: T_ij, i = derivative direction for gradients
// (OpenFOAM: grad(D)_ij = d D_j / d x_i).
struct T9 { double xx, xy, xz, yx, yy, yz, zx, zy, zz; };
// Symmetric tensor XX XY XZ YY YZ ZZ.
struct S6 { double xx, xy, xz, yy, yz, zz; };

inline T9 zeroT() { return {0, 0, 0, 0, 0, 0, 0, 0, 0}; }
inline T9 identT() { return {1, 0, 0, 0, 1, 0, 0, 0, 1}; }
inline S6 zeroS() { return {0, 0, 0, 0, 0, 0}; }
inline T9 operator+(const T9& a, const T9& b) {
  return {a.xx + b.xx, a.xy + b.xy, a.xz + b.xz, a.yx + b.yx, a.yy + b.yy,
          a.yz + b.yz, a.zx + b.zx, a.zy + b.zy, a.zz + b.zz};
}
inline T9 operator-(const T9& a, const T9& b) {
  return {a.xx - b.xx, a.xy - b.xy, a.xz - b.xz, a.yx - b.yx, a.yy - b.yy,
          a.yz - b.yz, a.zx - b.zx, a.zy - b.zy, a.zz - b.zz};
}
inline T9 operator*(double s, const T9& a) {
  return {s * a.xx, s * a.xy, s * a.xz, s * a.yx, s * a.yy, s * a.yz,
          s * a.zx, s * a.zy, s * a.zz};
}
inline T9& operator+=(T9& a, const T9& b) { a = a + b; return a; }
// a (x) b : T_ij = a_i b_j
inline T9 outer(V3 a, V3 b) {
  return {a.x * b.x, a.x * b.y, a.x * b.z, a.y * b.x, a.y * b.y,
          a.y * b.z, a.z * b.x, a.z * b.y, a.z * b.z};
}
// v & T : (v.T)_j = sum_i v_i T_ij
inline V3 dotVT(V3 v, const T9& t) {
  return {v.x * t.xx + v.y * t.yx + v.z * t.zx,
          v.x * t.xy + v.y * t.yy + v.z * t.zy,
          v.x * t.xz + v.y * t.yz + v.z * t.zz};
}
inline T9 transposeT(const T9& t) {
  return {t.xx, t.yx, t.zx, t.xy, t.yy, t.zy, t.xz, t.yz, t.zz};
}
inline T9 dotTT(const T9& a, const T9& b) {
  return {a.xx * b.xx + a.xy * b.yx + a.xz * b.zx,
          a.xx * b.xy + a.xy * b.yy + a.xz * b.zy,
          a.xx * b.xz + a.xy * b.yz + a.xz * b.zz,
          a.yx * b.xx + a.yy * b.yx + a.yz * b.zx,
          a.yx * b.xy + a.yy * b.yy + a.yz * b.zy,
          a.yx * b.xz + a.yy * b.yz + a.yz * b.zz,
          a.zx * b.xx + a.zy * b.yx + a.zz * b.zx,
          a.zx * b.xy + a.zy * b.yy + a.zz * b.zy,
          a.zx * b.xz + a.zy * b.yz + a.zz * b.zz};
}
inline double detT(const T9& t) {
  return t.xx * (t.yy * t.zz - t.yz * t.zy) - t.xy * (t.yx * t.zz - t.yz * t.zx) +
         t.xz * (t.yx * t.zy - t.yy * t.zx);
}
inline T9 invT(const T9& t) {
  double d = detT(t);
  T9 c = {t.yy * t.zz - t.yz * t.zy, t.xz * t.zy - t.xy * t.zz, t.xy * t.yz - t.xz * t.yy,
          t.yz * t.zx - t.yx * t.zz, t.xx * t.zz - t.xz * t.zx, t.xz * t.yx - t.xx * t.yz,
          t.yx * t.zy - t.yy * t.zx, t.xy * t.zx - t.xx * t.zy, t.xx * t.yy - t.xy * t.yx};
  return (1.0 / d) * c;
}
inline S6 symmT(const T9& t) {
  return {t.xx, 0.5 * (t.xy + t.yx), 0.5 * (t.xz + t.zx), t.yy,
          0.5 * (t.yz + t.zy), t.zz};
}
inline T9 fromS(const S6& s) {
  return {s.xx, s.xy, s.xz, s.xy, s.yy, s.yz, s.xz, s.yz, s.zz};
}
inline double trS(const S6& s) { return s.xx + s.yy + s.zz; }
inline double trT(const T9& t) { return t.xx + t.yy + t.zz; }
inline S6 devS(const S6& s) {
  double m = trS(s) / 3.0;
  return {s.xx - m, s.xy, s.xz, s.yy - m, s.yz, s.zz - m};
}
inline S6 operator+(const S6& a, const S6& b) {
  return {a.xx + b.xx, a.xy + b.xy, a.xz + b.xz, a.yy + b.yy, a.yz + b.yz, a.zz + b.zz};
}
inline S6 operator*(double s, const S6& a) {
  return {s * a.xx, s * a.xy, s * a.xz, s * a.yy, s * a.yz, s * a.zz};
}
inline S6 addI(const S6& a, double s) {
  return {a.xx + s, a.xy, a.xz, a.yy + s, a.yz, a.zz + s};
}
// v & S
inline V3 dotVS(V3 v, const S6& s) {
  return {v.x * s.xx + v.y * s.xy + v.z * s.xz,
          v.x * s.xy + v.y * s.yy + v.z * s.yz,
          v.x * s.xz + v.y * s.yz + v.z * s.zz};
}
// inverse of a symmetric tensor (full rank)
inline S6 invS(const S6& s) {
  double d = s.xx * (s.yy * s.zz - s.yz * s.yz) - s.xy * (s.xy * s.zz - s.yz * s.xz) +
             s.xz * (s.xy * s.yz - s.yy * s.xz);
  S6 c = {s.yy * s.zz - s.yz * s.yz, s.xz * s.yz - s.xy * s.zz, s.xy * s.yz - s.xz * s.yy,
          s.xx * s.zz - s.xz * s.xz, s.xy * s.xz - s.xx * s.yz, s.xx * s.yy - s.xy * s.xy};
  return (1.0 / d) * c;
}

inline V3 getV(const double* a, long i) { return {a[3 * i], a[3 * i + 1], a[3 * i + 2]}; }

// ---------------------------------------------------------------- mesh ---

struct Mesh {
  int nC = 0, nF = 0, nI = 0, nB = 0;
  std::vector<int> own, nei;
  std::vector<V3> C, Cf, Sf;
  std::vector<double> V;
  std::vector<int> pStart, pSize;  // absolute face index
  std::vector<int> patchOfB;       // boundary face -> patch

  // derived geometry (OpenFOAM surfaceInterpolation / fvPatch conventions)
  std::vector<double> magSf;         // nF
  std::vector<V3> nf;                // nF unit normals
  std::vector<double> w;             // nI linear weights (owner side)
  std::vector<double> nonOrthDelta;  // nI
  std::vector<V3> corrVec;           // nI nonOrthCorrectionVectors
  std::vector<double> bDelta;        // nB boundary deltaCoeffs
  std::vector<V3> kb;                // nB patchCorrectionVectors
  std::vector<V3> lsP, lsN;          // nI leastSquares vectors
  std::vector<V3> lsB;               // nB

  // cell -> internal faces (increasing face index), cell -> boundary faces
  std::vector<int> cfStart, cfFace, cbStart, cbFace;
  std::vector<int> newOfCaller;  // caller cell -> solver cell

  bool build(const orc_mesh_desc* d, const int* perm, int lsBoundaryDelta, int emptyDir = 0);
};

bool Mesh::build(const orc_mesh_desc* d, const int* perm, int lsBoundaryDelta, int emptyDir) {
  nC = d->n_cells; nF = d->n_faces; nI = d->n_internal_faces; nB = nF - nI;
  if (nC <= 0 || nI < 0 || nB < 0) return false;
  std::vector<int> newOf(nC);
  if (perm) {
    std::vector<char> seen(nC, 0);
    for (int i = 0; i < nC; ++i) {
      if (perm[i] < 0 || perm[i] >= nC || seen[perm[i]]) return false;
      seen[perm[i]] = 1;
      newOf[perm[i]] = i;
    }
  } else {
    std::iota(newOf.begin(), newOf.end(), 0);
  }
  newOfCaller = newOf;
  C.resize(nC); V.resize(nC);
  for (int c = 0; c < nC; ++c) {
    C[newOf[c]] = getV(d->C, c);
    V[newOf[c]] = d->V[c];
  }
  // Internal faces: renumber, flip to owner < neighbour, sort upper-triangular
  // (as OpenFOAM's renumberMesh does).
  struct IF { int o, n; V3 cf, sf; };
  std::vector<IF> fi(nI);
  for (int f = 0; f < nI; ++f) {
    int o = newOf[d->owner[f]], n = newOf[d->neighbour[f]];
    V3 sf = getV(d->Sf, f);
    if (o > n) { std::swap(o, n); sf = -1.0 * sf; }
    if (o == n) return false;
    fi[f] = {o, n, getV(d->Cf, f), sf};
  }
  std::stable_sort(fi.begin(), fi.end(), [](const IF& a, const IF& b) {
    return a.o != b.o ? a.o < b.o : a.n < b.n;
  });
  own.resize(nF); nei.resize(nI); Cf.resize(nF); Sf.resize(nF);
  for (int f = 0; f < nI; ++f) { own[f] = fi[f].o; nei[f] = fi[f].n; Cf[f] = fi[f].cf; Sf[f] = fi[f].sf; }
  for (int f = nI; f < nF; ++f) {
    own[f] = newOf[d->owner[f]];
    Cf[f] = getV(d->Cf, f); Sf[f] = getV(d->Sf, f);
  }
  pStart.assign(d->patch_start, d->patch_start + d->n_patches);
  pSize.assign(d->patch_size, d->patch_size + d->n_patches);
  patchOfB.assign(nB, -1);
  for (int p = 0; p < d->n_patches; ++p)
    for (int i = 0; i < pSize[p]; ++i) {
      int b = pStart[p] + i - nI;
      if (b < 0 || b >= nB) return false;
      patchOfB[b] = p;
    }
  for (int b = 0; b < nB; ++b) if (patchOfB[b] < 0) return false;

  magSf.resize(nF); nf.resize(nF);
  for (int f = 0; f < nF; ++f) { magSf[f] = mag(Sf[f]); nf[f] = (1.0 / magSf[f]) * Sf[f]; }

  // surfaceInterpolation::makeWeights
  w.resize(nI); nonOrthDelta.resize(nI); corrVec.resize(nI);
  for (int f = 0; f < nI; ++f) {
    double sfdOwn = std::fabs(dot(Sf[f], Cf[f] - C[own[f]]));
    double sfdNei = std::fabs(dot(Sf[f], C[nei[f]] - Cf[f]));
    w[f] = sfdNei / (sfdOwn + sfdNei);
    V3 dl = C[nei[f]] - C[own[f]];
    // stabilised non-orthogonal delta: 1/max(n.d, 0.05|d|)
    nonOrthDelta[f] = 1.0 / std::max(dot(nf[f], dl), 0.05 * mag(dl));
    corrVec[f] = nf[f] - nonOrthDelta[f] * dl;
  }
  // boundary: patch-normal delta n (n.(Cf - C)) for non-coupled patches
  bDelta.resize(nB); kb.resize(nB);
  std::vector<V3> dB(nB);
  for (int b = 0; b < nB; ++b) {
    int f = nI + b;
    V3 dfull = Cf[f] - C[own[f]];
    V3 dn = dot(nf[f], dfull) * nf[f];
    bDelta[b] = 1.0 / mag(dn);
    kb[b] = dfull - dot(nf[f], dfull) * nf[f];  // (I - n n) & (Cf - C)
    dB[b] = lsBoundaryDelta ? dfull : dn;
  }

  // cell -> faces
  cfStart.assign(nC + 1, 0); cbStart.assign(nC + 1, 0);
  for (int f = 0; f < nI; ++f) { cfStart[own[f] + 1]++; cfStart[nei[f] + 1]++; }
  for (int b = 0; b < nB; ++b) cbStart[own[nI + b] + 1]++;
  for (int c = 0; c < nC; ++c) { cfStart[c + 1] += cfStart[c]; cbStart[c + 1] += cbStart[c]; }
  cfFace.resize(2 * (size_t)nI); cbFace.resize(nB);
  {
    std::vector<int> fill(cfStart.begin(), cfStart.end() - 1);
    for (int f = 0; f < nI; ++f) { cfFace[fill[own[f]]++] = f; cfFace[fill[nei[f]]++] = f; }
    std::vector<int> fb(cbStart.begin(), cbStart.end() - 1);
    for (int b = 0; b < nB; ++b) cbFace[fb[own[nI + b]]++] = b;
  }

  // leastSquaresVectors: dd = sum d d^T/|d|^2 over internal and boundary faces
  std::vector<S6> dd(nC, zeroS());
  for (int c = 0; c < nC; ++c) {
    S6 acc = zeroS();
    for (int e = cfStart[c]; e < cfStart[c + 1]; ++e) {
      int f = cfFace[e];
      V3 dl = C[nei[f]] - C[own[f]];
      double r = 1.0 / magSqr(dl);
      S6 wdd = {r * dl.x * dl.x, r * dl.x * dl.y, r * dl.x * dl.z,
                r * dl.y * dl.y, r * dl.y * dl.z, r * dl.z * dl.z};
      acc = acc + wdd;
    }
    for (int e = cbStart[c]; e < cbStart[c + 1]; ++e) {
      V3 dl = dB[cbFace[e]];
      double r = 1.0 / magSqr(dl);
      S6 wdd = {r * dl.x * dl.x, r * dl.x * dl.y, r * dl.x * dl.z,
                r * dl.y * dl.y, r * dl.y * dl.z, r * dl.z * dl.z};
      acc = acc + wdd;
    }
    dd[c] = acc;
  }
  // In a 2-D mesh dd has no component along the empty direction: as
  // OpenFOAM's inv(symmTensorField) does, add 1 there, invert, and take the
  // 1 away again, so the gradient has no derivative across it.
  auto addEmpty = [emptyDir](S6 s, double v) {
    if (emptyDir == 1) s.xx += v;
    else if (emptyDir == 2) s.yy += v;
    else if (emptyDir == 3) s.zz += v;
    return s;
  };
  std::vector<S6> invDd(nC);
  for (int c = 0; c < nC; ++c) invDd[c] = addEmpty(invS(addEmpty(dd[c], 1.0)), -1.0);
  lsP.resize(nI); lsN.resize(nI); lsB.resize(nB);
  for (int f = 0; f < nI; ++f) {
    V3 dl = C[nei[f]] - C[own[f]];
    double r = 1.0 / magSqr(dl);
    lsP[f] = r * dotVS(dl, invDd[own[f]]);
    lsN[f] = -r * dotVS(dl, invDd[nei[f]]);
  }
  for (int b = 0; b < nB; ++b) {
    V3 dl = dB[b];
    lsB[b] = (1.0 / magSqr(dl)) * dotVS(dl, invDd[own[nI + b]]);
  }
  return true;
}

// ----------------------------------------------------------- LDU / PCG ---

struct Ldu {
  std::vector<double> diag, upper;
};

// y = A x, face-order accumulation per cell.
void amul(const Mesh& m, const Ldu& A, const double* x, double* y, int nt) {
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
  for (int c = 0; c < m.nC; ++c) {
    double acc = A.diag[c] * x[c];
    for (int e = m.cfStart[c]; e < m.cfStart[c + 1]; ++e) {
      int f = m.cfFace[e];
      int o = (m.own[f] == c) ? m.nei[f] : m.own[f];
      acc += A.upper[f] * x[o];
    }
    y[c] = acc;
  }
}

// DIC preconditioner (OpenFOAM DICPreconditioner semantics).  The factor and
// the sweeps ignore faces that couple different subdomains (processor-local
// DIC, as in a decomposed run): the thread subdomains with nt > 1, or the
// caller's cell-to-subdomain map when one is given.
struct Dic {
  std::vector<double> rD;
  std::vector<int> dom;  // subdomain of each cell
  int nd = 1;            // thread subdomains: contiguous ranges of cells
  int nthreads = 1;
  bool callerDomains = false;
  std::vector<int> domStart, domCells;  // caller subdomains: their cells, ascending
  void build(const Mesh& m, const Ldu& A, int nt, const std::vector<int>* domain = nullptr) {
    nthreads = std::max(1, nt);
    nd = nthreads;
    dom.resize(m.nC);
    for (int c = 0; c < m.nC; ++c) dom[c] = (int)((long long)c * nd / m.nC);
    if (domain) {
      dom = *domain;
      callerDomains = true;
      int n = 0;
      for (int c = 0; c < m.nC; ++c) n = std::max(n, dom[c] + 1);
      domStart.assign(n + 1, 0);
      for (int c = 0; c < m.nC; ++c) domStart[dom[c] + 1]++;
      for (int d = 0; d < n; ++d) domStart[d + 1] += domStart[d];
      domCells.resize(m.nC);
      std::vector<int> fill(domStart.begin(), domStart.end() - 1);
      for (int c = 0; c < m.nC; ++c) domCells[fill[dom[c]]++] = c;
    }
    rD = A.diag;
    // calcReciprocalD: rD[u] -= upper^2/rD[l] over faces in order
    for (int u = 0; u < m.nC; ++u)
      for (int e = m.cfStart[u]; e < m.cfStart[u + 1]; ++e) {
        int f = m.cfFace[e];
        int l = m.own[f];
        if (m.nei[f] != u || dom[l] != dom[u]) continue;
        rD[u] -= A.upper[f] * A.upper[f] / rD[l];
      }
    for (int c = 0; c < m.nC; ++c) rD[c] = 1.0 / rD[c];
  }
  // The substitutions of one subdomain; the cells are visited in increasing
  // (forward) and decreasing (backward) order, given as a list or a range.
  template <class CellAt>
  void sweep(const Mesh& m, const Ldu& A, const double* r, double* wv, int n, CellAt at) const {
    for (int q = 0; q < n; ++q) {
      const int u = at(q);
      double v = rD[u] * r[u];
      for (int e = m.cfStart[u]; e < m.cfStart[u + 1]; ++e) {
        int f = m.cfFace[e];
        if (m.nei[f] != u) continue;
        int l = m.own[f];
        if (dom[l] != dom[u]) continue;
        v -= rD[u] * A.upper[f] * wv[l];
      }
      wv[u] = v;
    }
    for (int q = n - 1; q >= 0; --q) {
      const int l = at(q);
      double v = wv[l];
      for (int e = m.cfStart[l + 1] - 1; e >= m.cfStart[l]; --e) {
        int f = m.cfFace[e];
        if (m.own[f] != l) continue;
        int u = m.nei[f];
        if (dom[u] != dom[l]) continue;
        v -= rD[l] * A.upper[f] * wv[u];
      }
      wv[l] = v;
    }
  }
  void apply(const Mesh& m, const Ldu& A, const double* r, double* wv) const {
    if (callerDomains) {
      // the subdomains are independent: in parallel, each in cell order
      const int n = (int)domStart.size() - 1;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads) if (nthreads > 1)
      for (int d = 0; d < n; ++d) {
        const int* cells = domCells.data() + domStart[d];
        sweep(m, A, r, wv, domStart[d + 1] - domStart[d], [&](int q) { return cells[q]; });
      }
    } else if (nd == 1) {
      sweep(m, A, r, wv, m.nC, [](int q) { return q; });
    } else {
#pragma omp parallel for schedule(static, 1) num_threads(nd)
      for (int d = 0; d < nd; ++d) {
        int c0 = (int)(((long long)d * m.nC + nd - 1) / nd);
        int c1 = (int)(((long long)(d + 1) * m.nC + nd - 1) / nd);
        sweep(m, A, r, wv, c1 - c0, [&](int q) { return c0 + q; });
      }
    }
  }
};

double sumMag(const std::vector<double>& a, int nt) {
  double s = 0;
#pragma omp parallel for reduction(+ : s) num_threads(nt) if (nt > 1)
  for (long i = 0; i < (long)a.size(); ++i) s += std::fabs(a[i]);
  return s;
}
double sumProd(const std::vector<double>& a, const std::vector<double>& b, int nt) {
  double s = 0;
#pragma omp parallel for reduction(+ : s) num_threads(nt) if (nt > 1)
  for (long i = 0; i < (long)a.size(); ++i) s += a[i] * b[i];
  return s;
}

struct SolverPerf { double initRes = 0, finalRes = 0; int nIter = 0; };

// OpenFOAM PCG (lduMatrix solver) with normFactor residual normalisation.
SolverPerf pcg(const Mesh& m, const Ldu& A, const Dic* dic,
               const std::vector<double>& b, std::vector<double>& x,
               double tol, double relTol, int maxIter, int nt) {
  const int n = m.nC;
  SolverPerf sp;
  std::vector<double> wA(n), rA(n), pA(n, 0.0), tmp(n);
  amul(m, A, x.data(), wA.data(), nt);
  for (int i = 0; i < n; ++i) rA[i] = b[i] - wA[i];
  // normFactor: sumA = row sums; xRef = average(x)
  double xRef = 0;
  for (int i = 0; i < n; ++i) xRef += x[i];
  xRef /= n;
  for (int c = 0; c < n; ++c) {
    double s = A.diag[c];
    for (int e = m.cfStart[c]; e < m.cfStart[c + 1]; ++e) s += A.upper[m.cfFace[e]];
    tmp[c] = s * xRef;
  }
  double normFactor = 0;
  for (int i = 0; i < n; ++i)
    normFactor += std::fabs(wA[i] - tmp[i]) + std::fabs(b[i] - tmp[i]);
  normFactor += 1e-20;
  sp.initRes = sumMag(rA, nt) / normFactor;
  sp.finalRes = sp.initRes;
  auto converged = [&]() {
    return sp.finalRes < tol || (relTol > 1e-20 && sp.finalRes < relTol * sp.initRes);
  };
  if (converged()) return sp;
  double wArA = 1e300, wArAold = 0;
  do {
    wArAold = wArA;
    if (dic) dic->apply(m, A, rA.data(), wA.data());
    else for (int i = 0; i < n; ++i) wA[i] = rA[i] / A.diag[i];
    wArA = sumProd(wA, rA, nt);
    if (sp.nIter == 0) {
      for (int i = 0; i < n; ++i) pA[i] = wA[i];
    } else {
      double beta = wArA / wArAold;
      for (int i = 0; i < n; ++i) pA[i] = wA[i] + beta * pA[i];
    }
    amul(m, A, pA.data(), wA.data(), nt);
    double wApA = sumProd(wA, pA, nt);
    if (std::fabs(wApA) / normFactor < 1e-300) break;  // singular
    double alpha = wArA / wApA;
#pragma omp parallel for num_threads(nt) if (nt > 1)
    for (int i = 0; i < n; ++i) { x[i] += alpha * pA[i]; rA[i] -= alpha * wA[i]; }
    sp.finalRes = sumMag(rA, nt) / normFactor;
  } while (++sp.nIter < maxIter && !converged());
  return sp;
}

// -------------------------------------------------------------- solver ---

struct Bc {
  int type;
  std::vector<V3> value;   // per patch face
  std::vector<double> p;   // per patch face
  double relax = 1.0;      // relaxationFactor (traction patches)
};

struct Solver {
  const Mesh& m;
  const orc_settings& s;
  std::vector<Bc> bcs;
  int nt;
  bool tl;                 // total Lagrangian (either form)
  bool incr;               // incremental form (solves DD); else total D
  double mu, K, lambda, impK, rImpK;
  double loadFactor = 1.0;

  // fields (cells + boundary faces)
  std::vector<V3> U, Ub;         // the solved field: D (linear) or DD (TL)
  std::vector<T9> G, Gb;         // grad of the solved field
  std::vector<S6> sig, sigb;
  std::vector<V3> g;             // traction snGrad per boundary face
  std::vector<V3> D, Db, D0, D0b;  // total displacement and old time
  std::vector<T9> GD, GDb, GD0, GD0b;  // TL: total gradient and old
  std::vector<T9> Finv, Finvb;   // TL: solver F inverse
  std::vector<double> J, Jb;
  std::vector<T9> FL, FLb, FL0, FL0b;  // TL: law's F and F.oldTime
  std::vector<S6> sig0, sig0b;
  bool enforceLinear = false;
  // Aitken relaxation (solidModel.C:842-896): aitkenAlpha and aitkenResidual,
  // volScalarField 1 and volVectorField 0 at construction (calculated
  // patches: cells and every boundary face)
  std::vector<double> aitA, aitAb;
  std::vector<V3> aitR, aitRb;

  Ldu A;
  Dic dic;
  orc_perf perf{};

  Solver(const Mesh& mesh, const orc_settings& st, const orc_bc* in)
      : m(mesh), s(st) {
    nt = std::max(1, s.n_threads);
    tl = s.model == ORC_NONLIN_GEOM_TOTAL_LAG || s.model == ORC_NONLIN_GEOM_TOTAL_LAG_TOTAL_DISP;
    incr = s.model == ORC_NONLIN_GEOM_TOTAL_LAG;
    if (s.use_mu_K) {
      mu = s.mu; K = s.K; lambda = K - 2.0 * mu / 3.0;
    } else {
      mu = s.E / (2.0 * (1.0 + s.nu));
      lambda = s.nu * s.E / ((1.0 + s.nu) * (1.0 - 2.0 * s.nu));
      K = (s.nu * s.E / ((1.0 + s.nu) * (1.0 - 2.0 * s.nu))) + (2.0 / 3.0) * mu;
    }
    if (s.law == ORC_LINEAR_ELASTIC) {
      // linearElastic.C:62-133: K = E/(3(1-2nu)) in the 3-D branch
      if (!s.use_mu_K) K = s.E / (3.0 * (1.0 - 2.0 * s.nu));
      impK = 2.0 * mu + lambda;
    } else {
      impK = (4.0 / 3.0) * mu + K;
    }
    rImpK = 1.0 / impK;
    bcs.resize(m.pStart.size());
    for (size_t p = 0; p < bcs.size(); ++p) {
      bcs[p].type = in[p].type;
      bcs[p].relax = in[p].relaxation_factor > 0 ? in[p].relaxation_factor : 1.0;
      int n = m.pSize[p];
      bcs[p].value.assign(n, V3{0, 0, 0});
      bcs[p].p.assign(n, 0.0);
      for (int i = 0; i < n; ++i) {
        if (in[p].value) bcs[p].value[i] = getV(in[p].value, i);
        if (in[p].pressure) bcs[p].p[i] = in[p].pressure[i];
      }
    }
    int nC = m.nC, nB = m.nB;
    U.assign(nC, V3{0, 0, 0}); Ub.assign(nB, V3{0, 0, 0});
    G.assign(nC, zeroT()); Gb.assign(nB, zeroT());
    sig.assign(nC, zeroS()); sigb.assign(nB, zeroS());
    g.assign(nB, V3{0, 0, 0});
    D = U; Db = Ub; D0 = U; D0b = Ub;
    if (tl) {
      GD = G; GDb = Gb; GD0 = G; GD0b = Gb;
      Finv.assign(nC, identT()); Finvb.assign(nB, identT());
      J.assign(nC, 1.0); Jb.assign(nB, 1.0);
      FL = Finv; FLb = Finvb; FL0 = FL; FL0b = FLb;
      sig0 = sig; sig0b = sigb;
    }
    assembleMatrix();
    if (s.preconditioner == ORC_DIC) {
      if (s.dic_domain) {
        std::vector<int> dom(m.nC);
        for (int c = 0; c < m.nC; ++c) dom[m.newOfCaller[c]] = s.dic_domain[c];
        dic.build(m, A, nt, &dom);
      } else {
        dic.build(m, A, nt);
      }
    }
  }

  int patchType(int b) const { return bcs[m.patchOfB[b]].type; }
  int patchLocal(int b) const { return m.nI + b - m.pStart[m.patchOfB[b]]; }

  // fvm::laplacian(impKf, U) negated by '==': SPD LDU matrix.
  void assembleMatrix() {
    A.diag.assign(m.nC, 0.0);
    A.upper.resize(m.nI);
    for (int f = 0; f < m.nI; ++f) A.upper[f] = m.nonOrthDelta[f] * (impK * m.magSf[f]);
    for (int c = 0; c < m.nC; ++c) {
      double d = 0;
      for (int e = m.cfStart[c]; e < m.cfStart[c + 1]; ++e) d -= A.upper[m.cfFace[e]];
      for (int e = m.cbStart[c]; e < m.cbStart[c + 1]; ++e) {
        int b = m.cbFace[e];
        if (patchType(b) == ORC_FIXED_DISPLACEMENT)
          d += impK * m.magSf[m.nI + b] * (-m.bDelta[b]);  // internalCoeffs
      }
      A.diag[c] = -d;
    }
    for (int f = 0; f < m.nI; ++f) A.upper[f] = -A.upper[f];
  }

  // Fixed displacement value of the solved field on face b.
  V3 fixedValue(int b) const {
    V3 v = loadFactor * bcs[m.patchOfB[b]].value[patchLocal(b)];
    if (incr) v -= D0b[b];  // fixedDisplacement...C:273-285: DD = D - D.oldTime
    return v;
  }

  // solidTraction::updateCoeffs (solidTraction...C:321-395) with the model's
  // tractionBoundarySnGrad, relaxed against the previous gradient
  // (solidTraction...C:387-392): g = f g_new + (1 - f) g.
  void updateTraction() {
    for (int b = 0; b < m.nB; ++b) {
      if (patchType(b) != ORC_SOLID_TRACTION) continue;
      const Bc& bc = bcs[m.patchOfB[b]];
      int i = patchLocal(b);
      V3 t = loadFactor * bc.value[i];
      double p = loadFactor * bc.p[i];
      V3 n = m.nf[m.nI + b];
      V3 gn;
      if (!tl) {
        // linGeomTotalDispSolid.C:261-270
        T9 a = fromS(sigb[b]) - impK * Gb[b];
        gn = rImpK * ((t - p * n) - dotVT(n, a));
      } else if (enforceLinear) {
        // nonLinGeomTotalLagSolid.C:296-305
        gn = rImpK * ((t - p * n) - dotVS(n, sigb[b]) + impK * dotVT(n, Gb[b]));
      } else {
        // nonLinGeomTotalLagSolid.C:307-323: deformed normal
        V3 nc = dotVT(n, Finvb[b]);  // Finv^T & n
        nc = (1.0 / mag(nc)) * nc;
        gn = rImpK * ((t - p * nc) - dotVS(nc, sigb[b]) + impK * dotVT(n, Gb[b]));
      }
      g[b] = bc.relax == 1.0 ? gn : bc.relax * gn + (1.0 - bc.relax) * g[b];
    }
    for (int b = 0; b < m.nB; ++b)
      if (patchType(b) == ORC_FIXED_DISPLACEMENT) Ub[b] = fixedValue(b);
  }

  // correctBoundaryConditions: solidTraction::evaluate (:398-463) with
  // non-orthogonal correction; fixedDisplacement keeps its value.
  void evaluateBoundary() {
    for (int b = 0; b < m.nB; ++b) {
      int P = m.own[m.nI + b];
      if (patchType(b) == ORC_SOLID_TRACTION)
        Ub[b] = U[P] + dotVT(m.kb[b], G[P]) + (1.0 / m.bDelta[b]) * g[b];
      else
        Ub[b] = fixedValue(b);
    }
  }

  // Patch snGrad of the solved field (uses the current gradient field G).
  V3 snGrad(int b) const {
    if (patchType(b) == ORC_SOLID_TRACTION) return g[b];
    int P = m.own[m.nI + b];
    return m.bDelta[b] * (Ub[b] - (U[P] + dotVT(m.kb[b], G[P])));
  }

  // mechanicalModel::grad -> fvc::grad leastSquares + boundary correction.
  void gradient() {
    std::vector<T9> Gn(m.nC);
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (int c = 0; c < m.nC; ++c) {
      T9 acc = zeroT();
      for (int e = m.cfStart[c]; e < m.cfStart[c + 1]; ++e) {
        int f = m.cfFace[e];
        V3 dv = U[m.nei[f]] - U[m.own[f]];
        if (m.own[f] == c) acc += outer(m.lsP[f], dv);
        else acc = acc - outer(m.lsN[f], dv);
      }
      for (int e = m.cbStart[c]; e < m.cbStart[c + 1]; ++e) {
        int b = m.cbFace[e];
        acc += outer(m.lsB[b], Ub[b] - U[c]);
      }
      Gn[c] = acc;
    }
    // boundary: Gb = G_P + n (snGrad - n.G_P); snGrad of fixedDisplacement
    // uses the gradient field as it was before this call.
    std::vector<T9> Gbn(m.nB);
    for (int b = 0; b < m.nB; ++b) {
      int P = m.own[m.nI + b];
      V3 n = m.nf[m.nI + b];
      V3 sg = snGrad(b);
      Gbn[b] = Gn[P] + outer(n, sg - dotVT(n, Gn[P]));
    }
    G.swap(Gn);
    Gb.swap(Gbn);
  }

  S6 hooke(const T9& gr) const {
    S6 eps = symmT(gr);
    return addI((2.0 * mu) * devS(eps), K * trS(eps));
  }

  S6 neoHookean(const T9& F) const {
    double Jl = detT(F);
    T9 b = dotTT(F, transposeT(F));
    S6 bEbar = std::pow(Jl, -2.0 / 3.0) * symmT(b);
    S6 sdev = mu * devS(bEbar);
    double sigmaHyd = 0.5 * K * (std::pow(Jl, 2.0) - 1.0);
    return (1.0 / Jl) * addI(sdev, sigmaHyd);
  }

  void correctStress() {
    if (!tl) {
#pragma omp parallel for num_threads(nt) if (nt > 1)
      for (int c = 0; c < m.nC; ++c) sig[c] = hooke(G[c]);
      for (int b = 0; b < m.nB; ++b) sigb[b] = hooke(Gb[b]);
      return;
    }
    // updateF (mechanicalLaw.C:1041-1160): TL incremental F = F.oldTime +
    // gradDD^T; TL total F = I + gradD^T
#pragma omp parallel for num_threads(nt) if (nt > 1)
    for (int c = 0; c < m.nC; ++c) FL[c] = (incr ? FL0[c] : identT()) + transposeT(G[c]);
    for (int b = 0; b < m.nB; ++b) FLb[b] = (incr ? FL0b[b] : identT()) + transposeT(Gb[b]);
    if (enforceLinear) {
      auto lin = [&](const S6& s0, const T9& gdd) {
        return addI(s0 + (2.0 * mu) * devS(symmT(gdd)), K * trT(gdd));
      };
      for (int c = 0; c < m.nC; ++c) sig[c] = lin(sig0[c], G[c]);
      for (int b = 0; b < m.nB; ++b) sigb[b] = lin(sig0b[b], Gb[b]);
      return;
    }
#pragma omp parallel for num_threads(nt) if (nt > 1)
    for (int c = 0; c < m.nC; ++c) sig[c] = neoHookean(FL[c]);
    for (int b = 0; b < m.nB; ++b) sigb[b] = neoHookean(FLb[b]);
  }

  // Explicit source of the momentum equation, volume-integrated, in the
  // operator form  A U = b  (A from assembleMatrix).
  void buildSource(std::vector<V3>& b) {
    const double gam = impK;                   // impKf (uniform material)
    const double gamS = s.stab_scale * impK;   // RhieChow gamma, 0 on boundary
    b.assign(m.nC, V3{0, 0, 0});
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (int c = 0; c < m.nC; ++c) {
      V3 fvmCorr = {0, 0, 0}, fvcLap = {0, 0, 0}, divS = {0, 0, 0}, stab = {0, 0, 0};
      for (int e = m.cfStart[c]; e < m.cfStart[c + 1]; ++e) {
        int f = m.cfFace[e];
        int P = m.own[f], N = m.nei[f];
        double sgn = (P == c) ? 1.0 : -1.0;
        double wf = m.w[f];
        T9 gf = wf * G[P] + (1.0 - wf) * G[N];        // linear interpolate(grad)
        V3 kCorr = dotVT(m.corrVec[f], gf);            // k & grad_f
        V3 dU = U[N] - U[P];
        // gaussLaplacianScheme corrected: gamma|S| (delta (U_N - U_P) + k.grad_f)
        V3 corrFlux = (gam * m.magSf[f]) * kCorr;
        V3 lapFlux = (gam * m.magSf[f]) * (m.nonOrthDelta[f] * dU + kCorr);
        V3 stabLap = (gamS * m.magSf[f]) * (m.nonOrthDelta[f] * dU + kCorr);
        V3 stabDiv = gamS * dotVT(m.Sf[f], gf);
        V3 sigFlux;
        if (!tl) {
          S6 sf = wf * sig[P] + (1.0 - wf) * sig[N];
          sigFlux = dotVS(m.Sf[f], sf);
        } else if (enforceLinear) {
          S6 sf = wf * sig[P] + (1.0 - wf) * sig[N];
          sigFlux = dotVS(m.Sf[f], sf);
        } else {
          T9 tP = J[P] * dotTT(Finv[P], fromS(sig[P]));
          T9 tN = J[N] * dotTT(Finv[N], fromS(sig[N]));
          T9 tf = wf * tP + (1.0 - wf) * tN;
          sigFlux = dotVT(m.Sf[f], tf);
        }
        fvmCorr += sgn * corrFlux;
        fvcLap += sgn * lapFlux;
        divS += sgn * sigFlux;
        stab += sgn * (stabLap - stabDiv);
      }
      V3 bcCoeffs = {0, 0, 0};
      for (int e = m.cbStart[c]; e < m.cbStart[c + 1]; ++e) {
        int bb = m.cbFace[e];
        int f = m.nI + bb;
        double gms = gam * m.magSf[f];
        if (patchType(bb) == ORC_FIXED_DISPLACEMENT) {
          // boundaryCoeffs = gamma|S| gradientBoundaryCoeffs
          bcCoeffs += (gms * m.bDelta[bb]) * (Ub[bb] - dotVT(m.kb[bb], G[c]));
        } else {
          bcCoeffs += gms * g[bb];
        }
        fvcLap += gms * snGrad(bb);
        if (!tl || enforceLinear) {
          divS += dotVS(m.Sf[f], sigb[bb]);
        } else {
          T9 tb = Jb[bb] * dotTT(Finvb[bb], fromS(sigb[bb]));
          divS += dotVT(m.Sf[f], tb);
        }
      }
      b[c] = fvmCorr + bcCoeffs - fvcLap + divS + stab;
    }
  }

  // relaxField "Aitken" (solidModel.C:842-896) on the solved field:
  // r = D.prevIter - D; at iCorr 0 alpha = the field's relaxation factor
  // (1 without one), else alpha = alpha (r_prev . dr) / (|dr|^2 + SMALL),
  // dr = r_prev - r, bounded to [0, 2]; then D -= alpha r.  GeometricField
  // arithmetic gives every boundary face the same update from its own
  // values; the -= leaves fixed-value (fixedDisplacement) faces as they are.
  void aitken(int iCorr, const std::vector<V3>& prev, const std::vector<V3>& prevB) {
    if (aitA.empty()) {
      aitA.assign(m.nC, 1.0); aitAb.assign(m.nB, 1.0);
      aitR.assign(m.nC, V3{0, 0, 0}); aitRb.assign(m.nB, V3{0, 0, 0});
    }
    const double a0 = (s.field_relaxation > 0 && s.field_relaxation != 1.0) ? s.field_relaxation : 1.0;
    auto step = [&](double& a, V3& rPrev, V3& u, const V3& p, bool apply) {
      const V3 r = p - u;
      if (iCorr == 0) {
        a = a0;
      } else {
        const V3 dr = rPrev - r;
        const double num = rPrev.x * dr.x + rPrev.y * dr.y + rPrev.z * dr.z;
        const double den = dr.x * dr.x + dr.y * dr.y + dr.z * dr.z + SMALL;
        a = a * num / den;
        a = std::max(0.0, std::min(2.0, a));
      }
      rPrev = r;
      if (apply) u = u - a * r;
    };
    for (int c = 0; c < m.nC; ++c) step(aitA[c], aitR[c], U[c], prev[c], true);
    for (int b = 0; b < m.nB; ++b)
      step(aitAb[b], aitRb[b], Ub[b], prevB[b], patchType(b) != ORC_FIXED_DISPLACEMENT);
  }

  // One call of the model's evolve() for the current load factor.
  bool evolve(int& correctorsLeft) {
    int iCorr = 0;
    double initResMag = 0, relRes = 0;
    int maxIters = 0;
    bool conv = false;
    std::vector<V3> src, prev;
    std::vector<double> bc(m.nC), xc(m.nC);
    if (tl) enforceLinear = false;
    do {
      prev = U;                          // storePrevIter
      const std::vector<V3> prevB = Ub;  // (the boundary values too)
      updateTraction();                  // fvMatrix construction: updateCoeffs
      buildSource(src);
      double r2 = 0;
      maxIters = 0;
      for (int cmpt = 0; cmpt < 3; ++cmpt) {
        // the empty direction's component is not solved (fvMatrix solves
        // only the mesh's solution directions)
        if (cmpt + 1 == s.empty_direction) continue;
        for (int c = 0; c < m.nC; ++c) {
          bc[c] = cmpt == 0 ? src[c].x : cmpt == 1 ? src[c].y : src[c].z;
          xc[c] = cmpt == 0 ? U[c].x : cmpt == 1 ? U[c].y : U[c].z;
        }
        SolverPerf sp = pcg(m, A, s.preconditioner == ORC_DIC ? &dic : nullptr,
                            bc, xc, s.tolerance, s.rel_tol, s.max_iter, nt);
        for (int c = 0; c < m.nC; ++c) {
          if (cmpt == 0) U[c].x = xc[c]; else if (cmpt == 1) U[c].y = xc[c]; else U[c].z = xc[c];
        }
        r2 += sp.initRes * sp.initRes;
        maxIters = std::max(maxIters, sp.nIter);
        perf.total_lin_iters += sp.nIter;
      }
      initResMag = std::sqrt(r2);
      evaluateBoundary();                // psi.correctBoundaryConditions()
      // relaxField, "fixed" (solidModel.C:837-841): D.relax() with the field's
      // relaxation factor, D == D.prevIter + f (D - D.prevIter) on the cells
      // and, by the forced assignment, on every boundary face
      const double fr = s.field_relaxation;
      if (s.relaxation_method == 1) {
        aitken(iCorr, prev, prevB);
      } else if (fr > 0 && fr != 1.0) {
        for (int c = 0; c < m.nC; ++c) U[c] = prev[c] + fr * (U[c] - prev[c]);
        for (int b = 0; b < m.nB; ++b) Ub[b] = prevB[b] + fr * (Ub[b] - prevB[b]);
      }
      if (!tl) {
        gradient();
        correctStress();
      } else {
        // incremental: D = D.oldTime + DD, gradD = gradD.oldTime + gradDD;
        // total (nonLinGeomTotalLagTotalDispSolid.C:224-239): D and gradD
        // are the solved field and its gradient
        for (int c = 0; c < m.nC; ++c) D[c] = incr ? D0[c] + U[c] : U[c];
        for (int b = 0; b < m.nB; ++b) Db[b] = incr ? D0b[b] + Ub[b] : Ub[b];
        gradient();
        for (int c = 0; c < m.nC; ++c) {
          GD[c] = incr ? GD0[c] + G[c] : G[c];
          T9 F = identT() + transposeT(GD[c]);
          Finv[c] = invT(F); J[c] = detT(F);
        }
        for (int b = 0; b < m.nB; ++b) {
          GDb[b] = incr ? GD0b[b] + Gb[b] : Gb[b];
          T9 F = identT() + transposeT(GDb[b]);
          Finvb[b] = invT(F); Jb[b] = detT(F);
        }
        // only the incremental form checks J (nonLinGeomTotalLagSolid.C:203-207)
        if (incr && !enforceLinear) {
          double minJ = 1e300, maxJ = -1e300;
          for (int c = 0; c < m.nC; ++c) { minJ = std::min(minJ, J[c]); maxJ = std::max(maxJ, J[c]); }
          for (int b = 0; b < m.nB; ++b) { minJ = std::min(minJ, Jb[b]); maxJ = std::max(maxJ, Jb[b]); }
          if (minJ < 0.01 || maxJ > 100) { enforceLinear = true; perf.enforce_linear = 1; }
        }
        correctStress();
      }
      // converged(): solidModelTemplates.C:26-188
      double denom = 0, resMax = 0;
      for (int c = 0; c < m.nC; ++c) {
        double dn = incr ? mag(U[c]) : mag(U[c] - D0[c]);
        denom = std::max(denom, dn);
        resMax = std::max(resMax, mag(U[c] - prev[c]));
      }
      if (denom < SMALL) {
        double mx = 0;
        for (int c = 0; c < m.nC; ++c) mx = std::max(mx, mag(U[c]));
        denom = std::max(mx, SMALL);
      }
      relRes = resMax / denom;
      // The max-reductions above drop NaN (std::max(0, NaN) is 0), so a
      // non-finite field is caught here and ends the solve, unconverged.
      bool finite = true;
      for (int c = 0; c < m.nC && finite; ++c)
        finite = std::isfinite(U[c].x) && std::isfinite(U[c].y) && std::isfinite(U[c].z);
      if (!finite) {
        perf.nan_detected = 1;
        perf.n_correctors++;
        conv = false;
        correctorsLeft = 0;
        break;
      }
      const double materialResidual = 0.0;
      conv = false;
      if (iCorr > 1 && materialResidual < s.material_tol) {
        if (initResMag < s.solution_tol && relRes < s.solution_tol) conv = true;
        else if (relRes < s.alternative_tol) conv = true;
        else if (initResMag < s.alternative_tol) conv = true;
      }
      perf.n_correctors++;
      if (--correctorsLeft == 0) break;
      if (s.max_seconds > 0 &&
          std::chrono::duration<double>(std::chrono::steady_clock::now() - tStart).count() >
              s.max_seconds) {
        correctorsLeft = 0;
        break;
      }
    } while (!conv && ++iCorr < s.n_correctors);
    perf.initial_residual = initResMag;
    perf.rel_residual = relRes;
    perf.converged = conv ? 1 : 0;
    return conv;
  }

  std::chrono::steady_clock::time_point tStart;

  void run() {
    tStart = std::chrono::steady_clock::now();
    int left = s.max_correctors_run > 0 ? s.max_correctors_run : -1;
    if (!tl) {
      // Constructor: D.correctBoundaryConditions(); grad(D)
      // (linGeomTotalDispSolid.C:64-105)
      updateTraction();
      evaluateBoundary();
      gradient();
      evolve(left);
      D = U; Db = Ub;
      return;
    }
    // TL constructor: DD (or D).correctBoundaryConditions() at time 0
    loadFactor = 0.0;
    updateTraction();
    evaluateBoundary();
    const int nInc = std::max(1, s.n_increments);
    for (int n = 1; n <= nInc; ++n) {
      // new time step: old-time fields take the converged values; the total
      // form reads only D.oldTime (converged()), the solved D carries over
      D0 = D; D0b = Db;
      if (incr) {
        GD0 = GD; GD0b = GDb; FL0 = FL; FL0b = FLb;
        sig0 = sig; sig0b = sigb;
      }
      loadFactor = (double)n / nInc;
      evolve(left);
      for (int c = 0; c < m.nC; ++c) D[c] = incr ? D0[c] + U[c] : U[c];
      for (int b = 0; b < m.nB; ++b) Db[b] = incr ? D0b[b] + Ub[b] : Ub[b];
      if (left == 0) break;
    }
  }
};

bool validSettings(const orc_settings* s) {
  if (!s) return false;
  if (s->model != ORC_LIN_GEOM_TOTAL_DISP && s->model != ORC_NONLIN_GEOM_TOTAL_LAG &&
      s->model != ORC_NONLIN_GEOM_TOTAL_LAG_TOTAL_DISP) return false;
  if (s->model != ORC_LIN_GEOM_TOTAL_DISP && s->law != ORC_NEO_HOOKEAN) return false;
  if (s->model == ORC_LIN_GEOM_TOTAL_DISP && s->law != ORC_LINEAR_ELASTIC) return false;
  if (s->max_iter < 1 || s->n_correctors < 1) return false;
  return true;
}

}  // namespace

extern "C" {

void orc_default_settings(orc_settings* s) {
  std::memset(s, 0, sizeof(*s));
  s->model = ORC_LIN_GEOM_TOTAL_DISP;
  s->law = ORC_LINEAR_ELASTIC;
  s->E = 200e9; s->nu = 0.3;
  s->preconditioner = ORC_DIC;
  s->tolerance = 1e-9; s->rel_tol = 0.1; s->max_iter = 1000;
  s->n_correctors = 2000;
  s->solution_tol = 1e-6; s->alternative_tol = 1e-7; s->material_tol = 1e-5;
  s->stab_scale = 0.1;
  s->ls_boundary_delta = 0;
  s->n_increments = 1;
  s->n_threads = 1;
  s->max_correctors_run = 0;
  s->dic_domain = nullptr;
  s->max_seconds = 0;
}

int orc_solve(const orc_mesh_desc* md, const orc_bc* bcs, const orc_settings* s,
              const int* perm, double* D_out, double* sigma_out,
              double* gradD_out, orc_perf* perf) {
  if (!md || !bcs || !validSettings(s)) return 1;
  Mesh m;
  if (s->empty_direction < 0 || s->empty_direction > 3) return 1;
  if (!m.build(md, perm, s->ls_boundary_delta, s->empty_direction)) return 2;
  auto t0 = std::chrono::steady_clock::now();
  Solver sol(m, *s, bcs);
  sol.run();
  auto t1 = std::chrono::steady_clock::now();
  sol.perf.seconds = std::chrono::duration<double>(t1 - t0).count();
  // caller cell perm[i] is solver cell i
  std::vector<int> newOf(md->n_cells);
  for (int i = 0; i < md->n_cells; ++i) newOf[perm ? perm[i] : i] = i;
  const std::vector<T9>& gradOut = s->model != ORC_LIN_GEOM_TOTAL_DISP ? sol.GD : sol.G;
  for (int c = 0; c < md->n_cells; ++c) {
    int i = newOf[c];
    if (D_out) { D_out[3 * c] = sol.D[i].x; D_out[3 * c + 1] = sol.D[i].y; D_out[3 * c + 2] = sol.D[i].z; }
    if (sigma_out) {
      const S6& q = sol.sig[i];
      double* o = sigma_out + 6 * (size_t)c;
      o[0] = q.xx; o[1] = q.xy; o[2] = q.xz; o[3] = q.yy; o[4] = q.yz; o[5] = q.zz;
    }
    if (gradD_out) std::memcpy(gradD_out + 9 * (size_t)c, &gradOut[i], sizeof(T9));
  }
  if (perf) *perf = sol.perf;
  return 0;
}

int orc_assemble_matrix(const orc_mesh_desc* md, const orc_bc* bcs, double impK,
                        double* diag, double* upper) {
  Mesh m;
  if (!m.build(md, nullptr, 0)) return 2;
  orc_settings s;
  orc_default_settings(&s);
  Solver sol(m, s, bcs);
  // rescale to the requested impK (the solver used 2mu+lambda of E, nu)
  double r = impK / sol.impK;
  for (int c = 0; c < m.nC; ++c) diag[c] = sol.A.diag[c] * r;
  for (int f = 0; f < m.nI; ++f) upper[f] = sol.A.upper[f] * r;
  return 0;
}

int orc_amul(const orc_mesh_desc* md, const double* diag, const double* upper,
             const double* x, double* y) {
  Mesh m;
  if (!m.build(md, nullptr, 0)) return 2;
  Ldu A;
  A.diag.assign(diag, diag + m.nC);
  A.upper.assign(upper, upper + m.nI);
  amul(m, A, x, y, 1);
  return 0;
}

int orc_dic_precondition(const orc_mesh_desc* md, const double* diag,
                         const double* upper, const double* r, double* w) {
  Mesh m;
  if (!m.build(md, nullptr, 0)) return 2;
  Ldu A;
  A.diag.assign(diag, diag + m.nC);
  A.upper.assign(upper, upper + m.nI);
  Dic dic;
  dic.build(m, A, 1);
  dic.apply(m, A, r, w);
  return 0;
}

int orc_ls_grad(const orc_mesh_desc* md, int lsBoundaryDelta, const double* D,
                const double* Db, const double* snGradB, double* Gout,
                double* Gbout) {
  Mesh m;
  if (!m.build(md, nullptr, lsBoundaryDelta)) return 2;
  for (int c = 0; c < m.nC; ++c) {
    T9 acc = zeroT();
    V3 Dc = getV(D, c);
    for (int e = m.cfStart[c]; e < m.cfStart[c + 1]; ++e) {
      int f = m.cfFace[e];
      V3 dv = getV(D, m.nei[f]) - getV(D, m.own[f]);
      if (m.own[f] == c) acc += outer(m.lsP[f], dv);
      else acc = acc - outer(m.lsN[f], dv);
    }
    for (int e = m.cbStart[c]; e < m.cbStart[c + 1]; ++e) {
      int b = m.cbFace[e];
      acc += outer(m.lsB[b], getV(Db, b) - Dc);
    }
    std::memcpy(Gout + 9 * (size_t)c, &acc, sizeof(T9));
  }
  for (int b = 0; b < m.nB; ++b) {
    int P = m.own[m.nI + b];
    T9 gp;
    std::memcpy(&gp, Gout + 9 * (size_t)P, sizeof(T9));
    V3 n = m.nf[m.nI + b];
    T9 gb = gp + outer(n, getV(snGradB, b) - dotVT(n, gp));
    std::memcpy(Gbout + 9 * (size_t)b, &gb, sizeof(T9));
  }
  return 0;
}

}  // extern "C"
