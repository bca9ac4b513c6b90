// Finite-volume kernels of the segregated solid solve: once-per-mesh geometry
// and matrix, the post-solve pass (gradient, law, boundary conditions,
// convergence reductions) and the right-hand-side pass (divergence of stress,
// Rhie-Chow stabilisation, boundary terms).
//
// Reference arithmetic (paths relative to the solids4foam tree):
//   outer loop     solidModels/linGeomTotalDispSolid/linGeomTotalDispSolid.C:135-208
//   TL loop        solidModels/nonLinGeomTotalLagSolid/nonLinGeomTotalLagSolid.C:145-240
//   traction BC    solidModels/fvPatchFields/solidTraction/solidTractionFvPatchVectorField.C:321-463
//                  + tractionBoundarySnGrad linGeomTotalDispSolid.C:235-271,
//                    nonLinGeomTotalLagSolid.C:263-325
//   fixed disp BC  .../fixedDisplacement/fixedDisplacementFvPatchVectorField.C:258-356
//   correction k   numerics/patchCorrectionVectors/patchCorrectionVectors.C:24-36
//   Rhie-Chow      solidModels/solidModel/momentumStabilisation/momentumStabilisation.C:79-217
//   laws           linearElastic.C:318-339 (+ mechanicalLaw.C:983-1001),
//                  neoHookeanElastic.C:275-303 (+ mechanicalLaw.C:1095-1159)
//   converged()    solidModels/solidModel/solidModelTemplates.C:26-188
// OpenFOAM operators (leastSquares gradient, Gauss linear corrected laplacian,
// Gauss linear divergence, linear interpolation) follow the published
// finite-volume formulation.
//
// The momentum system of one corrector is  M D_new = M D_old + R(D_old):
// the implicit (fvm) and explicit (fvc) laplacians of the reference cancel
// except for M (D_new - D_old), so the PCG solves M x = R for the correction
// x = D_new - D_old.  Each face flux is evaluated in the owner orientation by
// both cells that share it, so owner and neighbour contributions are exact
// negatives of each other; there are no atomics and sums run in a fixed order.

#include "kernels.cuh"

namespace s4g {
namespace {

__device__ __forceinline__ S6 hooke(const Controls& c, const T9& g) {
  S6 eps = symmT(g);
  return addI((2.0 * c.mu) * devS(eps), c.K * trS(eps));
}

__device__ __forceinline__ S6 neoHookean(const Controls& c, const T9& F) {
  double J = detT(F);
  T9 b = dotTT(F, transposeT(F));
  S6 bEbar = pow(J, -2.0 / 3.0) * symmT(b);
  S6 sdev = c.mu * devS(bEbar);
  double sigmaHyd = 0.5 * c.K * (pow(J, 2.0) - 1.0);
  return (1.0 / J) * addI(sdev, sigmaHyd);
}

// ------------------------------------------------------------- geometry ---

__global__ void kGeomCells(MeshView mv, GeomInputs in, GeomOutputs out) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= mv.nC) return;
  int c = in.s2c[s];
  stV(out.C, s, ldV(in.Cc, c));
}

__global__ void kGeomFaces(MeshView mv, GeomInputs in, GeomOutputs out) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= mv.nI) return;
  int f = in.fcaller[k];
  V3 S = ldV(in.Sfc, f);
  if (in.fflip[k]) S = -1.0 * S;
  V3 Cf = ldV(in.Cfc, f);
  V3 Co = ldV(out.C, mv.fown[k]), Cn = ldV(out.C, mv.fnei[k]);
  double magS = mag(S);
  V3 n = (1.0 / magS) * S;
  // surfaceInterpolation::makeWeights
  double sfdOwn = fabs(dot(S, Cf - Co));
  double sfdNei = fabs(dot(S, Cn - Cf));
  double w = sfdNei / (sfdOwn + sfdNei);
  V3 d = Cn - Co;
  // stabilised non-orthogonal deltaCoeffs 1/max(n.d, 0.05|d|)
  double delta = 1.0 / fmax(dot(n, d), 0.05 * mag(d));
  stV(out.fS, k, S);
  out.fmagS[k] = magS;
  out.fw[k] = w;
  out.fdelta[k] = delta;
}

// Boundary geometry that does not need the least-squares tensor.
__global__ void kGeomBFaces1(MeshView mv, GeomInputs in, GeomOutputs out, double* bd) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= mv.nB) return;
  int f = mv.nI + in.bcaller[k];
  V3 S = ldV(in.Sfc, f);
  V3 Cf = ldV(in.Cfc, f);
  V3 Cp = ldV(out.C, in.bcell[k]);
  double magS = mag(S);
  V3 n = (1.0 / magS) * S;
  V3 dfull = Cf - Cp;
  V3 dn = dot(n, dfull) * n;             // fvPatch::delta(): patch-normal
  stV(out.bS, k, S);
  out.bmagS[k] = magS;
  stV(out.bn, k, n);
  out.bdelta[k] = 1.0 / mag(dn);
  stV(out.bk, k, dfull - dot(n, dfull) * n);  // (I - n n) & (Cf - C)
  stV(bd, k, in.lsBoundaryDelta ? dfull : dn);
}

// leastSquaresVectors: dd = sum d d^T/|d|^2 over the cell's faces, inverted.
__global__ void kGeomLs(MeshView mv, GeomOutputs out, const double* bd) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= mv.nC) return;
  V3 Cs = ldV(out.C, s);
  S6 acc = {0, 0, 0, 0, 0, 0};
  for (int e = mv.rowptr[s]; e < mv.rowptr[s + 1]; ++e) {
    V3 d = ldV(out.C, mv.col[e]) - Cs;
    double r = 1.0 / magSqr(d);
    S6 wdd = {r * d.x * d.x, r * d.x * d.y, r * d.x * d.z, r * d.y * d.y, r * d.y * d.z, r * d.z * d.z};
    acc = acc + wdd;
  }
  for (int b = mv.browptr[s]; b < mv.browptr[s + 1]; ++b) {
    V3 d = ldV(bd, b);
    double r = 1.0 / magSqr(d);
    S6 wdd = {r * d.x * d.x, r * d.x * d.y, r * d.x * d.z, r * d.y * d.y, r * d.y * d.z, r * d.z * d.z};
    acc = acc + wdd;
  }
  S6 inv;
  if (mv.emptyDir) {
    // 2-D: dd has no component along the empty direction; as OpenFOAM's
    // inv(symmTensorField) does, add 1 there, invert, take the 1 away
    const double e[3] = {mv.emptyDir == 1 ? 1.0 : 0.0, mv.emptyDir == 2 ? 1.0 : 0.0,
                         mv.emptyDir == 3 ? 1.0 : 0.0};
    const S6 a = {acc.xx + e[0], acc.xy, acc.xz, acc.yy + e[1], acc.yz, acc.zz + e[2]};
    inv = invS(a);
    inv.xx -= e[0]; inv.yy -= e[1]; inv.zz -= e[2];
  } else {
    inv = invS(acc);
  }
  stS(out.invDd, s, inv);
  // per CSR entry, oriented so that grad += lsv (x) (U_nb - U_P) on both sides
  for (int e = mv.rowptr[s]; e < mv.rowptr[s + 1]; ++e) {
    const V3 Cn = ldV(out.C, mv.col[e]);
    V3 v;
    if (mv.fidx[e] >= 0) {
      const V3 d = Cn - Cs;
      const double r = 1.0 / magSqr(d);
      v = r * dotVS(d, inv);
    } else {
      const V3 d = Cs - Cn;
      const double r = 1.0 / magSqr(d);
      v = -r * dotVS(d, inv);
    }
    stV(out.lsv, e, v);
  }
  for (int b = mv.browptr[s]; b < mv.browptr[s + 1]; ++b) {
    V3 d = ldV(bd, b);
    stV(out.bls, b, (1.0 / magSqr(d)) * dotVS(d, inv));
  }
}

__global__ void kMatrix(MeshView mv, double gamma, double* val, double* diag) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= mv.nC) return;
  double d = 0;
  for (int e = mv.rowptr[s]; e < mv.rowptr[s + 1]; ++e) {
    int fk = mv.fidx[e];
    int f = fk >= 0 ? fk : ~fk;
    double upper = mv.fdelta[f] * (gamma * mv.fmagS[f]);
    d -= upper;
    val[e] = -upper;
  }
  for (int b = mv.browptr[s]; b < mv.browptr[s + 1]; ++b)
    if (mv.btype[b] == 0) d += gamma * mv.bmagS[b] * (-mv.bdelta[b]);
  diag[s] = -d;
}

// ---------------------------------------------------------- traction BC ---

__device__ __forceinline__ V3 tractionSnGrad(const MeshView& mv, const Controls& c, int b,
                                             const S6& sb, const T9& Gb, const T9* Finvb,
                                             int enforceLinear) {
  V3 t = c.loadFactor * ldV(mv.bval, b);
  double p = c.loadFactor * mv.bpress[b];
  V3 n = ldV(mv.bn, b);
  if (!c.tl) {
    T9 a = fromS(sb) - c.impK * Gb;
    return c.rImpK * ((t - p * n) - dotVT(n, a));
  }
  if (enforceLinear || !Finvb)
    return c.rImpK * ((t - p * n) - dotVS(n, sb) + c.impK * dotVT(n, Gb));
  V3 nc = dotVT(n, *Finvb);
  nc = (1.0 / mag(nc)) * nc;
  return c.rImpK * ((t - p * nc) - dotVS(nc, sb) + c.impK * dotVT(n, Gb));
}

// Relaxed update of the traction gradient (solidTraction...C:387-392):
// g = f g_new + (1 - f) g_old; f = 1 leaves g_new as it is.
__device__ __forceinline__ V3 relaxG(const MeshView& mv, int b, V3 gNew, V3 gOld) {
  const double rf = mv.brelax[b];
  return rf == 1.0 ? gNew : rf * gNew + (1.0 - rf) * gOld;
}

// The first update of an increment or time step.  The g it relaxes against
// is the one the previous corrector used (gPrev, zero at the start): that
// corrector has already written the update it would have used next.
__global__ void kTractionInit(MeshView mv, Controls c, FieldPtrs f) {
  f = caseFields(f, blockIdx.y, mv.nC, mv.nB, mv.nI);
  caseView(mv, blockIdx.y);
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= mv.nB || mv.btype[b] != 1) return;
  T9 Fi;
  const T9* pF = nullptr;
  if (c.tl) { Fi = ldT(f.Finvb, b); pF = &Fi; }
  const V3 gOld = ldV(f.gPrev, b);
  stV(f.g, b, relaxG(mv, b, tractionSnGrad(mv, c, b, ldS(f.sigb, b), ldT(f.Gb, b), pF, 0), gOld));
}

// Boundary value of the solved field on face b of cell s (correctBoundaryConditions).
__device__ __forceinline__ V3 boundaryValue(const MeshView& mv, const Controls& c,
                                            const FieldPtrs& f, int b, V3 Up, const T9& Gold) {
  if (mv.btype[b] == 1)
    return Up + dotVT(ldV(mv.bk, b), Gold) + (1.0 / mv.bdelta[b]) * ldV(f.g, b);
  V3 v = c.loadFactor * ldV(mv.bval, b);
  if (c.tl == 1) v = v - ldV(f.D0b, b);  // DD = D - D.oldTime
  return v;
}

// --------------------------------------------------------- post-solve pass ---
// relaxField "Aitken" (solidModel.C:842-896) of one cell or boundary face:
// r = D.prevIter - D (p the value before the solve, u the solved one); at
// an increment's first corrector alpha = aitkenA0 (the field's relaxation
// factor, else 1), later alpha = alpha (r_prev . dr) / (|dr|^2 + SMALL) with
// dr = r_prev - r, bounded to [0, 2]; then D -= alpha r (apply false: a
// fixed-value face, which the -= leaves as it is).  Explicitly rounded
// operations, in the oracle's order.
__device__ __forceinline__ V3 aitkenRelax(const Controls& c, bool first, double* a,
                                          double* rPrev, V3 p, V3 u, bool apply) {
  const V3 r{__dsub_rn(p.x, u.x), __dsub_rn(p.y, u.y), __dsub_rn(p.z, u.z)};
  double al;
  if (first) {
    al = c.aitkenA0;
  } else {
    const V3 rp = ldV(rPrev, 0);
    const V3 dr{__dsub_rn(rp.x, r.x), __dsub_rn(rp.y, r.y), __dsub_rn(rp.z, r.z)};
    const double num = __dadd_rn(__dadd_rn(__dmul_rn(rp.x, dr.x), __dmul_rn(rp.y, dr.y)),
                                 __dmul_rn(rp.z, dr.z));
    const double den = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(dr.x, dr.x), __dmul_rn(dr.y, dr.y)),
                                           __dmul_rn(dr.z, dr.z)),
                                 1e-15);
    al = __ddiv_rn(__dmul_rn(*a, num), den);
    al = fmax(0.0, fmin(2.0, al));
  }
  *a = al;
  stV(rPrev, 0, r);
  if (!apply) return u;
  return V3{__dsub_rn(u.x, __dmul_rn(al, r.x)), __dsub_rn(u.y, __dmul_rn(al, r.y)),
            __dsub_rn(u.z, __dmul_rn(al, r.z))};
}

// D_new = D + x (the correction of the corrector; x in the PCG type).  With
// a field relaxation factor f (relaxField "fixed", solidModel.C:837-841):
// D_new = D.prevIter + f (D_solved - D.prevIter) = D + f x; with Aitken the
// cell's own factor (aitkenRelax).  The processor-local PCG leaves the last
// iteration's x += alpha p to the pass after the loop (DevState::xPend):
// it is applied here first, the same operation as in the SpMV pass.
template <typename T>
__global__ void __launch_bounds__(kRowBlock)
kApplyX(MeshView mv, Controls c, FieldPtrs f, T* __restrict__ x, const T* pA, const T* pB,
        const DevState* st) {
  const int cs = blockIdx.y;
  f = caseFields(f, cs, mv.nC, mv.nB, mv.nI);
  x += (size_t)cs * 3 * mv.nC;
  st += cs;
  if (!st->caseLive) return;
  if (st->xPend[0] | st->xPend[1] | st->xPend[2]) {
    const T* __restrict__ pg = (st->pbuf ? pB : pA) + (size_t)cs * 3 * mv.nC;
    bool xp[3];
    T al[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) { xp[k] = st->xPend[k] != 0; al[k] = (T)st->alpha[k]; }
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < mv.nC; s += gridDim.x * blockDim.x)
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (xp[k]) x[3 * (size_t)s + k] = x[3 * (size_t)s + k] + al[k] * pg[3 * (size_t)s + k];
  }
  const int dc = st->dcur;
  const double* Uold = f.D[dc];
  double* Unew = f.D[dc ^ 1];
  const double fr = c.fieldRelax;
  if (c.aitken) {
    const bool first = st->iCorr == 0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < mv.nC; s += gridDim.x * blockDim.x) {
      const V3 uo = ldV(Uold, s);
      const V3 us = uo + ldVT(x, s);
      stV(Unew, s, aitkenRelax(c, first, f.aitA + s, f.aitR + 3 * (size_t)s, uo, us, true));
    }
  } else if (fr == 1.0)
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < mv.nC; s += gridDim.x * blockDim.x)
      stV(Unew, s, ldV(Uold, s) + ldVT(x, s));
  else
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < mv.nC; s += gridDim.x * blockDim.x)
      stV(Unew, s, ldV(Uold, s) + fr * ldVT(x, s));
}

// mode 0 (constructor): gradient only, from the current field.
// mode 1 (corrector): apply the correction x, gradient, law, boundary, g.
// With field relaxation the boundary values are relaxed too (the forced
// assignment of GeometricField::relax): Ub = Ub.prevIter + f (Ub_new -
// Ub.prevIter), Ub.prevIter kept in f.Ubr (mode 0 stores the constructor's).
// For the TL model the law needs the global J check first, so mode 1 stops
// after the kinematics (F, F^-1, J) and kPostLawTL finishes the pass.

template <typename T>
__global__ void __launch_bounds__(kRowBlock)
kPost(MeshView mv, Controls c, FieldPtrs f, const T* __restrict__ x, DevState* st,
      double* partials, int mode) {
  __shared__ double smem[32 * 6];
  {
    const int cs = blockIdx.y;
    f = caseFields(f, cs, mv.nC, mv.nB, mv.nI);
    caseView(mv, cs);
    x += (size_t)cs * 3 * mv.nC;
    st += cs;
    partials += (size_t)cs * mv.caseRec;
  }
  if (mode == 1 && !st->caseLive) return;
  const int dc = st->dcur;
  const bool apply = (mode == 1);
  // the corrected field D + x, written by kApplyX (mode 1), or D (mode 0)
  const double* U = f.D[apply ? dc ^ 1 : dc];
  const bool relax = c.fieldRelax != 1.0 || c.aitken;
  double red[6] = {0, 0, 0, 0, 0, 0};  // sum U
  double mx[3] = {0, 0, 0};            // max|x|, max|U-D0|, max|U|
  double minJ = 1e300, maxJ = -1e300;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < mv.nC; s += gridDim.x * blockDim.x) {
    const V3 Up = ldV(U, s);
    const bool hasB = mv.browptr[s + 1] > mv.browptr[s];
    T9 Gold = hasB ? ldT(f.G, s) : zeroT();
    // leastSquares gradient with the precomputed vectors of the cell's faces
    T9 acc = zeroT();
    for (int e = mv.rowptr[s]; e < mv.rowptr[s + 1]; ++e)
      acc = acc + outer(ldV(mv.lsv, e), ldV(U, mv.col[e]) - Up);
    // relaxed: the boundary values come from the field as solved, then
    // relax against their previous values (the cells were relaxed already)
    const V3 UpSolved = (relax && apply) ? ldV(f.D[dc], s) + ldVT(x, s) : Up;
    for (int b = mv.browptr[s]; b < mv.browptr[s + 1]; ++b) {
      V3 Ub = boundaryValue(mv, c, f, b, UpSolved, Gold);
      if (relax) {
        if (apply) {
          const V3 pb = ldV(f.Ubr, b);
          if (c.aitken)
            Ub = aitkenRelax(c, st->iCorr == 0, f.aitA + mv.nC + b, f.aitR + 3 * ((size_t)mv.nC + b),
                             pb, Ub, mv.btype[b] == 1);
          else
            Ub = pb + c.fieldRelax * (Ub - pb);
        }
        stV(f.Ubr, b, Ub);
      }
      acc = acc + outer(ldV(mv.bls, b), Ub - Up);
    }
    const T9 G = acc;
    stT(f.G, s, G);
    // boundary gradient: Gb = G + n (snGrad - n.G)
    for (int b = mv.browptr[s]; b < mv.browptr[s + 1]; ++b) {
      V3 n = ldV(mv.bn, b);
      V3 sg;
      if (mv.btype[b] == 1) {
        sg = ldV(f.g, b);
      } else {
        const V3 Ub = relax ? ldV(f.Ubr, b) : boundaryValue(mv, c, f, b, Up, Gold);
        sg = mv.bdelta[b] * (Ub - (Up + dotVT(ldV(mv.bk, b), Gold)));
      }
      T9 Gb = G + outer(n, sg - dotVT(n, G));
      stT(f.Gb, b, Gb);
      if (!c.tl) {
        S6 sb = mode == 1 ? hooke(c, Gb) : ldS(f.sigb, b);
        if (mode == 1) stS(f.sigb, b, sb);
        if (mv.btype[b] == 1) {
          stV(f.gPrev, b, sg);
          stV(f.g, b, relaxG(mv, b, tractionSnGrad(mv, c, b, sb, Gb, nullptr, 0), sg));
        }
      }
    }
    if (!c.tl) {
      if (mode == 1) stS(f.sig, s, hooke(c, G));
    } else if (mode == 1) {
      // TL kinematics: gradD = gradD.oldTime + gradDD; F = I + gradD^T
      T9 GD = ldT(f.GD0, s) + G;
      stT(f.GD, s, GD);
      T9 F = transposeT(GD);
      F.xx += 1.0; F.yy += 1.0; F.zz += 1.0;
      stT(f.Finv, s, invT(F));
      double J = detT(F);
      f.J[s] = J;
      minJ = fmin(minJ, J); maxJ = fmax(maxJ, J);
      for (int b = mv.browptr[s]; b < mv.browptr[s + 1]; ++b) {
        T9 GDb = ldT(f.GD0b, b) + ldT(f.Gb, b);
        stT(f.GDb, b, GDb);
        T9 Fb = transposeT(GDb);
        Fb.xx += 1.0; Fb.yy += 1.0; Fb.zz += 1.0;
        stT(f.Finvb, b, invT(Fb));
        double Jb = detT(Fb);
        f.Jb[b] = Jb;
        minJ = fmin(minJ, Jb); maxJ = fmax(maxJ, Jb);
      }
    }
    if (apply) {
      // maxima of squared magnitudes; the square root is taken once at the end
      // max|D - D.prevIter|: the correction, or its relaxed part
      const V3 xs = relax ? Up - ldV(f.D[dc], s) : ldVT(x, s);
      mx[0] = fmax(mx[0], magSqr(xs));
      mx[1] = fmax(mx[1], c.tl == 1 ? magSqr(Up) : magSqr(Up - ldV(f.D0, s)));
      mx[2] = fmax(mx[2], magSqr(Up));
      red[0] += Up.x; red[1] += Up.y; red[2] += Up.z;
      if (!(isfinite(Up.x) && isfinite(Up.y) && isfinite(Up.z))) atomicOr(&st->status, kErrNaN);
    }
  }
  if (mode == 0) return;
  double sums[3] = {red[0], red[1], red[2]};
  blockSum<3>(sums, smem);
  double mxs[5] = {mx[0], mx[1], mx[2], -minJ, maxJ};
  blockMax<5>(mxs, smem);
  if (threadIdx.x == 0) {
    double* p = partials + 8 * (size_t)blockIdx.x;
    p[0] = sums[0]; p[1] = sums[1]; p[2] = sums[2];
    p[3] = mxs[0]; p[4] = mxs[1]; p[5] = mxs[2]; p[6] = mxs[3]; p[7] = mxs[4];
  }
  if (!lastBlockDone(&st->counter[0], gridDim.x)) return;
  double S[3], M[5];
  reducePartials<3>(partials, 8, gridDim.x, S, smem);
  reducePartialsMax<5>(partials + 3, 8, gridDim.x, M, smem);
  if (threadIdx.x != 0) return;
  for (int k = 0; k < 3; ++k) M[k] = sqrt(M[k]);
  st->counter[0] = 0;
  st->dcur = dc ^ 1;
  // converged(): relative displacement residual
  double denom = M[1];
  if (denom < 1e-15) denom = fmax(M[2], 1e-15);
  double relRes = M[0] / denom;
  double r2 = 0;
  int maxIt = 0;
  for (int k = 0; k < 3; ++k) {
    r2 += st->initRes[k] * st->initRes[k];
    maxIt = max(maxIt, st->nIter[k]);
    st->totalLinIters += st->nIter[k];
  }
  double initResMag = sqrt(r2);
  st->relRes = relRes;
  st->initResMag = initResMag;
  st->lastMaxIters = maxIt;
  for (int k = 0; k < 3; ++k) st->xbar[k] = S[k] / mv.nC;
  if (c.tl) {
    st->minJ = -M[3]; st->maxJ = M[4];
    // only the incremental form checks J (nonLinGeomTotalLagSolid.C:203-207)
    if (c.tl == 1 && !st->enforceLinear && (st->minJ < 0.01 || st->maxJ > 100))
      st->enforceLinear = 1;
  }
  const int iCorr = st->iCorr;
  const double materialResidual = 0.0;
  bool conv = false;
  if (iCorr > 1 && materialResidual < c.matTol) {
    if (initResMag < c.solTol && relRes < c.solTol) conv = true;
    else if (relRes < c.altTol) conv = true;
    else if (initResMag < c.altTol) conv = true;
  }
  // fmax drops NaN, so a non-finite field can pass the test above: the
  // NaN flag (set by any block's isfinite check) overrides it
  st->converged = (conv && !(st->status & kErrNaN)) ? 1 : 0;
  st->nCorrDone += 1;
  st->iCorr = iCorr + 1;
  st->outerContinue = (!conv && iCorr + 1 < c.nCorr) ? 1 : 0;
  if (st->status & kErrNaN) st->outerContinue = 0;
  st->caseLive = st->outerContinue;
}

// TL second half: law (with the enforceLinear decision of this corrector),
// boundary stress and the next traction snGrad.
__global__ void __launch_bounds__(kRowBlock)
kPostLawTL(MeshView mv, Controls c, FieldPtrs f, const DevState* st) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= mv.nC) return;
  const int el = st->enforceLinear;
  T9 G = ldT(f.G, s);
  T9 FL = ldT(f.FL0, s) + transposeT(G);
  stT(f.FL, s, FL);
  S6 sg;
  if (el) {
    S6 s0 = ldS(f.sig0, s);
    sg = addI(s0 + (2.0 * c.mu) * devS(symmT(G)), c.K * trT(G));
  } else {
    sg = neoHookean(c, FL);
  }
  stS(f.sig, s, sg);
  for (int b = mv.browptr[s]; b < mv.browptr[s + 1]; ++b) {
    T9 Gb = ldT(f.Gb, b);
    T9 FLb = ldT(f.FL0b, b) + transposeT(Gb);
    stT(f.FLb, b, FLb);
    S6 sb;
    if (el) sb = addI(ldS(f.sig0b, b) + (2.0 * c.mu) * devS(symmT(Gb)), c.K * trT(Gb));
    else sb = neoHookean(c, FLb);
    stS(f.sigb, b, sb);
    if (mv.btype[b] == 1) {
      T9 Fi = ldT(f.Finvb, b);
      const V3 gOld = ldV(f.g, b);
      stV(f.gPrev, b, gOld);
      stV(f.g, b, relaxG(mv, b, tractionSnGrad(mv, c, b, sb, Gb, &Fi, el), gOld));
    }
  }
}

// --------------------------------------------------------------- RHS pass ---
// Face pass: for every internal face, in owner orientation (storage owner =
// lower row), the flux of R -- S.sigma_f + RhieChow -- and the
// gamma |S| delta (D_N - D_P) term of M D.  Each face is evaluated once; the
// cell pass adds it to the owner and subtracts it from the neighbour.
__global__ void __launch_bounds__(kRowBlock)
kRhsFace(MeshView mv, Controls c, FieldPtrs f, const DevState* st) {
  f = caseFields(f, blockIdx.y, mv.nC, mv.nB, mv.nI);
  st += blockIdx.y;
  if (!st->caseLive) return;
  const double* U = f.D[st->dcur];
  const int el = c.tl ? st->enforceLinear : 1;
  for (int fi = blockIdx.x * blockDim.x + threadIdx.x; fi < mv.nI; fi += gridDim.x * blockDim.x) {
    const int o = mv.fown[fi], n = mv.fnei[fi];
    const double w = mv.fw[fi];
    const V3 S = ldV(mv.fS, fi);
    const double cm = mv.fmagS[fi] * mv.fdelta[fi];
    const V3 dU = ldV(U, n) - ldV(U, o);
    const V3 d = ldV(mv.C, n) - ldV(mv.C, o);
    const T9 Gf = w * ldT(f.G, o) + (1.0 - w) * ldT(f.G, n);
    const S6 So = ldS(f.sig, o), Sn = ldS(f.sig, n);
    V3 sigFlux;
    if (el) {
      sigFlux = dotVS(S, w * So + (1.0 - w) * Sn);
    } else {
      const T9 To = f.J[o] * dotTT(ldT(f.Finv, o), fromS(So));
      const T9 Tn = f.J[n] * dotTT(ldT(f.Finv, n), fromS(Sn));
      sigFlux = dotVT(S, w * To + (1.0 - w) * Tn);
    }
    // Rhie-Chow: gammaS |S| delta (dU - d.grad_f)
    const V3 flux = sigFlux + (c.gammaS * cm) * (dU - dotVT(d, Gf));
    const V3 mflux = (c.gamma * cm) * dU;
    double* q = f.flux + 6 * (size_t)fi;
    q[0] = flux.x; q[1] = flux.y; q[2] = flux.z;
    q[3] = mflux.x; q[4] = mflux.y; q[5] = mflux.z;
  }
}

template <typename T>
__global__ void __launch_bounds__(kRowBlock)
kRhs(MeshView mv, Controls c, FieldPtrs f, T* __restrict__ x, T* __restrict__ r,
     DevState* st, double* partials) {
  __shared__ double smem[32 * 6];
  {
    const int cs = blockIdx.y;
    f = caseFields(f, cs, mv.nC, mv.nB, mv.nI);
    caseView(mv, cs);
    x += (size_t)cs * 3 * mv.nC;
    r += (size_t)cs * 3 * mv.nC;
    st += cs;
    partials += (size_t)cs * mv.caseRec;
  }
  if (!st->caseLive) return;
  const double* U = f.D[st->dcur];
  double part[6] = {0, 0, 0, 0, 0, 0};  // normFactor (3), sum|R| (3)
  const int el = c.tl ? st->enforceLinear : 1;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < mv.nC; s += gridDim.x * blockDim.x) {
    const V3 Us = ldV(U, s);
    V3 R = {0, 0, 0}, MD = {0, 0, 0};
    double sumA = 0;
    for (int e = mv.rowptr[s]; e < mv.rowptr[s + 1]; ++e) {
      const int fk = mv.fidx[e];
      const bool own = fk >= 0;
      const double* q = f.flux + 6 * (size_t)(own ? fk : ~fk);
      const V3 flux = {q[0], q[1], q[2]}, mflux = {q[3], q[4], q[5]};
      if (own) { R = R + flux; MD = MD - mflux; }
      else { R = R - flux; MD = MD + mflux; }
    }
    for (int b = mv.browptr[s]; b < mv.browptr[s + 1]; ++b) {
      const V3 S = ldV(mv.bS, b);
      const S6 sb = ldS(f.sigb, b);
      if (el) {
        R = R + dotVS(S, sb);
      } else {
        T9 tb = f.Jb[b] * dotTT(ldT(f.Finvb, b), fromS(sb));
        R = R + dotVT(S, tb);
      }
      if (mv.btype[b] == 0) {
        double a = c.gamma * mv.bmagS[b] * mv.bdelta[b];
        MD = MD + a * Us;
        sumA += a;
      }
    }
    // 2-D: the empty direction's component is not solved (its residual is
    // zero, so its PCG stops before the first iteration and D keeps 0 there)
    if (mv.emptyDir == 1) R.x = 0.0;
    else if (mv.emptyDir == 2) R.y = 0.0;
    else if (mv.emptyDir == 3) R.z = 0.0;
    stVT(r, s, R);
    stVT(x, s, V3{0, 0, 0});
    const double xb[3] = {st->xbar[0], st->xbar[1], st->xbar[2]};
    const double md[3] = {MD.x, MD.y, MD.z}, rr[3] = {R.x, R.y, R.z};
    for (int k = 0; k < 3; ++k) {
      double t = sumA * xb[k];
      part[k] += fabs(md[k] - t) + fabs(md[k] + rr[k] - t);
      part[3 + k] += fabs(rr[k]);
    }
  }
  blockSum<6>(part, smem);
  if (threadIdx.x == 0) {
    double* p = partials + 8 * (size_t)blockIdx.x;
    for (int k = 0; k < 6; ++k) p[k] = part[k];
  }
  if (!lastBlockDone(&st->counter[1], gridDim.x)) return;
  double S[6];
  reducePartials<6>(partials, 8, gridDim.x, S, smem);
  if (threadIdx.x != 0) return;
  st->counter[1] = 0;
  int any = 0;
  for (int k = 0; k < 3; ++k) {
    double nf = S[k] + 1e-20;
    st->normFactor[k] = nf;
    st->initRes[k] = S[3 + k] / nf;
    st->finalRes[k] = st->initRes[k];
    st->nIter[k] = 0;
    st->pending[k] = 0;
    st->xPend[k] = 0;
    st->active[k] = (st->initRes[k] < c.tol) ? 0 : 1;
    st->wArA[k] = 1e20;
    any |= st->active[k];
  }
  st->pcgContinue = (any && c.maxIter > 0) ? 1 : 0;
}

__global__ void kSetLoopCond(cudaGraphConditionalHandle h, DevState* st, int nRun, int which,
                             int first, unsigned limit) {
  unsigned* count = which == 0 ? &st[0].loopPcg : &st[0].loopOuter;
  if (first) *count = 0;
  else *count += 1;
  int any = 0;
  for (int cs = 0; cs < nRun; ++cs) {
    // a case whose wait gave up or whose field is not finite stops here
    if (st[cs].status & (kErrTimeout | kErrNaN)) {
      st[cs].pcgContinue = 0;
      if (which == 1) st[cs].caseLive = 0;
      continue;
    }
    any |= which == 0 ? st[cs].pcgContinue : st[cs].caseLive;
  }
  if (any && *count >= limit) {
    for (int cs = 0; cs < nRun; ++cs) {
      st[cs].status |= kErrTimeout;
      st[cs].pcgContinue = 0;
      if (which == 1) st[cs].caseLive = 0;
    }
    any = 0;
  }
  cudaGraphSetConditional(h, any ? 1u : 0u);
}

// pointD after the loop (enhancedVolPointInterpolate.C:351-423 via
// mechanicalModel.C:829-841): per point the inverse-distance-weighted
// average over its cells of D_c + (x_p - C_c) . gradD_c.  The operations are
// rounded one by one (no fused multiply-add) in the order of the host step
// s4g_point_interpolate, so both give the same bits.
__global__ void kPointInterp(int nP, const double* __restrict__ pts, const int* __restrict__ pcs,
                             const int* __restrict__ pcc, const int* __restrict__ c2s,
                             const double* __restrict__ C, const double* __restrict__ U,
                             const double* __restrict__ G, double* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nP) return;
  const double x0 = pts[3 * (size_t)p], x1 = pts[3 * (size_t)p + 1], x2 = pts[3 * (size_t)p + 2];
  double a0 = 0, a1 = 0, a2 = 0, sumW = 0;
  for (int k = pcs[p]; k < pcs[p + 1]; ++k) {
    const size_t s = (size_t)c2s[pcc[k]];
    const double d0 = __dsub_rn(x0, C[3 * s]), d1 = __dsub_rn(x1, C[3 * s + 1]),
                 d2 = __dsub_rn(x2, C[3 * s + 2]);
    const double m2 = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
    const double w = __ddiv_rn(1.0, __dsqrt_rn(m2));
    const double* g = G + 9 * s;
    const double* u = U + 3 * s;
    double e[3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
      e[j] = __dmul_rn(w, __dadd_rn(u[j], __dadd_rn(__dadd_rn(__dmul_rn(d0, g[j]), __dmul_rn(d1, g[3 + j])),
                                                    __dmul_rn(d2, g[6 + j]))));
    a0 = __dadd_rn(a0, e[0]); a1 = __dadd_rn(a1, e[1]); a2 = __dadd_rn(a2, e[2]);
    sumW = __dadd_rn(sumW, w);
  }
  // normalised where the weight sum exceeds OpenFOAM's ROOTVSMALL
  const bool nrm = sumW > 1e-150;
  out[3 * (size_t)p] = nrm ? __ddiv_rn(a0, sumW) : a0;
  out[3 * (size_t)p + 1] = nrm ? __ddiv_rn(a1, sumW) : a1;
  out[3 * (size_t)p + 2] = nrm ? __ddiv_rn(a2, sumW) : a2;
}

__global__ void kGather(int n, int width, const int* c2s, const double* in, double* out) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= (long)n * width) return;
  int c = (int)(i / width), k = (int)(i % width);
  out[i] = in[(long)c2s[c] * width + k];
}

// New load increment: D.oldTime = D, gradD.oldTime = gradD, F.oldTime = F,
// sigma.oldTime = sigma (OpenFOAM stores old-time values when time advances).
// The total form (tl == 2) keeps gradD.oldTime = 0 and F.oldTime = I, so
// that the TL kinematics give gradD = grad D and F = I + gradD^T; only
// D.oldTime, which converged() reads, moves on.
__global__ void kTlShift(MeshView mv, Controls c, FieldPtrs f, const DevState* st) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < mv.nC) {
    const double* U = f.D[st->dcur];
    if (c.tl == 2) {
      stV(f.D0, s, ldV(U, s));
      return;
    }
    stV(f.D0, s, ldV(f.D0, s) + ldV(U, s));
    stT(f.GD0, s, ldT(f.GD, s));
    stT(f.FL0, s, ldT(f.FL, s));
    stS(f.sig0, s, ldS(f.sig, s));
  }
}

__global__ void kTlShiftB(MeshView mv, Controls c, FieldPtrs f) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= mv.nB) return;
  // Only fixedDisplacement faces read D.oldTime on the boundary; at the end of
  // an increment their total displacement is the prescribed value.
  if (mv.btype[b] == 0) stV(f.D0b, b, c.loadFactor * ldV(mv.bval, b));
  stT(f.GD0b, b, ldT(f.GDb, b));
  stT(f.FL0b, b, ldT(f.FLb, b));
  stS(f.sig0b, b, ldS(f.sigb, b));
}

}  // namespace

void launchGeometry(const MeshView& mv, const GeomInputs& in, const GeomOutputs& out,
                    cudaStream_t s) {
  const int B = kRowBlock;
  kGeomCells<<<(mv.nC + B - 1) / B, B, 0, s>>>(mv, in, out);
  if (mv.nI > 0) kGeomFaces<<<(mv.nI + B - 1) / B, B, 0, s>>>(mv, in, out);
  double* bd = nullptr;
  cudaMallocAsync(&bd, sizeof(double) * 3 * (size_t)(mv.nB > 0 ? mv.nB : 1), s);
  if (mv.nB > 0) kGeomBFaces1<<<(mv.nB + B - 1) / B, B, 0, s>>>(mv, in, out, bd);
  kGeomLs<<<(mv.nC + B - 1) / B, B, 0, s>>>(mv, out, bd);
  cudaFreeAsync(bd, s);
}

void launchMatrix(const MeshView& mv, double gamma, double* val, double* diag, cudaStream_t s) {
  kMatrix<<<(mv.nC + kRowBlock - 1) / kRowBlock, kRowBlock, 0, s>>>(mv, gamma, val, diag);
}

void launchTractionInit(const MeshView& mv, const Controls& c, const FieldPtrs& f,
                        cudaStream_t s, int nCases) {
  if (mv.nB == 0) return;
  kTractionInit<<<dim3((mv.nB + kRowBlock - 1) / kRowBlock, nCases), kRowBlock, 0, s>>>(mv, c, f);
}

template <typename T>
void launchPost(const MeshView& mv, const Controls& c, const FieldPtrs& f, const T* x,
                DevState* st, double* partials, int mode, cudaStream_t s, LaunchTimer* tm,
                int nCases, const T* pA, const T* pB) {
  const int grid = (mv.nC + kRowBlock - 1) / kRowBlock;
  TimeScope ts(tm, S4G_K_POST, s);
  const dim3 g(mv.rowGrid, nCases);
  if (mode == 1) kApplyX<T><<<g, kRowBlock, 0, s>>>(mv, c, f, const_cast<T*>(x), pA, pB, st);
  kPost<T><<<g, kRowBlock, 0, s>>>(mv, c, f, x, st, partials, mode);
  if (c.tl && mode == 1) kPostLawTL<<<grid, kRowBlock, 0, s>>>(mv, c, f, st);
}

template <typename T>
void launchRhs(const MeshView& mv, const Controls& c, const FieldPtrs& f, T* x, T* r,
               DevState* st, double* partials, cudaStream_t s, LaunchTimer* tm, int nCases) {
  TimeScope ts(tm, S4G_K_RHS, s);
  const dim3 g(mv.rowGrid, nCases);
  if (mv.nI > 0) kRhsFace<<<g, kRowBlock, 0, s>>>(mv, c, f, st);
  kRhs<T><<<g, kRowBlock, 0, s>>>(mv, c, f, x, r, st, partials);
}

template void launchPost<double>(const MeshView&, const Controls&, const FieldPtrs&, const double*,
                                 DevState*, double*, int, cudaStream_t, LaunchTimer*, int,
                                 const double*, const double*);
template void launchPost<float>(const MeshView&, const Controls&, const FieldPtrs&, const float*,
                                DevState*, double*, int, cudaStream_t, LaunchTimer*, int,
                                const float*, const float*);
template void launchRhs<double>(const MeshView&, const Controls&, const FieldPtrs&, double*, double*,
                                DevState*, double*, cudaStream_t, LaunchTimer*, int);
template void launchRhs<float>(const MeshView&, const Controls&, const FieldPtrs&, float*, float*,
                               DevState*, double*, cudaStream_t, LaunchTimer*, int);

void launchGather(int n, int width, const int* c2s, const double* in, double* out, cudaStream_t s) {
  long tot = (long)n * width;
  kGather<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, width, c2s, in, out);
}

void launchPointInterp(int nP, const double* pts, const int* pcs, const int* pcc, const int* c2s,
                       const double* C, const double* U, const double* G, double* out,
                       cudaStream_t s) {
  if (nP > 0) kPointInterp<<<(nP + 255) / 256, 256, 0, s>>>(nP, pts, pcs, pcc, c2s, C, U, G, out);
}

void launchSetLoopCond(cudaGraphConditionalHandle h, DevState* st, int nRun, int which, int first,
                       unsigned limit, cudaStream_t s) {
  kSetLoopCond<<<1, 1, 0, s>>>(h, st, nRun, which, first, limit);
}

void launchTlShift(const MeshView& mv, const Controls& c, const FieldPtrs& f, DevState* st,
                   cudaStream_t s) {
  kTlShift<<<(mv.nC + kRowBlock - 1) / kRowBlock, kRowBlock, 0, s>>>(mv, c, f, st);
  if (mv.nB > 0 && c.tl == 1) kTlShiftB<<<(mv.nB + kRowBlock - 1) / kRowBlock, kRowBlock, 0, s>>>(mv, c, f);
}

}  // namespace s4g
