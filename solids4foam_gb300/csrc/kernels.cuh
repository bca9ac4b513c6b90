// Kernel launchers (host-callable wrappers around the device kernels).
#pragma once

#include <string>

#include "device_common.cuh"
#include "s4g.h"

namespace s4g {

// Optional per-kernel timing: before/after bracket one launch of a kernel
// kind (S4G_K_* of s4g.h) on the launch stream.
struct LaunchTimer {
  virtual void before(int kind, cudaStream_t s) = 0;
  virtual void after(int kind, cudaStream_t s) = 0;
  virtual ~LaunchTimer() {}
};
struct TimeScope {
  LaunchTimer* t; int k; cudaStream_t s;
  TimeScope(LaunchTimer* t_, int k_, cudaStream_t s_) : t(t_), k(k_), s(s_) { if (t) t->before(k, s); }
  ~TimeScope() { if (t) t->after(k, s); }
};

// ---- once per mesh (kernels_fv.cu) -----------------------------------------
struct GeomInputs {
  const double* Cc; const double* Cfc; const double* Sfc;  // caller order
  const int* s2c; const int* fcaller; const char* fflip; const int* bcaller;
  const int* bcell;
  int lsBoundaryDelta;
};
struct GeomOutputs {
  double* C; double* invDd;
  double* fS; double* fmagS; double* fw; double* fdelta;
  double* bS; double* bmagS; double* bn; double* bk; double* bdelta; double* bls;
  double* lsv;  // [2 nI][3] leastSquares vector of each CSR entry
};
void launchGeometry(const MeshView& mv, const GeomInputs& in, const GeomOutputs& out,
                    cudaStream_t s);

// Scalar momentum matrix (fvm::laplacian negated, SPD): val per CSR entry and
// diag per row, in FP64.
void launchMatrix(const MeshView& mv, double gamma, double* val, double* diag, cudaStream_t s);

// ---- per corrector (kernels_fv.cu) -----------------------------------------
struct FieldPtrs {
  double* D[2];  // [nC][3] double-buffered solved field (D or DD)
  double* D0;    // [nC][3] old-time total displacement
  double* D0b;   // [nB][3] old-time boundary displacement (TL)
  double* G;     // [nC][9] gradient of the solved field
  double* sig;   // [nC][6]
  double* Gb;    // [nB][9]
  double* sigb;  // [nB][6]
  double* g;     // [nB][3] traction snGrad
  double* gPrev; // [nB][3] the g the last corrector used (before its update)
  double* Ubr;   // [nB][3] field relaxation: the boundary values of the solved
                 // field after the last relaxation (D.prevIter on the boundary)
  double* aitA;  // [nC + nB] Aitken factor of each cell, then of each boundary face
  double* aitR;  // [nC + nB][3] Aitken residual D.prevIter - D of the last corrector
  // total Lagrangian extras
  double* GD;  double* GD0;  double* GDb; double* GD0b;  // total gradient and old time
  double* Finv; double* Finvb; double* J; double* Jb;
  double* FL; double* FL0; double* FLb; double* FL0b;    // law's F and F.oldTime
  double* sig0; double* sig0b;                           // sigma.oldTime
  double* flux;  // [nI][6] per internal face: owner-oriented flux of R and gamma|S|delta dU
};

// The fields of load case cs of a batch (linear-geometry model: the total
// Lagrangian fields are never batched).
__host__ __device__ inline FieldPtrs caseFields(FieldPtrs f, int cs, int nC, int nB, int nI) {
  if (cs == 0) return f;
  const size_t c = (size_t)cs;
  f.D[0] += c * 3 * nC; f.D[1] += c * 3 * nC; f.D0 += c * 3 * nC;
  if (f.D0b) f.D0b += c * 3 * nB;
  f.G += c * 9 * nC; f.sig += c * 6 * nC;
  f.Gb += c * 9 * nB; f.sigb += c * 6 * nB; f.g += c * 3 * nB;
  f.Ubr += c * 3 * nB; f.gPrev += c * 3 * nB;
  if (f.aitA) { f.aitA += c * (nC + nB); f.aitR += c * 3 * (nC + nB); }
  f.flux += c * 6 * nI;
  return f;
}

// g = tractionBoundarySnGrad with the current sigma_b / grad_b (constructor).
void launchTractionInit(const MeshView& mv, const Controls& c, const FieldPtrs& f,
                        cudaStream_t s, int nCases = 1);
// Post-solve pass: D += x, boundary values, leastSquares gradient, law,
// boundary gradient/stress, next traction snGrad, convergence reductions.
// mode 0: constructor pass (no correction, no stress); 1: corrector.
// pA, pB: the fused PCG's two p buffers (a pending x += alpha p is applied
// from the one DevState::pbuf names); null for the other PCG forms.
template <typename T>
void launchPost(const MeshView& mv, const Controls& c, const FieldPtrs& f, const T* x,
                DevState* st, double* partials, int mode, cudaStream_t s,
                LaunchTimer* tm = nullptr, int nCases = 1, const T* pA = nullptr,
                const T* pB = nullptr);
// RHS pass (FP64): R = div(sigma) + RhieChow + boundary terms, M*D_old for the
// residual normalisation; zeroes x, sets r = R rounded to the PCG type.
template <typename T>
void launchRhs(const MeshView& mv, const Controls& c, const FieldPtrs& f, T* x, T* r,
               DevState* st, double* partials, cudaStream_t s, LaunchTimer* tm = nullptr,
               int nCases = 1);
// pointD [nP][3] (caller point order) from the storage-order cell centres C,
// field U and gradient G, over the points' cells pcc (caller cell ids,
// CSR pcs); see kPointInterp.
void launchPointInterp(int nP, const double* pts, const int* pcs, const int* pcc, const int* c2s,
                       const double* C, const double* U, const double* G, double* out,
                       cudaStream_t s);
// out[c] = in[c2s[c]] for rows of `width` doubles.
void launchGather(int n, int width, const int* c2s, const double* in, double* out, cudaStream_t s);
// TL: new time step -- old-time fields take the converged values.
void launchTlShift(const MeshView& mv, const Controls& c, const FieldPtrs& f, DevState* st,
                   cudaStream_t s);

// Device-resident loops (CUDA graph conditional WHILE nodes): sets the
// condition of a loop from the device state of the nRun cases.  which = 0:
// the PCG loop of a corrector, continue while any case's pcgContinue (first
// = 1 at the corrector's start resets the iteration count); which = 1: the
// corrector loop, continue while any case is live.  Each loop is also
// bounded by `limit` iterations, past which the cases stop with the
// timeout bit set, so that a loop always ends; a case whose status has the
// timeout or NaN bit stops at once.
void launchSetLoopCond(cudaGraphConditionalHandle h, DevState* st, int nRun, int which, int first,
                       unsigned limit, cudaStream_t s);

// ---- PCG (kernels_pcg.cu) ----------------------------------------------------
// PCG arrays in the value type T of the inner solve: double (plain FP64) or
// float (FP32 inner solve of the mixed-precision path).
template <typename T>
struct PcgPtrs {
  const T* val; const T* diag; const T* rD;
  const T* rDa;        // rD[row] * val[e] per CSR entry (FDIC coefficients)
  T* x; T* r; T* w; T* p; T* q;
  unsigned* flags[2];  // per-part sweep flags (forward, backward)
  T* p2;               // second p buffer of the fused iteration
  const T* lcoef;      // in-part FDIC coefficients (processor-local DIC tables)
};

// The PCG vectors of load case cs of a batch ([case][nC][3] each); the
// matrix, the factor and the tables are shared.
template <typename T>
__host__ __device__ inline PcgPtrs<T> casePcg(PcgPtrs<T> p, int cs, int nC) {
  if (cs == 0) return p;
  const size_t o = (size_t)cs * 3 * nC;
  p.x += o; p.r += o; p.w += o; p.p += o; p.q += o;
  if (p.p2) p.p2 += o;
  return p;
}

// DIC factor in FP64: rD64 = 1/pivots by a scheduled forward sweep
// (flags[0] of the FP64 set), then rDa64 = rD64[row]*val64[e].
void launchDicFactor(const MeshView& mv, const double* val, const double* diag, double* rD,
                     double* rDa, unsigned* flags, DevState* st, int grid, cudaStream_t s);
// Diagonal preconditioner coefficients: rD = 1/diag, rDa unused.
void launchReciprocal(int n, const double* diag, double* rD, cudaStream_t s);
// FP32 copies of the FP64 matrix and factor for the mixed-precision path.
void launchToFloat(size_t n, const double* in, float* out, cudaStream_t s);

// One PCG iteration for the three components (skips when converged).
template <typename T>
void launchPcgIteration(const MeshView& mv, const Controls& c, const PcgPtrs<T>& p, DevState* st,
                        double* partials, int sweepGrid, cudaStream_t s, long long* launches,
                        LaunchTimer* tm = nullptr);
// Shared memory of the staged sweeps and the per-kernel attribute set-up
// (returns resident sweep blocks per SM).
template <typename T>
size_t sweepSmemBytes(const MeshView& mv);
template <typename T>
cudaError_t sweepPrepare(const MeshView& mv, int* blocksPerSM);
// Operator checks.
template <typename T>
void launchAmul(const MeshView& mv, const T* val, const T* diag, const T* x, T* y, cudaStream_t s);
template <typename T>
void launchPrecondOnly(const MeshView& mv, const Controls& c, const PcgPtrs<T>& p, DevState* st,
                       double* partials, int sweepGrid, cudaStream_t s);

// ---- processor-local DIC PCG (kernels_local.cu) -----------------------------
// Gathers the n in-part FDIC coefficients of the local tables from rDa (FP64):
// lcoef[i] = rDa[src[i]], 0 where src[i] < 0 (padding).
template <typename T>
void launchLocalGather(int n, const int* src, const double* rDa, T* lcoef, cudaStream_t s);
// Variant choice of the fused iteration (set by the engine's autotuner):
// the preconditioner runs with kLocVariantsNT[0] threads per part on
// grid[0] resident blocks; uIdx selects the fused SpMV with a plain (0) or
// unrolled (1) entry loop, or the split p-update + SpMV (2).  All SpMV
// variants compute bit-identical results.
constexpr int kLocNumNT = 2, kLocNumU = 3;
extern const int kLocVariantsNT[kLocNumNT];
// Threads per part of preconditioner variant `variant` on this mesh.
int localPartThreads(const MeshView& mv, int variant);
extern const int kLocVariantsU[kLocNumU];
struct LocalTuning {
  int ntIdx = 0, uIdx = 0;
  int grid[kLocNumNT] = {1, 1};
};
// One fused PCG iteration (two kernels): [x, r update of the previous
// iteration + residual test + processor-local DIC + w.r] and
// [p = w + beta p, q = A p, p.q].
template <typename T>
void launchLocalIteration(const MeshView& mv, const Controls& c, const PcgPtrs<T>& p,
                          DevState* st, double* partials, const LocalTuning& t, cudaStream_t s,
                          long long* launches, LaunchTimer* tm = nullptr, int nCases = 1);
// The two kernels on their own (autotuner).
template <typename T>
void launchLocalPrecond(const MeshView& mv, const Controls& c, const PcgPtrs<T>& p, DevState* st,
                        double* partials, const LocalTuning& t, cudaStream_t s, int nCases = 1);
template <typename T>
void launchLocalSpmv(const MeshView& mv, const PcgPtrs<T>& p, DevState* st, double* partials,
                     const LocalTuning& t, cudaStream_t s, int nCases = 1);
template <typename T>
size_t localSmemBytes(const MeshView& mv);
// Sets the shared-memory attribute of every preconditioner variant and
// returns resident blocks per SM of each (blocksPerSM[kLocNumNT]).
template <typename T>
cudaError_t localPrepare(const MeshView& mv, int* blocksPerSM);

// ---- operator product without allocation (noalloc.cu) ------------------------
// y = A x and x.Ax for k columns of host vectors in caller order, through the
// work vectors work0/work1 ([nC][3] doubles each) and a static scratch block;
// the matrix (val, diag) must already be assembled.  See noalloc.cu.
s4g_status opAmulDotNoAlloc(const MeshView& mv, const int* c2s, const double* val,
                            const double* diag, double* work0, double* work1, int device,
                            cudaStream_t s, int k, const double* x, double* y, double* xAx,
                            std::string& err);

}  // namespace s4g
