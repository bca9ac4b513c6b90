// Kernel launchers (host-callable wrappers around the device kernels).
#pragma once

#include "device_common.cuh"

namespace s4g {

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
  // total Lagrangian extras
  double* GD;  double* GD0;  double* GDb; double* GD0b;  // total gradient and old time
  double* Finv; double* Finvb; double* J; double* Jb;
  double* FL; double* FL0; double* FLb; double* FL0b;    // law's F and F.oldTime
  double* sig0; double* sig0b;                           // sigma.oldTime
};

// g = tractionBoundarySnGrad with the current sigma_b / grad_b (constructor).
void launchTractionInit(const MeshView& mv, const Controls& c, const FieldPtrs& f,
                        cudaStream_t s);
// Post-solve pass: D += x, boundary values, leastSquares gradient, law,
// boundary gradient/stress, next traction snGrad, convergence reductions.
// mode 0: constructor pass (no correction, no stress); 1: corrector.
void launchPost(const MeshView& mv, const Controls& c, const FieldPtrs& f, const double* x,
                DevState* st, double* partials, int mode, cudaStream_t s);
// RHS pass: R = div(sigma) + RhieChow + boundary terms, M*D_old for the
// residual normalisation; zeroes x, sets r = R.
void launchRhs(const MeshView& mv, const Controls& c, const FieldPtrs& f, double* x,
               double* r, DevState* st, double* partials, cudaStream_t s);
// out[c] = in[c2s[c]] for rows of `width` doubles.
void launchGather(int n, int width, const int* c2s, const double* in, double* out, cudaStream_t s);
// TL: new time step -- old-time fields take the converged values.
void launchTlShift(const MeshView& mv, const Controls& c, const FieldPtrs& f, DevState* st,
                   cudaStream_t s);

// ---- PCG (kernels_pcg.cu) ----------------------------------------------------
struct PcgPtrs {
  const double* val; const double* diag; double* rD;
  double* x; double* r; double* w; double* p[2]; double* q;
  unsigned* flags[2];  // per-part sweep flags (forward, backward)
};
// DIC factor: rD = 1/pivots by a scheduled forward sweep.
void launchDicFactor(const MeshView& mv, const PcgPtrs& p, DevState* st, int grid, cudaStream_t s);
// One PCG iteration for the three components (skips when converged).
void launchPcgIteration(const MeshView& mv, const Controls& c, const PcgPtrs& p, DevState* st,
                        double* partials, int sweepGrid, cudaStream_t s, long long* launches);
// Shared memory of the staged sweeps, threads per sweep block, and the
// per-kernel attribute set-up (returns resident sweep blocks per SM).
size_t sweepSmemBytes(const MeshView& mv);
int sweepBlockThreads();
cudaError_t sweepPrepare(const MeshView& mv, int* blocksPerSM);
void launchReciprocal(int n, double* rD, cudaStream_t s);
// Operator checks.
void launchAmul(const MeshView& mv, const double* val, const double* diag, const double* x,
                double* y, cudaStream_t s);
void launchPrecondOnly(const MeshView& mv, const Controls& c, const PcgPtrs& p, DevState* st,
                       double* partials, int sweepGrid, cudaStream_t s);

}  // namespace s4g
