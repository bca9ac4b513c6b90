// PCG kernels for the three displacement components of the segregated solve.
//
// Restates OpenFOAM's PCG solver (lduMatrix) with the DIC and diagonal
// preconditioners, as called by fvMatrix::solveSegregated from
// linGeomTotalDispSolid.C:164 / nonLinGeomTotalLagSolid.C:180: per component
// an independent conjugate-gradient iteration with its own alpha/beta, the
// residual normalised by OpenFOAM's normFactor, stopping at tolerance,
// relTol*initialResidual or maxIter.  The three components share the matrix,
// so every kernel streams the matrix once for all three right-hand sides.
//
// DIC sweeps.  The incomplete-Cholesky (zero fill) forward and backward
// substitutions are sequential in the DIC cell order.  Rows are stored in a
// topological order of that order's lower-triangular DAG, split into
// contiguous parts; inside a part, rows are grouped by in-part level.  A
// persistent grid takes parts from a ticket counter in topological order
// (forward) or reverse topological order (backward), waits -- with an
// iteration limit -- for the parts it depends on to publish an epoch flag,
// stages the part (its rows, its matrix entries and the remote values it
// reads) in shared memory, walks its levels with __syncthreads between them,
// writes the part back and publishes its own flag.  Every part a CTA waits
// for was taken earlier by a running CTA, so the scheme cannot deadlock.
// Values written by other CTAs in the same sweep are read with ld.global.cg
// (L2), never from a possibly stale L1 line.

#include "kernels.cuh"

namespace s4g {
namespace {

constexpr int kSweepSmBlock = 256;

__device__ __forceinline__ void waitPart(const unsigned* flag, unsigned epoch, unsigned* status) {
  for (int it = 0; it < kSpinLimit; ++it) {
    if (ldAcquire(flag) == epoch) return;
    if ((it & 63) == 63) __nanosleep(32);
  }
  atomicOr(status, kErrTimeout);
}

__device__ __forceinline__ int takeTicket(unsigned* ticket, int* sPart) {
  if (threadIdx.x == 0) *sPart = (int)atomicAdd(ticket, 1u);
  __syncthreads();
  const int t = *sPart;
  __syncthreads();
  return t;
}

__device__ __forceinline__ void sweepEpilogue(DevState* st, int dir, unsigned epoch) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&st->ctasDone[dir], 1u) == gridDim.x - 1) {
      st->ticket[dir] = 0;
      st->ctasDone[dir] = 0;
      st->epoch[dir] = epoch + 1;
      __threadfence();
    }
  }
}

// DIC factor (calcReciprocalD): pivot_u = diag_u - sum upper^2/pivot_l,
// once per matrix, scheduled like the forward sweep but reading global memory.
__global__ void __launch_bounds__(kSweepBlock)
kSweepFactor(MeshView mv, PcgPtrs p, DevState* st) {
  __shared__ int sPart;
  const unsigned epoch = st->epoch[0];
  for (;;) {
    const int part = takeTicket(&st->ticket[0], &sPart);
    if (part >= mv.nParts) break;
    const int pLo = mv.partStart[part];
    if (!mv.subdomains)
      for (int i = mv.upPtr[part] + threadIdx.x; i < mv.upPtr[part + 1]; i += blockDim.x)
        waitPart(p.flags[0] + mv.upIdx[i], epoch, &st->status);
    __syncthreads();
    for (int lvl = mv.lvlOff[part]; lvl < mv.lvlOff[part + 1]; ++lvl) {
      for (int row = mv.lvlStart[lvl] + threadIdx.x; row < mv.lvlStart[lvl + 1]; row += blockDim.x) {
        double dv = p.diag[row];
        for (int e = mv.rowptr[row]; e < mv.rowptr[row + 1]; ++e) {
          const int cl = mv.col[e];
          if (cl >= row) break;
          if (mv.subdomains && cl < pLo) continue;
          const double a = p.val[e];
          dv -= a * a / __ldcg(p.rD + cl);
        }
        __stcg(p.rD + row, dv);
      }
      __threadfence();
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      __threadfence();
      stRelease(p.flags[0] + part, epoch);
    }
  }
  sweepEpilogue(st, 0, epoch);
}

// Preconditioner sweep with the part staged in shared memory.
//   DIR 0 (forward):  w_u = rD_u r_u - sum_{l<u} (rD_u a_ul) w_l
//   DIR 1 (backward): w_l = w_l - sum_{u>l} (rD_l a_lu) w_u, plus w.r sums
// (OpenFOAM DICPreconditioner::precondition, face order per row.)
template <int DIR>
__global__ void __launch_bounds__(kSweepSmBlock)
kSweepSm(MeshView mv, PcgPtrs p, DevState* st, double* partials) {
  if (!st->pcgContinue) return;
  extern __shared__ double smem[];
  const int P = mv.maxRows, H = mv.maxHalo, EM = mv.maxEntries;
  double* wS = smem;                       // (P + H + 1) * 3
  double* rS = wS + 3 * (P + H + 1);       // P * 3
  double* dS = rS + 3 * P;                 // P
  double* vS = dS + P;                     // EM
  int* sS = (int*)(vS + EM);               // EM
  int* rpS = sS + EM;                      // P + 1
  __shared__ int sPart;
  __shared__ int sLast;
  __shared__ double red[32 * 3];
  const unsigned epoch = st->epoch[DIR];
  unsigned* flags = p.flags[DIR];
  for (;;) {
    const int t = takeTicket(&st->ticket[DIR], &sPart);
    if (t >= mv.nParts) break;
    const int part = DIR == 0 ? t : mv.nParts - 1 - t;
    const int pLo = mv.partStart[part], pHi = mv.partStart[part + 1];
    const int nR = pHi - pLo;
    const int e0 = mv.rowptr[pLo], nE = mv.rowptr[pHi] - e0;
    // stage what does not depend on other parts while waiting
    for (int i = threadIdx.x; i < nR; i += blockDim.x) {
      const int row = pLo + i;
      dS[i] = p.rD[row];
      rS[3 * i] = p.r[3 * row]; rS[3 * i + 1] = p.r[3 * row + 1]; rS[3 * i + 2] = p.r[3 * row + 2];
      rpS[i] = mv.rowptr[row] - e0;
      if (DIR == 1) {
        wS[3 * i] = __ldcg(p.w + 3 * row);
        wS[3 * i + 1] = __ldcg(p.w + 3 * row + 1);
        wS[3 * i + 2] = __ldcg(p.w + 3 * row + 2);
      }
    }
    for (int j = threadIdx.x; j < nE; j += blockDim.x) {
      vS[j] = p.val[e0 + j];
      sS[j] = mv.slot[e0 + j];
    }
    if (threadIdx.x == 0) rpS[nR] = nE;
    if (threadIdx.x < 3) wS[3 * (P + H) + threadIdx.x] = 0.0;  // zero slot
    // wait for the parts this one reads
    if (!mv.subdomains) {
      const int* dep = DIR == 0 ? mv.upIdx : mv.dnIdx;
      const int d0 = DIR == 0 ? mv.upPtr[part] : mv.dnPtr[part];
      const int d1 = DIR == 0 ? mv.upPtr[part + 1] : mv.dnPtr[part + 1];
      for (int i = d0 + threadIdx.x; i < d1; i += blockDim.x) waitPart(flags + dep[i], epoch, &st->status);
    }
    __syncthreads();
    {
      const int* hIdx = DIR == 0 ? mv.haloFIdx : mv.haloBIdx;
      const int h0 = DIR == 0 ? mv.haloFPtr[part] : mv.haloBPtr[part];
      const int h1 = DIR == 0 ? mv.haloFPtr[part + 1] : mv.haloBPtr[part + 1];
      for (int h = h0 + threadIdx.x; h < h1; h += blockDim.x) {
        const int row = hIdx[h];
        double* dst = wS + 3 * (P + h - h0);
        dst[0] = __ldcg(p.w + 3 * row);
        dst[1] = __ldcg(p.w + 3 * row + 1);
        dst[2] = __ldcg(p.w + 3 * row + 2);
      }
    }
    __syncthreads();
    const int l0 = mv.lvlOff[part], l1 = mv.lvlOff[part + 1];
    double dot[3] = {0, 0, 0};
    for (int li = 0; li < l1 - l0; ++li) {
      const int lvl = DIR == 0 ? l0 + li : l1 - 1 - li;
      const int r0 = mv.lvlStart[lvl] - pLo, r1 = mv.lvlStart[lvl + 1] - pLo;
      for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        const double rd = dS[i];
        const int j0 = rpS[i], j1 = rpS[i + 1];
        double v0, v1, v2;
        if (DIR == 0) {
          v0 = rd * rS[3 * i]; v1 = rd * rS[3 * i + 1]; v2 = rd * rS[3 * i + 2];
          for (int j = j0; j < j1; ++j) {
            const int sl = sS[j];
            if (sl < 0) break;
            const double tt = rd * vS[j];
            v0 -= tt * wS[3 * sl]; v1 -= tt * wS[3 * sl + 1]; v2 -= tt * wS[3 * sl + 2];
          }
        } else {
          v0 = wS[3 * i]; v1 = wS[3 * i + 1]; v2 = wS[3 * i + 2];
          for (int j = j1 - 1; j >= j0; --j) {
            const int sl = sS[j];
            if (sl >= 0) break;
            const int su = ~sl;
            const double tt = rd * vS[j];
            v0 -= tt * wS[3 * su]; v1 -= tt * wS[3 * su + 1]; v2 -= tt * wS[3 * su + 2];
          }
          dot[0] += v0 * rS[3 * i]; dot[1] += v1 * rS[3 * i + 1]; dot[2] += v2 * rS[3 * i + 2];
        }
        wS[3 * i] = v0; wS[3 * i + 1] = v1; wS[3 * i + 2] = v2;
      }
      __syncthreads();
    }
    // write the part back and publish it
    for (int k = threadIdx.x; k < 3 * nR; k += blockDim.x) __stcg(p.w + 3 * (size_t)pLo + k, wS[k]);
    if (DIR == 1) {
      blockSum<3>(dot, red);
      if (threadIdx.x == 0) {
        double* q = partials + 4 * (size_t)part;
        q[0] = dot[0]; q[1] = dot[1]; q[2] = dot[2];
      }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) stRelease(flags + part, epoch);
    if (DIR == 1) {
      // the CTA completing the last part reduces the w.r products
      if (threadIdx.x == 0) sLast = (atomicAdd(&st->partsDone[1], 1u) == (unsigned)mv.nParts - 1);
      __syncthreads();
      if (sLast) {
        double s[3];
        reducePartials<3>(partials, 4, mv.nParts, s, red);
        if (threadIdx.x == 0) {
          st->partsDone[1] = 0;
          for (int k = 0; k < 3; ++k)
            if (st->active[k]) {
              st->beta[k] = st->nIter[k] == 0 ? 0.0 : s[k] / st->wArA[k];
              st->wArA[k] = s[k];
            }
        }
      }
    }
  }
  sweepEpilogue(st, DIR, epoch);
}

__global__ void kReciprocal(int n, double* rD) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) rD[i] = 1.0 / rD[i];
}

// diagonal preconditioner: w = rD r, with the w.r sums
__global__ void __launch_bounds__(kRowBlock)
kDiagPrecond(MeshView mv, PcgPtrs p, DevState* st, double* partials) {
  if (!st->pcgContinue) return;
  __shared__ double smem[32 * 3];
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[3] = {0, 0, 0};
  if (s < mv.nC) {
    const double rd = p.rD[s];
    for (int k = 0; k < 3; ++k) {
      double v = rd * p.r[3 * s + k];
      p.w[3 * s + k] = v;
      acc[k] = v * p.r[3 * s + k];
    }
  }
  blockSum<3>(acc, smem);
  if (threadIdx.x == 0) {
    double* q = partials + 4 * (size_t)blockIdx.x;
    q[0] = acc[0]; q[1] = acc[1]; q[2] = acc[2];
  }
  if (!lastBlockDone(&st->counter[2], gridDim.x)) return;
  double sum[3];
  reducePartials<3>(partials, 4, gridDim.x, sum, smem);
  if (threadIdx.x != 0) return;
  st->counter[2] = 0;
  for (int k = 0; k < 3; ++k)
    if (st->active[k]) {
      st->beta[k] = st->nIter[k] == 0 ? 0.0 : sum[k] / st->wArA[k];
      st->wArA[k] = sum[k];
    }
}

// p = w + beta p (first iteration: p = w), q = A p, and the p.q products.
// Neighbour values of p are rebuilt from w and the previous p buffer, so one
// kernel both updates the search direction and multiplies by A.
__global__ void __launch_bounds__(kRowBlock)
kSpmvP(MeshView mv, PcgPtrs p, DevState* st, double* partials) {
  if (!st->pcgContinue) return;
  __shared__ double smem[32 * 3];
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int par = st->pcgIter & 1;
  const double* __restrict__ pold = p.p[par];
  double* __restrict__ pnew = p.p[par ^ 1];
  const double b0 = st->beta[0], b1 = st->beta[1], b2 = st->beta[2];
  const bool f0 = st->nIter[0] == 0, f1 = st->nIter[1] == 0, f2 = st->nIter[2] == 0;
  double acc[3] = {0, 0, 0};
  if (s < mv.nC) {
    const double dg = p.diag[s];
    const double w0 = p.w[3 * s], w1 = p.w[3 * s + 1], w2 = p.w[3 * s + 2];
    const double p0 = f0 ? w0 : w0 + b0 * pold[3 * s];
    const double p1 = f1 ? w1 : w1 + b1 * pold[3 * s + 1];
    const double p2 = f2 ? w2 : w2 + b2 * pold[3 * s + 2];
    double y0 = dg * p0, y1 = dg * p1, y2 = dg * p2;
    const int e1 = mv.rowptr[s + 1];
    for (int e = mv.rowptr[s]; e < e1; ++e) {
      const int cl = mv.col[e];
      const double a = p.val[e];
      const double n0 = p.w[3 * cl], n1 = p.w[3 * cl + 1], n2 = p.w[3 * cl + 2];
      y0 += a * (f0 ? n0 : n0 + b0 * pold[3 * cl]);
      y1 += a * (f1 ? n1 : n1 + b1 * pold[3 * cl + 1]);
      y2 += a * (f2 ? n2 : n2 + b2 * pold[3 * cl + 2]);
    }
    pnew[3 * s] = p0; pnew[3 * s + 1] = p1; pnew[3 * s + 2] = p2;
    p.q[3 * s] = y0; p.q[3 * s + 1] = y1; p.q[3 * s + 2] = y2;
    acc[0] = y0 * p0; acc[1] = y1 * p1; acc[2] = y2 * p2;
  }
  blockSum<3>(acc, smem);
  if (threadIdx.x == 0) {
    double* q = partials + 4 * (size_t)blockIdx.x;
    q[0] = acc[0]; q[1] = acc[1]; q[2] = acc[2];
  }
  if (!lastBlockDone(&st->counter[3], gridDim.x)) return;
  double sum[3];
  reducePartials<3>(partials, 4, gridDim.x, sum, smem);
  if (threadIdx.x != 0) return;
  st->counter[3] = 0;
  for (int k = 0; k < 3; ++k) {
    if (!st->active[k]) continue;
    st->wApA[k] = sum[k];
    if (fabs(sum[k]) / st->normFactor[k] < 1e-300) {  // checkSingularity: stop this component
      st->active[k] = 0;
      continue;
    }
    if (sum[k] <= 0) atomicOr(&st->status, kErrIndefinite);
    st->alpha[k] = st->wArA[k] / sum[k];
  }
}

// x += alpha p, r -= alpha q, residual sums and the convergence test.
__global__ void __launch_bounds__(kRowBlock)
kUpdate(MeshView mv, Controls c, PcgPtrs p, DevState* st, double* partials) {
  if (!st->pcgContinue) return;
  __shared__ double smem[32 * 3];
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int par = st->pcgIter & 1;
  const double* pnew = p.p[par ^ 1];
  const bool a0 = st->active[0], a1 = st->active[1], a2 = st->active[2];
  const double al0 = st->alpha[0], al1 = st->alpha[1], al2 = st->alpha[2];
  double acc[3] = {0, 0, 0};
  if (s < mv.nC) {
    double r0 = p.r[3 * s], r1 = p.r[3 * s + 1], r2 = p.r[3 * s + 2];
    if (a0) { p.x[3 * s] += al0 * pnew[3 * s]; r0 -= al0 * p.q[3 * s]; p.r[3 * s] = r0; }
    if (a1) { p.x[3 * s + 1] += al1 * pnew[3 * s + 1]; r1 -= al1 * p.q[3 * s + 1]; p.r[3 * s + 1] = r1; }
    if (a2) { p.x[3 * s + 2] += al2 * pnew[3 * s + 2]; r2 -= al2 * p.q[3 * s + 2]; p.r[3 * s + 2] = r2; }
    acc[0] = fabs(r0); acc[1] = fabs(r1); acc[2] = fabs(r2);
  }
  blockSum<3>(acc, smem);
  if (threadIdx.x == 0) {
    double* q = partials + 4 * (size_t)blockIdx.x;
    q[0] = acc[0]; q[1] = acc[1]; q[2] = acc[2];
  }
  if (!lastBlockDone(&st->counter[4], gridDim.x)) return;
  double sum[3];
  reducePartials<3>(partials, 4, gridDim.x, sum, smem);
  if (threadIdx.x != 0) return;
  st->counter[4] = 0;
  int any = 0;
  for (int k = 0; k < 3; ++k) {
    if (!st->active[k]) continue;
    const double fr = sum[k] / st->normFactor[k];
    st->finalRes[k] = fr;
    st->nIter[k] += 1;
    const bool conv = fr < c.tol || (c.relTol > 1e-20 && fr < c.relTol * st->initRes[k]);
    if (!isfinite(fr)) atomicOr(&st->status, kErrNaN);
    st->active[k] = (!conv && st->nIter[k] < c.maxIter && isfinite(fr)) ? 1 : 0;
    any |= st->active[k];
  }
  st->pcgIter += 1;
  st->pcgContinue = any;
}

__global__ void __launch_bounds__(kRowBlock)
kAmul(MeshView mv, const double* val, const double* diag, const double* x, double* y) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= mv.nC) return;
  double acc[3];
  for (int k = 0; k < 3; ++k) acc[k] = diag[s] * x[3 * s + k];
  for (int e = mv.rowptr[s]; e < mv.rowptr[s + 1]; ++e) {
    const int cl = mv.col[e];
    for (int k = 0; k < 3; ++k) acc[k] += val[e] * x[3 * cl + k];
  }
  for (int k = 0; k < 3; ++k) y[3 * s + k] = acc[k];
}

int rowGrid(const MeshView& mv) { return (mv.nC + kRowBlock - 1) / kRowBlock; }

void launchSweeps(const MeshView& mv, const PcgPtrs& p, DevState* st, double* partials,
                  int sweepGrid, cudaStream_t s) {
  const size_t sm = sweepSmemBytes(mv);
  kSweepSm<0><<<sweepGrid, kSweepSmBlock, sm, s>>>(mv, p, st, partials);
  kSweepSm<1><<<sweepGrid, kSweepSmBlock, sm, s>>>(mv, p, st, partials);
}

}  // namespace

size_t sweepSmemBytes(const MeshView& mv) {
  const size_t P = mv.maxRows, H = mv.maxHalo, EM = mv.maxEntries;
  return sizeof(double) * (3 * (P + H + 1) + 3 * P + P + EM) + sizeof(int) * (EM + P + 1);
}

int sweepBlockThreads() { return kSweepSmBlock; }

cudaError_t sweepPrepare(const MeshView& mv, int* blocksPerSM) {
  const int sm = (int)sweepSmemBytes(mv);
  cudaError_t e = cudaFuncSetAttribute(kSweepSm<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(kSweepSm<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, kSweepSm<0>, kSweepSmBlock, sm);
}

void launchDicFactor(const MeshView& mv, const PcgPtrs& p, DevState* st, int grid, cudaStream_t s) {
  kSweepFactor<<<grid, kSweepBlock, 0, s>>>(mv, p, st);
  kReciprocal<<<(mv.nC + 255) / 256, 256, 0, s>>>(mv.nC, p.rD);
}

void launchPcgIteration(const MeshView& mv, const Controls& c, const PcgPtrs& p, DevState* st,
                        double* partials, int sweepGrid, cudaStream_t s, long long* launches) {
  const int g = rowGrid(mv);
  if (c.precond == 0) {
    launchSweeps(mv, p, st, partials, sweepGrid, s);
    *launches += 2;
  } else {
    kDiagPrecond<<<g, kRowBlock, 0, s>>>(mv, p, st, partials);
    *launches += 1;
  }
  kSpmvP<<<g, kRowBlock, 0, s>>>(mv, p, st, partials);
  kUpdate<<<g, kRowBlock, 0, s>>>(mv, c, p, st, partials);
  *launches += 2;
}

void launchReciprocal(int n, double* rD, cudaStream_t s) {
  kReciprocal<<<(n + 255) / 256, 256, 0, s>>>(n, rD);
}

void launchAmul(const MeshView& mv, const double* val, const double* diag, const double* x,
                double* y, cudaStream_t s) {
  kAmul<<<rowGrid(mv), kRowBlock, 0, s>>>(mv, val, diag, x, y);
}

void launchPrecondOnly(const MeshView& mv, const Controls& c, const PcgPtrs& p, DevState* st,
                       double* partials, int sweepGrid, cudaStream_t s) {
  if (c.precond == 0) launchSweeps(mv, p, st, partials, sweepGrid, s);
  else kDiagPrecond<<<rowGrid(mv), kRowBlock, 0, s>>>(mv, p, st, partials);
}

}  // namespace s4g
