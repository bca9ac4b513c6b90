// PCG kernels for the three displacement components of the segregated solve.
//
// Restates OpenFOAM's PCG solver (lduMatrix) with the DIC and diagonal
// preconditioners, as called by fvMatrix::solveSegregated from
// linGeomTotalDispSolid.C:164 / nonLinGeomTotalLagSolid.C:180: per component
// an independent conjugate-gradient iteration with its own alpha/beta, the
// residual normalised by OpenFOAM's normFactor, stopping at tolerance,
// relTol*initialResidual or maxIter.  The three components share the matrix,
// so every kernel streams the matrix once for all three right-hand sides.
// The value type T is double for the plain FP64 path and float for the inner
// solve of the mixed-precision path; dot products and residual sums of the
// float path are compensated (Neumaier two-sum per thread, FP64 across
// threads).
//
// DIC sweeps.  The incomplete-Cholesky (zero fill) forward and backward
// substitutions are sequential in the DIC cell order.  Rows are stored in a
// topological order of that order's lower-triangular DAG, split into
// contiguous parts; inside a part, rows are grouped by in-part level.  A
// persistent grid takes parts from a ticket counter in topological order
// (forward) or reverse topological order (backward), waits -- with an
// iteration limit -- for the parts it depends on to publish an epoch flag,
// stages the part (its rows, its matrix coefficients and the remote values it
// reads) in shared memory, walks its levels with __syncthreads between them,
// writes the part back and publishes its own flag.  Every part a CTA waits
// for was taken earlier by a running CTA, so the scheme cannot deadlock.
// Values written by other CTAs in the same sweep are read with ld.global.cg
// (L2), never from a possibly stale L1 line.  The coefficients rD_row*a_e are
// precomputed once per matrix, as OpenFOAM's FDIC does (bit-identical to DIC).

#include <algorithm>

#include "kernels.cuh"
#include "pcg_common.cuh"

namespace s4g {
namespace {

constexpr int kSweepSmBlock = 64;

// Poll with relaxed loads (an acquire load per poll would also invalidate the
// SM's L1 each time), then one acquire fence once the flag is seen.
__device__ __forceinline__ void waitPart(const unsigned* flag, unsigned epoch, unsigned* status,
                                         int limit) {
  for (int it = 0; it < limit; ++it) {
    if (ldRelaxed(flag) == epoch) {
      fenceAcqRel();
      return;
    }
    if (it > 4096) __nanosleep(64);
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
// once per matrix in FP64, scheduled like the forward sweep but reading
// global memory.
__global__ void __launch_bounds__(kSweepBlock)
kSweepFactor(MeshView mv, const double* val, const double* diag, double* rD, unsigned* flags,
             DevState* st) {
  __shared__ int sPart;
  const unsigned epoch = st->epoch[0];
  for (;;) {
    const int part = takeTicket(&st->ticket[0], &sPart);
    if (part >= mv.nParts) break;
    const int pLo = mv.partStart[part];
    if (!mv.subdomains)
      for (int i = mv.upPtr[part] + threadIdx.x; i < mv.upPtr[part + 1]; i += blockDim.x)
        waitPart(flags + mv.upIdx[i], epoch, &st->status, mv.spinLimit);
    __syncthreads();
    for (int lvl = mv.lvlOff[part]; lvl < mv.lvlOff[part + 1]; ++lvl) {
      for (int row = mv.lvlStart[lvl] + threadIdx.x; row < mv.lvlStart[lvl + 1]; row += blockDim.x) {
        double dv = diag[row];
        for (int e = mv.rowptr[row]; e < mv.rowptr[row + 1]; ++e) {
          const int cl = mv.col[e];
          if (cl >= row) break;
          if (mv.subdomains && cl < pLo) continue;
          const double a = val[e];
          dv -= a * a / __ldcg(rD + cl);
        }
        __stcg(rD + row, dv);
      }
      __threadfence();
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      __threadfence();
      stRelease(flags + part, epoch);
    }
  }
  sweepEpilogue(st, 0, epoch);
}

// rD = 1/pivot; rDa[e] = rD[row]*val[e] (FDIC coefficients)
__global__ void kFactorFinish(MeshView mv, const double* val, double* rD, double* rDa) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= mv.nC) return;
  const double r = 1.0 / rD[s];
  rD[s] = r;
  for (int e = mv.rowptr[s]; e < mv.rowptr[s + 1]; ++e) rDa[e] = r * val[e];
}

__global__ void kReciprocal(int n, const double* diag, double* rD) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) rD[i] = 1.0 / diag[i];
}

__global__ void kToFloat(size_t n, const double* in, float* out) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}

// One thread's row of a level, read ahead of the level's barrier: start
// value (forward: rD r; backward: the forward result), the coefficients and
// shared-memory slots of the entries the sweep uses, in sweep order.
constexpr int kPreEntries = 4;
template <typename T>
struct RowPre {
  int i, n;
  T v0, v1, v2, r0, r1, r2;
  T a[kPreEntries];
  int sl[kPreEntries];
};

template <int DIR, typename T>
__device__ __forceinline__ void preRow(RowPre<T>& pr, int lvl, const int* lvS, const int* rpS,
                                       const int* loS, const int* sS, const T* aS, const T* dS,
                                       const T* rS, const T* wS, int pLo, int e0) {
  const int r0 = lvS[lvl] - pLo, r1 = lvS[lvl + 1] - pLo;
  const int i = r0 + threadIdx.x;
  if (i >= r1) { pr.i = -1; return; }
  pr.i = i;
  const int j0 = rpS[i] - e0, j1 = rpS[i + 1] - e0, nl = loS[i];
  if (DIR == 0) {
    const T rd = dS[i];
    pr.v0 = rd * rS[3 * i]; pr.v1 = rd * rS[3 * i + 1]; pr.v2 = rd * rS[3 * i + 2];
    pr.n = nl;
#pragma unroll
    for (int q = 0; q < kPreEntries; ++q)
      if (q < nl) { pr.sl[q] = sS[j0 + q]; pr.a[q] = aS[j0 + q]; }
  } else {
    pr.v0 = wS[3 * i]; pr.v1 = wS[3 * i + 1]; pr.v2 = wS[3 * i + 2];
    pr.r0 = rS[3 * i]; pr.r1 = rS[3 * i + 1]; pr.r2 = rS[3 * i + 2];
    pr.n = (j1 - j0) - nl;
#pragma unroll
    for (int q = 0; q < kPreEntries; ++q)
      if (q < pr.n) { pr.sl[q] = ~sS[j1 - 1 - q]; pr.a[q] = aS[j1 - 1 - q]; }
  }
}

// The same row update reading everything from shared memory (rows with more
// entries than kPreEntries, and rows beyond a thread's first of a level).
template <int DIR, typename T>
__device__ __forceinline__ void sweepRowGeneric(int i, T& v0, T& v1, T& v2, const int* rpS,
                                                const int* loS, const int* sS, const T* aS,
                                                const T* wS, int e0) {
  const int j0 = rpS[i] - e0, j1 = rpS[i + 1] - e0, nl = loS[i];
  if (DIR == 0) {
    for (int j = j0; j < j0 + nl; ++j) {
      const int sl = sS[j];
      const T a = aS[j];
      v0 -= a * wS[3 * sl]; v1 -= a * wS[3 * sl + 1]; v2 -= a * wS[3 * sl + 2];
    }
  } else {
    for (int j = j1 - 1; j >= j0 + nl; --j) {
      const int su = ~sS[j];
      const T a = aS[j];
      v0 -= a * wS[3 * su]; v1 -= a * wS[3 * su + 1]; v2 -= a * wS[3 * su + 2];
    }
  }
}

// Preconditioner sweep with the part staged in shared memory.
//   DIR 0 (forward):  w_u = rD_u r_u - sum_{l<u} (rD_u a_ul) w_l
//   DIR 1 (backward): w_l = w_l - sum_{u>l} (rD_l a_lu) w_u, plus w.r sums
// (OpenFOAM DIC/FDIC precondition, face order per row.)  NT threads per part.
template <int DIR, int NT, typename T>
__global__ void __launch_bounds__(NT, 1)
kSweepSm(MeshView mv, PcgPtrs<T> p, DevState* st, double* partials) {
  if (!st->pcgContinue) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int P = mv.maxRows, H = mv.maxHalo, EM = mv.maxEntries;
  T* wS = (T*)smraw;                       // (P + H + 1) * 3
  T* rS = wS + 3 * (P + H + 1);            // P * 3
  T* dS = rS + 3 * P;                      // P
  T* aS = dS + P;                          // EM: rD_row * a_e
  int* sS = (int*)(aS + EM);               // EM
  int* rpS = sS + EM;                      // P + 1
  int* lvS = rpS + P + 1;                  // maxLevels + 1: the part's level offsets
  int* loS = lvS + mv.maxLevels + 1;       // P: lower entries per row
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
    // stage what does not depend on other parts while waiting (the forward
    // results the backward sweep starts from were written by the previous
    // kernel, so they may go through L1)
    for (int j = threadIdx.x; j < nE; j += NT) {
      cpAsyncT(aS + j, p.rDa + e0 + j);
      cpAsync<4>(sS + j, mv.slot + e0 + j);
    }
    for (int i = threadIdx.x; i < nR; i += NT) {
      cpAsyncT(dS + i, p.rD + pLo + i);
      cpAsync<4>(rpS + i, mv.rowptr + pLo + i);
      cpAsync<4>(loS + i, mv.lowCnt + pLo + i);
    }
    for (int k = threadIdx.x; k < 3 * nR; k += NT) {
      cpAsyncT(rS + k, p.r + 3 * (size_t)pLo + k);
      if (DIR == 1) cpAsyncT(wS + k, p.w + 3 * (size_t)pLo + k);
    }
    const int l0 = mv.lvlOff[part], nL = mv.lvlOff[part + 1] - l0;
    for (int k = threadIdx.x; k <= nL; k += NT) cpAsync<4>(lvS + k, mv.lvlStart + l0 + k);
    if (threadIdx.x < 3) wS[3 * (P + H) + threadIdx.x] = T(0);  // zero slot
    // wait for the parts this one reads
    if (!mv.subdomains) {
      const int* dep = DIR == 0 ? mv.upIdx : mv.dnIdx;
      const int d0 = DIR == 0 ? mv.upPtr[part] : mv.dnPtr[part];
      const int d1 = DIR == 0 ? mv.upPtr[part + 1] : mv.dnPtr[part + 1];
      for (int i = d0 + threadIdx.x; i < d1; i += NT) waitPart(flags + dep[i], epoch, &st->status, mv.spinLimit);
    }
    __syncthreads();
    {
      const int* hIdx = DIR == 0 ? mv.haloFIdx : mv.haloBIdx;
      const int h0 = DIR == 0 ? mv.haloFPtr[part] : mv.haloBPtr[part];
      const int h1 = DIR == 0 ? mv.haloFPtr[part + 1] : mv.haloBPtr[part + 1];
      for (int h = h0 + threadIdx.x; h < h1; h += NT) {
        const int row = hIdx[h];
        const T a0 = __ldcg(p.w + 3 * row), a1 = __ldcg(p.w + 3 * row + 1),
                a2 = __ldcg(p.w + 3 * row + 2);
        T* dst = wS + 3 * (P + h - h0);
        dst[0] = a0; dst[1] = a1; dst[2] = a2;
      }
    }
    if (threadIdx.x == 0) rpS[nR] = e0 + nE;  // rpS holds absolute CSR offsets
    cpAsyncWaitAll();
    __syncthreads();
    Acc<T> dot0, dot1, dot2;
    // Software pipeline over levels: each thread's first row of the next
    // level has its static data (start value, coefficients, slots) read
    // before the barrier that ends the current level, so after the barrier
    // only the neighbour loads and the multiply-add chain remain.
    RowPre<T> cur, nxt;
    preRow<DIR>(cur, DIR == 0 ? 0 : nL - 1, lvS, rpS, loS, sS, aS, dS, rS, wS, pLo, e0);
    for (int li = 0; li < nL; ++li) {
      const int lvl = DIR == 0 ? li : nL - 1 - li;
      if (li + 1 < nL) preRow<DIR>(nxt, DIR == 0 ? li + 1 : nL - 2 - li, lvS, rpS, loS, sS, aS, dS, rS, wS, pLo, e0);
      if (cur.i >= 0) {
        T v0 = cur.v0, v1 = cur.v1, v2 = cur.v2;
        if (cur.n <= kPreEntries) {
#pragma unroll
          for (int q = 0; q < kPreEntries; ++q)
            if (q < cur.n) {
              const int sl = cur.sl[q];
              const T a = cur.a[q];
              v0 -= a * wS[3 * sl]; v1 -= a * wS[3 * sl + 1]; v2 -= a * wS[3 * sl + 2];
            }
        } else {
          sweepRowGeneric<DIR>(cur.i, v0, v1, v2, rpS, loS, sS, aS, wS, e0);
        }
        if (DIR == 1) { dot0.add(v0 * cur.r0); dot1.add(v1 * cur.r1); dot2.add(v2 * cur.r2); }
        wS[3 * cur.i] = v0; wS[3 * cur.i + 1] = v1; wS[3 * cur.i + 2] = v2;
      }
      // rows beyond the first NT of a wide level
      const int r0 = lvS[lvl] - pLo, r1 = lvS[lvl + 1] - pLo;
      for (int i = r0 + threadIdx.x + NT; i < r1; i += NT) {
        T v0, v1, v2;
        if (DIR == 0) {
          const T rd = dS[i];
          v0 = rd * rS[3 * i]; v1 = rd * rS[3 * i + 1]; v2 = rd * rS[3 * i + 2];
        } else {
          v0 = wS[3 * i]; v1 = wS[3 * i + 1]; v2 = wS[3 * i + 2];
        }
        sweepRowGeneric<DIR>(i, v0, v1, v2, rpS, loS, sS, aS, wS, e0);
        if (DIR == 1) { dot0.add(v0 * rS[3 * i]); dot1.add(v1 * rS[3 * i + 1]); dot2.add(v2 * rS[3 * i + 2]); }
        wS[3 * i] = v0; wS[3 * i + 1] = v1; wS[3 * i + 2] = v2;
      }
      cur = nxt;
      __syncthreads();
    }
    // write the part back and publish it: barrier, then one gpu-scope fence
    // and a release store by thread 0 (the cooperative-groups grid pattern)
    for (int k = threadIdx.x; k < 3 * nR; k += NT) __stcg(p.w + 3 * (size_t)pLo + k, wS[k]);
    if (DIR == 1) {
      double d3[3] = {dot0.value(), dot1.value(), dot2.value()};
      blockSum<3>(d3, red);
      if (threadIdx.x == 0) {
        double* q = partials + 4 * (size_t)part;
        q[0] = d3[0]; q[1] = d3[1]; q[2] = d3[2];
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      stRelease(flags + part, epoch);
    }
    if (DIR == 1) {
      // the CTA completing the last part reduces the w.r products
      if (threadIdx.x == 0) sLast = (atomicAdd(&st->partsDone[1], 1u) == (unsigned)mv.nParts - 1);
      __syncthreads();
      if (sLast) {
        double s[3];
        reduceRecords<3>(partials, 4, mv.nParts, s, (double*)smraw);  // the part is written back
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

// Row kernels: grid-stride loops over a few resident blocks per SM; the
// block that finishes last reduces the per-block records in a fixed order.
#define S4G_ROWS(s) for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < mv.nC; \
                         s += gridDim.x * blockDim.x)

// diagonal preconditioner: w = rD r, with the w.r sums
template <typename T>
__global__ void __launch_bounds__(kRowBlock)
kDiagPrecond(MeshView mv, PcgPtrs<T> p, DevState* st, double* partials) {
  if (!st->pcgContinue) return;
  __shared__ double smem[32 * 3];
  Acc<T> a0, a1, a2;
  S4G_ROWS(s) {
    const T rd = p.rD[s];
    const T r0 = p.r[3 * s], r1 = p.r[3 * s + 1], r2 = p.r[3 * s + 2];
    const T w0 = rd * r0, w1 = rd * r1, w2 = rd * r2;
    p.w[3 * s] = w0; p.w[3 * s + 1] = w1; p.w[3 * s + 2] = w2;
    a0.add(w0 * r0); a1.add(w1 * r1); a2.add(w2 * r2);
  }
  double acc[3] = {a0.value(), a1.value(), a2.value()};
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

// p = w (first iteration) or p = w + beta p
template <typename T>
__global__ void __launch_bounds__(kRowBlock)
kPUpdate(MeshView mv, PcgPtrs<T> p, const DevState* st) {
  if (!st->pcgContinue) return;
  bool act[3], first[3];
  T b[3];
  for (int k = 0; k < 3; ++k) {
    act[k] = st->active[k] != 0; first[k] = st->nIter[k] == 0; b[k] = (T)st->beta[k];
  }
  S4G_ROWS(s) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (!act[k]) continue;
      const T wv = p.w[3 * s + k];
      p.p[3 * s + k] = first[k] ? wv : wv + b[k] * p.p[3 * s + k];
    }
  }
}

// q = A p and the p.q products.
template <typename T>
__global__ void __launch_bounds__(kRowBlock)
kSpmv(MeshView mv, PcgPtrs<T> p, DevState* st, double* partials) {
  if (!st->pcgContinue) return;
  __shared__ double smem[32 * 3];
  Acc<T> a0, a1, a2;
  S4G_ROWS(s) {
    const T dg = p.diag[s];
    const T p0 = p.p[3 * s], p1 = p.p[3 * s + 1], p2 = p.p[3 * s + 2];
    T y0 = dg * p0, y1 = dg * p1, y2 = dg * p2;
    const int e1 = mv.rowptr[s + 1];
    for (int e = mv.rowptr[s]; e < e1; ++e) {
      const int cl = mv.col[e];
      const T a = p.val[e];
      y0 += a * p.p[3 * cl]; y1 += a * p.p[3 * cl + 1]; y2 += a * p.p[3 * cl + 2];
    }
    p.q[3 * s] = y0; p.q[3 * s + 1] = y1; p.q[3 * s + 2] = y2;
    a0.add(y0 * p0); a1.add(y1 * p1); a2.add(y2 * p2);
  }
  double acc[3] = {a0.value(), a1.value(), a2.value()};
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
template <typename T>
__global__ void __launch_bounds__(kRowBlock)
kUpdate(MeshView mv, Controls c, PcgPtrs<T> p, DevState* st, double* partials) {
  if (!st->pcgContinue) return;
  __shared__ double smem[32 * 3];
  bool act[3];
  T al[3];
  for (int k = 0; k < 3; ++k) { act[k] = st->active[k] != 0; al[k] = (T)st->alpha[k]; }
  Acc<T> acc3[3];
  S4G_ROWS(s) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      T rv = p.r[3 * s + k];
      if (act[k]) {
        p.x[3 * s + k] += al[k] * p.p[3 * s + k];
        rv -= al[k] * p.q[3 * s + k];
        p.r[3 * s + k] = rv;
      }
      acc3[k].add(fabs(rv));
    }
  }
  double acc[3] = {acc3[0].value(), acc3[1].value(), acc3[2].value()};
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

template <typename T>
__global__ void __launch_bounds__(kRowBlock)
kAmul(MeshView mv, const T* val, const T* diag, const T* x, T* y) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= mv.nC) return;
  T acc[3];
  for (int k = 0; k < 3; ++k) acc[k] = diag[s] * x[3 * s + k];
  for (int e = mv.rowptr[s]; e < mv.rowptr[s + 1]; ++e) {
    const int cl = mv.col[e];
    for (int k = 0; k < 3; ++k) acc[k] += val[e] * x[3 * cl + k];
  }
  for (int k = 0; k < 3; ++k) y[3 * s + k] = acc[k];
}

int rowGrid(const MeshView& mv) { return mv.rowGrid; }

template <typename T>
void launchSweeps(const MeshView& mv, const PcgPtrs<T>& p, DevState* st, double* partials,
                  int sweepGrid, cudaStream_t s, LaunchTimer* tm) {
  const size_t sm = sweepSmemBytes<T>(mv);
  {
    TimeScope ts(tm, S4G_K_SWEEP_FWD, s);
    kSweepSm<0, kSweepSmBlock, T><<<sweepGrid, kSweepSmBlock, sm, s>>>(mv, p, st, partials);
  }
  {
    TimeScope ts(tm, S4G_K_SWEEP_BWD, s);
    kSweepSm<1, kSweepSmBlock, T><<<sweepGrid, kSweepSmBlock, sm, s>>>(mv, p, st, partials);
  }
}

}  // namespace

template <typename T>
size_t sweepSmemBytes(const MeshView& mv) {
  const size_t P = mv.maxRows, H = mv.maxHalo, EM = mv.maxEntries;
  const size_t stage = sizeof(T) * (3 * (P + H + 1) + 3 * P + P + EM) +
                       sizeof(int) * (EM + P + 1 + mv.maxLevels + 1 + P);
  return std::max(stage, (size_t)256 * 3 * sizeof(double));  // final reduction scratch
}

template <typename T>
cudaError_t sweepPrepare(const MeshView& mv, int* blocksPerSM) {
  const int sm = (int)sweepSmemBytes<T>(mv);
  cudaError_t e = setMaxDynamicSmem(kSweepSm<0, kSweepSmBlock, T>);
  if (e != cudaSuccess) return e;
  e = setMaxDynamicSmem(kSweepSm<1, kSweepSmBlock, T>);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, kSweepSm<0, kSweepSmBlock, T>,
                                                       kSweepSmBlock, sm);
}

void launchDicFactor(const MeshView& mv, const double* val, const double* diag, double* rD,
                     double* rDa, unsigned* flags, DevState* st, int grid, cudaStream_t s) {
  kSweepFactor<<<grid, kSweepBlock, 0, s>>>(mv, val, diag, rD, flags, st);
  kFactorFinish<<<(mv.nC + kRowBlock - 1) / kRowBlock, kRowBlock, 0, s>>>(mv, val, rD, rDa);
}

void launchReciprocal(int n, const double* diag, double* rD, cudaStream_t s) {
  kReciprocal<<<(n + 255) / 256, 256, 0, s>>>(n, diag, rD);
}

void launchToFloat(size_t n, const double* in, float* out, cudaStream_t s) {
  if (n) kToFloat<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, in, out);
}

template <typename T>
void launchPcgIteration(const MeshView& mv, const Controls& c, const PcgPtrs<T>& p, DevState* st,
                        double* partials, int sweepGrid, cudaStream_t s, long long* launches,
                        LaunchTimer* tm) {
  const int g = rowGrid(mv);
  if (c.precond == 0) {
    launchSweeps(mv, p, st, partials, sweepGrid, s, tm);
    *launches += 2;
  } else {
    TimeScope ts(tm, S4G_K_DIAG, s);
    kDiagPrecond<T><<<g, kRowBlock, 0, s>>>(mv, p, st, partials);
    *launches += 1;
  }
  {
    TimeScope ts(tm, S4G_K_PUPDATE, s);
    kPUpdate<T><<<g, kRowBlock, 0, s>>>(mv, p, st);
  }
  {
    TimeScope ts(tm, S4G_K_SPMV, s);
    kSpmv<T><<<g, kRowBlock, 0, s>>>(mv, p, st, partials);
  }
  {
    TimeScope ts(tm, S4G_K_UPDATE, s);
    kUpdate<T><<<g, kRowBlock, 0, s>>>(mv, c, p, st, partials);
  }
  *launches += 3;
}

template <typename T>
void launchAmul(const MeshView& mv, const T* val, const T* diag, const T* x, T* y, cudaStream_t s) {
  kAmul<T><<<(mv.nC + kRowBlock - 1) / kRowBlock, kRowBlock, 0, s>>>(mv, val, diag, x, y);
}

template <typename T>
void launchPrecondOnly(const MeshView& mv, const Controls& c, const PcgPtrs<T>& p, DevState* st,
                       double* partials, int sweepGrid, cudaStream_t s) {
  if (c.precond == 0) launchSweeps(mv, p, st, partials, sweepGrid, s, nullptr);
  else kDiagPrecond<T><<<rowGrid(mv), kRowBlock, 0, s>>>(mv, p, st, partials);
}

#define S4G_INSTANTIATE(T)                                                                        \
  template size_t sweepSmemBytes<T>(const MeshView&);                                              \
  template cudaError_t sweepPrepare<T>(const MeshView&, int*);                                     \
  template void launchPcgIteration<T>(const MeshView&, const Controls&, const PcgPtrs<T>&,         \
                                      DevState*, double*, int, cudaStream_t, long long*,           \
                                      LaunchTimer*);                                               \
  template void launchAmul<T>(const MeshView&, const T*, const T*, const T*, T*, cudaStream_t);    \
  template void launchPrecondOnly<T>(const MeshView&, const Controls&, const PcgPtrs<T>&,          \
                                     DevState*, double*, int, cudaStream_t);
S4G_INSTANTIATE(double)
S4G_INSTANTIATE(float)
#undef S4G_INSTANTIATE

}  // namespace s4g
