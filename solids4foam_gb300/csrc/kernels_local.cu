// PCG with the processor-local DIC preconditioner, two kernels per iteration.
//
// In a decomposed run OpenFOAM's DIC preconditioner works on each
// processor's own matrix: coefficients that couple two processors are left
// out of the factor and out of the substitutions (block Jacobi over
// processors, an incomplete Cholesky inside each).  Here the processors are
// the library's cell parts.  With no coupling between parts, a part's whole
// preconditioning -- forward and backward substitution -- runs inside one
// CTA from shared memory, and the PCG iteration (lduMatrix PCG, as in
// kernels_pcg.cu) needs only two kernels:
//
//   kLocPrecond  x += alpha p, r -= alpha q for the components whose
//                iteration is pending, sum|r| (the residual test of that
//                iteration), then w = M^-1 r per part and the w.r sums; the
//                last CTA decides convergence, beta and wArA.
//   kLocSpmv     p_new = w + beta p_old and q = A p_new in one pass (a
//                neighbour's p_new is recomputed from its w and p_old, so p
//                is double-buffered), with the p.q sums; the last CTA decides
//                alpha (and the singularity stop).
//
// The residual test of iteration n thus runs in the kernel that also
// preconditions for iteration n+1; when the test stops a component, that
// preconditioning is simply not used.  The arithmetic of every vector entry
// is the one of the separate kernels; only the order of the global sums
// differs.
//
// Variants.  The SpMV step runs fused with a plain or an unrolled entry
// loop, or split into a p-update pass and an SpMV; kLocPrecond streams a
// part's rows with 4 (FP32) or 2 (FP64) rows per thread in flight, or half
// that.  The autotuner (engine) times them on the mesh
// and keeps the fastest.  The SpMV variants sum in the same order (same grid
// and block); kLocPrecond sums each part in a fixed order that does not
// depend on its block size, then over the parts in index order.  So all
// variants give bit-identical results.
//
// Part tables (HostPrep step 9): in-part entries per row, lower entries in
// CSR order then upper entries in reverse CSR order, coefficient rD_row*a_e
// and the column's row index inside the part (16 bits); per-row metadata
// (entry offset, lower and upper counts).  Both are padded per part so that
// they are staged with 16-byte cp.async copies while the CTA streams the
// x/r update.

#include <algorithm>

#include "kernels.cuh"
#include "pcg_common.cuh"

namespace s4g {
namespace {

// Bytes of one part's staged region (tables, w with its zero row, r, level
// starts), or of the final reduction's scratch if that is larger; rounded
// to 16 bytes so that regions can follow one another.
template <typename T>
__host__ __device__ inline size_t locRegionBytes(const MeshView& mv) {
  const size_t P = mv.maxRows, EL = mv.maxLocEntries, ML = mv.maxLocMeta;
  const size_t tables = sizeof(T) * (EL + 6 * P + 3) + 4 * ML + 2 * EL + sizeof(int) * (mv.maxLevels + 1);
  const size_t b = tables > (size_t)256 * 6 * sizeof(double) ? tables : (size_t)256 * 6 * sizeof(double);
  return (b + 15) / 16 * 16;
}

template <typename T>
struct LocSmem {
  T* c; uint32_t* m; uint16_t* idx; T* w; T* r; int* lv;
};

template <typename T>
__device__ __forceinline__ LocSmem<T> locSmem(const MeshView& mv, unsigned char* raw) {
  LocSmem<T> s;
  const int P = mv.maxRows, EL = mv.maxLocEntries, ML = mv.maxLocMeta;
  s.c = (T*)raw;                              // EL coefficients (EL % 8 == 0)
  s.m = (uint32_t*)(s.c + EL);                // ML row metadata (ML % 4 == 0)
  s.idx = (uint16_t*)(s.m + ML);              // EL local columns
  s.w = (T*)(s.idx + EL);                     // 3P + 3: the substitutions' vector
                                              // and the zero row P of the slots
  s.r = s.w + 3 * P + 3;                      // 3P: the updated residual
  s.lv = (int*)(s.r + 3 * P);                 // maxLevels + 1
  return s;
}

// The static data of one thread's row of a level (its metadata, entry
// columns and coefficients), read before the barrier that ends the level
// in progress, so that after it only the loads of the neighbours' values
// and the multiply-add chain remain.
constexpr int kLocPre = 3;
template <typename T>
struct LocRow {
  int i, n, j0;
  int q[kLocPre];
  T a[kLocPre];
};

template <int DIR, typename T>
__device__ __forceinline__ void locPre(const LocSmem<T>& sm, int l, int off, LocRow<T>& row) {
  row.i = sm.lv[l] + off;
  row.n = 0;
  if (row.i >= sm.lv[l + 1]) { row.i = -1; return; }
  const uint32_t m = sm.m[row.i];
  const int nl = (m >> 16) & 0xff;
  row.j0 = DIR == 0 ? (int)(m & 0xffff) : (int)(m & 0xffff) + nl;
  row.n = DIR == 0 ? nl : (int)(m >> 24);
#pragma unroll
  for (int u = 0; u < kLocPre; ++u)
    if (u < row.n) { row.q[u] = sm.idx[row.j0 + u]; row.a[u] = sm.c[row.j0 + u]; }
}

// v -= sum_j c_j w_idx(j) over the row's entries, in entry order.
template <typename T>
__device__ __forceinline__ void locApply(const LocSmem<T>& sm, const LocRow<T>& row) {
  const int i = row.i;
  T v0 = sm.w[3 * i], v1 = sm.w[3 * i + 1], v2 = sm.w[3 * i + 2];
#pragma unroll
  for (int u = 0; u < kLocPre; ++u)
    if (u < row.n) {
      const int q = row.q[u];
      const T a = row.a[u];
      v0 -= a * sm.w[3 * q]; v1 -= a * sm.w[3 * q + 1]; v2 -= a * sm.w[3 * q + 2];
    }
  for (int j = row.j0 + kLocPre; j < row.j0 + row.n; ++j) {
    const int q = sm.idx[j];
    const T c = sm.c[j];
    v0 -= c * sm.w[3 * q]; v1 -= c * sm.w[3 * q + 1]; v2 -= c * sm.w[3 * q + 2];
  }
  sm.w[3 * i] = v0; sm.w[3 * i + 1] = v1; sm.w[3 * i + 2] = v2;
}

// Warps that walk a part's levels (the rest of the CTA waits at a barrier).
constexpr int kLocWalkWarps = 2;

// Barrier of the walking warps: a warp barrier for one warp, a named CTA
// barrier (id 1) over the walking warps for more.
template <int W>
__device__ __forceinline__ void walkBarrier() {
  if (W == 1) __syncwarp();
  else asm volatile("bar.sync 1, %0;" ::"r"(32 * W) : "memory");
}

// One substitution (DIR 0 forward, 1 backward) over the part's levels, by W
// warps: the rows of a level in parallel (two per thread, more for a level
// wider than 64 W rows), a barrier of the walking warps between levels,
// and the next level's static data in registers while the current level
// runs.  A level's rows are few (at most 48 in an 8^3-cell part), so a
// couple of warps walk them while the rest of the CTA waits.
template <int DIR, int W, typename T>
__device__ __forceinline__ void locSweep(const LocSmem<T>& sm, int nL) {
  if (nL <= 0) return;
  constexpr int NW = 32 * W;
  const int lane = (int)threadIdx.x;
  LocRow<T> n0, n1;
  locPre<DIR>(sm, DIR == 0 ? 0 : nL - 1, lane, n0);
  locPre<DIR>(sm, DIR == 0 ? 0 : nL - 1, lane + NW, n1);
  for (int s = 0; s < nL; ++s) {
    const int l = DIR == 0 ? s : nL - 1 - s;
    const LocRow<T> c0 = n0, c1 = n1;
    if (s + 1 < nL) {
      locPre<DIR>(sm, DIR == 0 ? l + 1 : l - 1, lane, n0);
      locPre<DIR>(sm, DIR == 0 ? l + 1 : l - 1, lane + NW, n1);
    }
    if (c0.i >= 0) locApply(sm, c0);
    if (c1.i >= 0) locApply(sm, c1);
    // rows beyond the first 2 NW of a wide level
    for (int off = lane + 2 * NW; sm.lv[l] + off < sm.lv[l + 1]; off += NW) {
      LocRow<T> row;
      locPre<DIR>(sm, l, off, row);
      locApply(sm, row);
    }
    walkBarrier<W>();
  }
}

// Fixed-slot tables (HostPrep::locSlots): row r's lower entries sit at
// 6 r .. 6 r + 2 and its upper ones at 6 r + 3 .. 6 r + 5, padded with a zero
// coefficient on the zero row, so a row's whole static data is two short
// loads away from its index.
template <typename T>
struct SlotRow {
  int i;
  int q[3];
  T a[3];
};

template <int DIR, typename T>
__device__ __forceinline__ void slotPre(const LocSmem<T>& sm, int lo, int hi, int off,
                                        SlotRow<T>& row) {
  row.i = lo + off;
  if (row.i >= hi) { row.i = -1; return; }
  const int b = 6 * row.i + (DIR == 0 ? 0 : 3);
#pragma unroll
  for (int u = 0; u < 3; ++u) { row.q[u] = sm.idx[b + u]; row.a[u] = sm.c[b + u]; }
}

// v -= a_u w_q(u) for the three slots in order (a padded slot subtracts an
// exact zero); OUT (the backward substitution, which leaves w final): w also
// goes to global memory and into the thread's w.r and sum|r| sums.
template <bool OUT, typename T>
__device__ __forceinline__ void slotApply(const LocSmem<T>& sm, const SlotRow<T>& row,
                                          T* __restrict__ wg, Acc<T> (&wr)[3], Acc<T> (&ar)[3]) {
  const int i = row.i;
  T v[3] = {sm.w[3 * i], sm.w[3 * i + 1], sm.w[3 * i + 2]};
  T x[3][3];
#pragma unroll
  for (int u = 0; u < 3; ++u)
#pragma unroll
    for (int k = 0; k < 3; ++k) x[u][k] = sm.w[3 * row.q[u] + k];
#pragma unroll
  for (int u = 0; u < 3; ++u)
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k] -= row.a[u] * x[u][k];
#pragma unroll
  for (int k = 0; k < 3; ++k) sm.w[3 * i + k] = v[k];
  if (OUT) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      wg[3 * i + k] = v[k];
      const T r = sm.r[3 * i + k];
      wr[k].add(v[k] * r);
      ar[k].add(fabs(r));
    }
  }
}

// One substitution over the part's levels by W warps with the slot tables:
// the level bounds two levels ahead and the next level's slots are in
// registers before the current level's neighbour loads, so each level costs
// one round of shared-memory loads, the multiply-adds and a barrier.
template <int DIR, int W, bool OUT, typename T>
__device__ __forceinline__ void slotSweep(const LocSmem<T>& sm, int nL, T* __restrict__ wg,
                                          Acc<T> (&wr)[3], Acc<T> (&ar)[3]) {
  if (nL <= 0) return;
  constexpr int NW = 32 * W;
  const int t = (int)threadIdx.x;
  auto lvl = [&](int q) { return DIR == 0 ? q : nL - 1 - q; };
  int lo = sm.lv[lvl(0)], hi = sm.lv[lvl(0) + 1];
  int lo1 = 0, hi1 = 0;
  if (nL > 1) { lo1 = sm.lv[lvl(1)]; hi1 = sm.lv[lvl(1) + 1]; }
  SlotRow<T> n0, n1;
  slotPre<DIR>(sm, lo, hi, t, n0);
  slotPre<DIR>(sm, lo, hi, t + NW, n1);
  for (int q = 0; q < nL; ++q) {
    const SlotRow<T> c0 = n0, c1 = n1;
    const int clo = lo, chi = hi;
    lo = lo1; hi = hi1;
    if (q + 2 < nL) { lo1 = sm.lv[lvl(q + 2)]; hi1 = sm.lv[lvl(q + 2) + 1]; }
    if (q + 1 < nL) {
      slotPre<DIR>(sm, lo, hi, t, n0);
      slotPre<DIR>(sm, lo, hi, t + NW, n1);
    }
    if (c0.i >= 0) slotApply<OUT>(sm, c0, wg, wr, ar);
    if (c1.i >= 0) slotApply<OUT>(sm, c1, wg, wr, ar);
    // rows beyond the first 2 NW of a wide level
    for (int off = t + 2 * NW; clo + off < chi; off += NW) {
      SlotRow<T> row;
      slotPre<DIR>(sm, clo, chi, off, row);
      slotApply<OUT>(sm, row, wg, wr, ar);
    }
    walkBarrier<W>();
  }
}

// Two parts walked together by the same threads: per level, thread t takes
// row t of part A's level and row t of part B's level (parts may have
// different level counts), and both rows' loads are issued before either's
// multiply-adds -- two independent latency chains per level instead of one.
template <bool OUT, typename T>
__device__ __forceinline__ void slotApplyAB(const LocSmem<T>& sa, const SlotRow<T>& ra,
                                            T* __restrict__ wga, Acc<T> (&wra)[3], Acc<T> (&ara)[3],
                                            const LocSmem<T>& sb, const SlotRow<T>& rb,
                                            T* __restrict__ wgb, Acc<T> (&wrb)[3],
                                            Acc<T> (&arb)[3]) {
  const bool ha = ra.i >= 0, hb = rb.i >= 0;
  T va[3], vb[3], xa[3][3], xb[3][3];
  if (ha) {
#pragma unroll
    for (int k = 0; k < 3; ++k) va[k] = sa.w[3 * ra.i + k];
#pragma unroll
    for (int u = 0; u < 3; ++u)
#pragma unroll
      for (int k = 0; k < 3; ++k) xa[u][k] = sa.w[3 * ra.q[u] + k];
  }
  if (hb) {
#pragma unroll
    for (int k = 0; k < 3; ++k) vb[k] = sb.w[3 * rb.i + k];
#pragma unroll
    for (int u = 0; u < 3; ++u)
#pragma unroll
      for (int k = 0; k < 3; ++k) xb[u][k] = sb.w[3 * rb.q[u] + k];
  }
  if (ha) {
#pragma unroll
    for (int u = 0; u < 3; ++u)
#pragma unroll
      for (int k = 0; k < 3; ++k) va[k] -= ra.a[u] * xa[u][k];
#pragma unroll
    for (int k = 0; k < 3; ++k) sa.w[3 * ra.i + k] = va[k];
  }
  if (hb) {
#pragma unroll
    for (int u = 0; u < 3; ++u)
#pragma unroll
      for (int k = 0; k < 3; ++k) vb[k] -= rb.a[u] * xb[u][k];
#pragma unroll
    for (int k = 0; k < 3; ++k) sb.w[3 * rb.i + k] = vb[k];
  }
  if (OUT) {
    if (ha) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        wga[3 * ra.i + k] = va[k];
        const T r = sa.r[3 * ra.i + k];
        wra[k].add(va[k] * r);
        ara[k].add(fabs(r));
      }
    }
    if (hb) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        wgb[3 * rb.i + k] = vb[k];
        const T r = sb.r[3 * rb.i + k];
        wrb[k].add(vb[k] * r);
        arb[k].add(fabs(r));
      }
    }
  }
}

// The level bounds of one part during a pair walk, two levels ahead.
struct LevelCursor {
  int lo, hi, lo1, hi1;
};

template <int DIR, typename T>
__device__ __forceinline__ void cursorInit(const LocSmem<T>& sm, int nL, LevelCursor& c) {
  c.lo = c.hi = c.lo1 = c.hi1 = 0;
  if (nL > 0) { const int l = DIR == 0 ? 0 : nL - 1; c.lo = sm.lv[l]; c.hi = sm.lv[l + 1]; }
  if (nL > 1) { const int l = DIR == 0 ? 1 : nL - 2; c.lo1 = sm.lv[l]; c.hi1 = sm.lv[l + 1]; }
}

// Advance to level q + 1 (the bounds of q + 2 are loaded); empty past nL.
template <int DIR, typename T>
__device__ __forceinline__ void cursorStep(const LocSmem<T>& sm, int nL, int q, LevelCursor& c) {
  c.lo = c.lo1; c.hi = c.hi1;
  if (q + 2 < nL) {
    const int l = DIR == 0 ? q + 2 : nL - 3 - q;
    c.lo1 = sm.lv[l]; c.hi1 = sm.lv[l + 1];
  } else {
    c.lo1 = c.hi1 = 0;
  }
}

template <int DIR, int W, bool OUT, typename T>
__device__ __forceinline__ void slotSweepPair(const LocSmem<T>& sa, int nLa, T* __restrict__ wga,
                                              Acc<T> (&wra)[3], Acc<T> (&ara)[3],
                                              const LocSmem<T>& sb, int nLb, T* __restrict__ wgb,
                                              Acc<T> (&wrb)[3], Acc<T> (&arb)[3]) {
  constexpr int NW = 32 * W;
  const int t = (int)threadIdx.x;
  const int nL = nLa > nLb ? nLa : nLb;
  LevelCursor ca, cb;
  cursorInit<DIR>(sa, nLa, ca);
  cursorInit<DIR>(sb, nLb, cb);
  SlotRow<T> na, nb;
  slotPre<DIR>(sa, ca.lo, ca.hi, t, na);
  slotPre<DIR>(sb, cb.lo, cb.hi, t, nb);
  for (int q = 0; q < nL; ++q) {
    const SlotRow<T> cra = na, crb = nb;
    const int aLo = ca.lo, aHi = ca.hi, bLo = cb.lo, bHi = cb.hi;
    cursorStep<DIR>(sa, nLa, q, ca);
    cursorStep<DIR>(sb, nLb, q, cb);
    slotPre<DIR>(sa, ca.lo, ca.hi, t, na);
    slotPre<DIR>(sb, cb.lo, cb.hi, t, nb);
    slotApplyAB<OUT>(sa, cra, wga, wra, ara, sb, crb, wgb, wrb, arb);
    // rows beyond the first NW of a wide level
    for (int off = t + NW; aLo + off < aHi; off += NW) {
      SlotRow<T> row;
      slotPre<DIR>(sa, aLo, aHi, off, row);
      slotApply<OUT>(sa, row, wga, wra, ara);
    }
    for (int off = t + NW; bLo + off < bHi; off += NW) {
      SlotRow<T> row;
      slotPre<DIR>(sb, bLo, bHi, off, row);
      slotApply<OUT>(sb, row, wgb, wrb, arb);
    }
    walkBarrier<W>();
  }
}

template <typename T>
__global__ void kLocGather(int n, const int* src, const double* rDa, T* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = src[i] >= 0 ? (T)rDa[src[i]] : T(0);
}

// Resident blocks the register budget is set for (NT threads, RPT rows per
// thread in flight at once in the streaming phase).
template <typename T, int NT, int RPT>
constexpr int locMinBlocks() {
  return sizeof(T) == 4 ? 4 : (RPT >= 2 ? 3 : 4);
}

// Staging of one part: its tables by 16-byte cp.async, its level starts,
// the zero row (slot tables), and the pending update x += alpha p,
// r -= alpha q with RPT rows per thread in flight (every load issued before
// any store); r and w = rD r into shared memory.  The caller waits for the
// cp.async group and synchronises.
template <typename T, int NT, int RPT, bool SLOT>
__device__ __forceinline__ void locStage(const MeshView& mv, const PcgPtrs<T>& p,
                                         const LocSmem<T>& sm, const T* __restrict__ pg,
                                         const bool (&pend)[3], const T (&al)[3], int4 dA,
                                         int4 dB) {
  const int pLo = dA.x, nR = dA.y, eLo = dA.z, nE = dA.w;
  const int mLo = dB.x, nM = dB.y, l0 = dB.z, nL = dB.w;
  const T* __restrict__ qg = p.q;
  const T* __restrict__ rDg = p.rD;
  T* __restrict__ xg = p.x;
  T* __restrict__ rg = p.r;
  // static part tables in flight while the vectors stream
  {
    const int nc = nE * (int)sizeof(T) / 16;
    const char* g = (const char*)(p.lcoef + eLo);
    for (int k = threadIdx.x; k < nc; k += NT) cpAsync16((char*)sm.c + 16 * k, g + 16 * k);
    const int ni = nE * 2 / 16;
    const char* gi = (const char*)(mv.locIdx + eLo);
    for (int k = threadIdx.x; k < ni; k += NT) cpAsync16((char*)sm.idx + 16 * k, gi + 16 * k);
    const int nm = nM * 4 / 16;
    const char* gm = (const char*)(mv.locMeta + mLo);
    for (int k = threadIdx.x; k < nm; k += NT) cpAsync16((char*)sm.m + 16 * k, gm + 16 * k);
  }
  for (int k = threadIdx.x; k <= nL; k += NT) sm.lv[k] = mv.lvlStart[l0 + k] - pLo;
  if (SLOT && threadIdx.x < 3) sm.w[3 * mv.maxRows + threadIdx.x] = T(0);  // the zero row
  // pending update: RPT rows per thread with every load issued before
  // any store; r and w = rD r into shared memory
  for (int i0 = threadIdx.x; i0 < nR; i0 += RPT * NT) {
    T rv[RPT][3], qv[RPT][3], pv[RPT][3], xv[RPT][3], rd[RPT];
#pragma unroll
    for (int h = 0; h < RPT; ++h) {
      const int i = i0 + h * NT;
      if (i < nR) {
        const size_t g = 3 * (size_t)(pLo + i);
        rd[h] = rDg[pLo + i];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          rv[h][k] = rg[g + k];
          if (pend[k]) { qv[h][k] = qg[g + k]; pv[h][k] = pg[g + k]; xv[h][k] = xg[g + k]; }
        }
      }
    }
#pragma unroll
    for (int h = 0; h < RPT; ++h) {
      const int i = i0 + h * NT;
      if (i < nR) {
        const size_t g = 3 * (size_t)(pLo + i);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          if (pend[k]) {
            xg[g + k] = xv[h][k] + al[k] * pv[h][k];
            rv[h][k] -= al[k] * qv[h][k];
            rg[g + k] = rv[h][k];
          }
          sm.r[3 * i + k] = rv[h][k];
          sm.w[3 * i + k] = rd[h] * rv[h][k];
        }
      }
    }
  }
}

// After every part: the last CTA sums the part records in part order and
// decides, per component, the residual test of the pending iteration, beta
// and wArA, and whether the loop goes on.
__device__ __forceinline__ void locDecide(const MeshView& mv, const Controls& c, DevState* st,
                                          double* partials, bool anyPend, unsigned char* smraw) {
  if (!lastBlockDone(&st->counter[5], gridDim.x)) return;
  double S[6];
  reduceRecords<6>(partials, 8, mv.nParts, S, (double*)smraw);
  if (threadIdx.x != 0) return;
  st->counter[5] = 0;
  st->locTicket = 0;
  int any = 0;
  for (int k = 0; k < 3; ++k) {
    if (st->pending[k]) {
      st->pending[k] = 0;
      const double fr = S[3 + k] / st->normFactor[k];
      st->finalRes[k] = fr;
      st->nIter[k] += 1;
      const bool conv = fr < c.tol || (c.relTol > 1e-20 && fr < c.relTol * st->initRes[k]);
      if (!isfinite(fr)) atomicOr(&st->status, kErrNaN);
      st->active[k] = (!conv && st->nIter[k] < c.maxIter && isfinite(fr)) ? 1 : 0;
    }
    if (st->active[k]) {
      st->beta[k] = st->nIter[k] == 0 ? 0.0 : S[k] / st->wArA[k];
      st->wArA[k] = S[k];
    }
    any |= st->active[k];
  }
  if (anyPend) st->pcgIter += 1;
  st->pcgContinue = any;
}

// The processor-local preconditioner of one PCG iteration: the pending
// update x += alpha p, r -= alpha q, w = rD r, the forward and backward
// substitutions of each part inside one CTA, and the w.r and sum|r| sums.
//
// Streaming: each thread issues the loads of RPT rows at once (all the
// part's rows in one round trip when NT * RPT covers the part), while the
// part's tables arrive by 16-byte cp.async.  The updated residual and w go
// to shared memory.  Sums: per part, in a fixed order independent of NT
// and RPT (64 lanes over the rows, lane l summing rows l, l+64, ..., then a
// fixed tree), one record per part; the last CTA sums the records in part
// order.  Every variant therefore gives bit-identical results.
template <typename T, int NT, int RPT, bool SLOT>
__global__ void __launch_bounds__(NT, (locMinBlocks<T, NT, RPT>()))
kLocPrecond(MeshView mv, Controls c, PcgPtrs<T> p, DevState* st, double* partials) {
  p = casePcg(p, blockIdx.y, mv.nC);
  st += blockIdx.y;
  partials += (size_t)blockIdx.y * mv.caseRec;
  if (!st->pcgContinue) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  const LocSmem<T> sm = locSmem<T>(mv, smraw);
  __shared__ double red[2 * 6];
  // the vectors never alias one another
  const T* __restrict__ pg = st->pbuf ? p.p2 : p.p;  // p of the pending iteration
  bool pend[3];
  T al[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) { pend[k] = st->pending[k] != 0; al[k] = (T)st->alpha[k]; }
  const bool anyPend = pend[0] || pend[1] || pend[2];
  // Parts come from a ticket counter: CTAs that finish early take more (no
  // tail of CTAs with one part more than the others); the next ticket and
  // its part's descriptor are fetched while the current part runs.
  __shared__ int sTicket, sNextTicket;
  __shared__ int4 sDesc[2], sNextDesc[2];
  if (threadIdx.x == 0) {
    const int t0 = (int)atomicAdd(&st->locTicket, 1u);
    sTicket = t0;
    if (t0 < mv.nParts) { sDesc[0] = mv.locDesc[2 * t0]; sDesc[1] = mv.locDesc[2 * t0 + 1]; }
  }
  __syncthreads();
  for (int part = sTicket; part < mv.nParts;) {
    const int4 dA = sDesc[0], dB = sDesc[1];
    const int pLo = dA.x, nR = dA.y, nL = dB.w;
    // the next part's ticket and descriptor go straight to shared memory
    // (nothing of them stays in registers across the part)
    if (threadIdx.x == 0) {
      const int nt = (int)atomicAdd(&st->locTicket, 1u);
      sNextTicket = nt;
      if (nt < mv.nParts) { sNextDesc[0] = mv.locDesc[2 * nt]; sNextDesc[1] = mv.locDesc[2 * nt + 1]; }
    }
    locStage<T, NT, RPT, SLOT>(mv, p, sm, pg, pend, al, dA, dB);
    cpAsyncWaitAll();
    __syncthreads();
    // forward substitution: w_u -= sum_{l<u in part} (rD_u a_ul) w_l, then
    // backward substitution: w_l -= sum_{u>l in part} (rD_l a_lu) w_u
    T* __restrict__ wg = p.w + 3 * (size_t)pLo;
    double d6[6] = {0, 0, 0, 0, 0, 0};
    if constexpr (SLOT) {
      // the backward substitution also writes w out and sums w.r and |r|
      // over each walking thread's rows, in a fixed order; then a fixed tree
      if (threadIdx.x < 32 * kLocWalkWarps) {
        Acc<T> wr[3], ar[3];
        slotSweep<0, kLocWalkWarps, false>(sm, nL, wg, wr, ar);
        slotSweep<1, kLocWalkWarps, true>(sm, nL, wg, wr, ar);
#pragma unroll
        for (int k = 0; k < 3; ++k) { d6[k] = wr[k].value(); d6[3 + k] = ar[k].value(); }
      }
    } else {
      if (threadIdx.x < 32 * kLocWalkWarps) {
        locSweep<0, kLocWalkWarps>(sm, nL);
        locSweep<1, kLocWalkWarps>(sm, nL);
      }
      __syncthreads();
      // w out
      for (int k = threadIdx.x; k < 3 * nR; k += NT) wg[k] = sm.w[k];
      // the part's w.r and sum|r|: 64 lanes over the rows, then a fixed tree
      if (threadIdx.x < 64) {
        Acc<T> wr[3], ar[3];
        for (int i = threadIdx.x; i < nR; i += 64)
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const T r = sm.r[3 * i + k];
            wr[k].add(sm.w[3 * i + k] * r);
            ar[k].add(fabs(r));
          }
#pragma unroll
        for (int k = 0; k < 3; ++k) { d6[k] = wr[k].value(); d6[3 + k] = ar[k].value(); }
      }
    }
    sum64<6>(d6, red);  // ends with a barrier: the next part may reuse the shared memory
    if (threadIdx.x == 0) {
      double* q = partials + 8 * (size_t)part;
      for (int k = 0; k < 6; ++k) q[k] = d6[k];
      sTicket = sNextTicket;
      sDesc[0] = sNextDesc[0];
      sDesc[1] = sNextDesc[1];
    }
    __syncthreads();
    part = sTicket;
  }
  locDecide(mv, c, st, partials, anyPend, smraw);
}

// The slot-table preconditioner with two parts per CTA at a time: both are
// staged together and walked together (slotSweepPair), so each level's
// latency serves two parts.  Per part the arithmetic and the order of its
// sums are those of kLocPrecond, so the results are bit-identical to it.
// Shared memory: two part regions of localSmemBytes (rounded to 16 bytes).
// Resident blocks of the paired kernel: its two part regions bound it to
// three CTAs per SM in FP32 and two in FP64, so registers are set for that.
template <typename T>
constexpr int pairMinBlocks() {
  return sizeof(T) == 4 ? 3 : 2;
}

template <typename T, int NT, int RPT>
__global__ void __launch_bounds__(NT, (pairMinBlocks<T>()))
kLocPrecondPair(MeshView mv, Controls c, PcgPtrs<T> p, DevState* st, double* partials) {
  p = casePcg(p, blockIdx.y, mv.nC);
  st += blockIdx.y;
  partials += (size_t)blockIdx.y * mv.caseRec;
  if (!st->pcgContinue) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  const size_t region = locRegionBytes<T>(mv);
  const LocSmem<T> sa = locSmem<T>(mv, smraw);
  const LocSmem<T> sb = locSmem<T>(mv, smraw + region);
  __shared__ double red[2 * 12];
  const T* __restrict__ pg = st->pbuf ? p.p2 : p.p;
  bool pend[3];
  T al[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) { pend[k] = st->pending[k] != 0; al[k] = (T)st->alpha[k]; }
  const bool anyPend = pend[0] || pend[1] || pend[2];
  // tickets two at a time; the next pair's descriptors come ahead
  __shared__ int sTicket, sNextTicket;
  __shared__ int4 sDesc[4], sNextDesc[4];
  if (threadIdx.x == 0) {
    const int t0 = (int)atomicAdd(&st->locTicket, 2u);
    sTicket = t0;
    for (int j = 0; j < 2; ++j)
      if (t0 + j < mv.nParts) {
        sDesc[2 * j] = mv.locDesc[2 * (t0 + j)];
        sDesc[2 * j + 1] = mv.locDesc[2 * (t0 + j) + 1];
      }
  }
  __syncthreads();
  for (int part = sTicket; part < mv.nParts;) {
    const bool two = part + 1 < mv.nParts;
    const int4 aA = sDesc[0], aB = sDesc[1];
    int4 bA = aA, bB = aB;
    if (two) { bA = sDesc[2]; bB = sDesc[3]; }
    if (threadIdx.x == 0) {
      const int nt = (int)atomicAdd(&st->locTicket, 2u);
      sNextTicket = nt;
      for (int j = 0; j < 2; ++j)
        if (nt + j < mv.nParts) {
          sNextDesc[2 * j] = mv.locDesc[2 * (nt + j)];
          sNextDesc[2 * j + 1] = mv.locDesc[2 * (nt + j) + 1];
        }
    }
    locStage<T, NT, RPT, true>(mv, p, sa, pg, pend, al, aA, aB);
    if (two) locStage<T, NT, RPT, true>(mv, p, sb, pg, pend, al, bA, bB);
    cpAsyncWaitAll();
    __syncthreads();
    const int nLa = aB.w, nLb = two ? bB.w : 0;
    T* __restrict__ wga = p.w + 3 * (size_t)aA.x;
    T* __restrict__ wgb = p.w + 3 * (size_t)bA.x;
    double d[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) d[k] = 0;
    if (threadIdx.x < 32 * kLocWalkWarps) {
      Acc<T> wra[3], ara[3], wrb[3], arb[3];
      slotSweepPair<0, kLocWalkWarps, false>(sa, nLa, wga, wra, ara, sb, nLb, wgb, wrb, arb);
      slotSweepPair<1, kLocWalkWarps, true>(sa, nLa, wga, wra, ara, sb, nLb, wgb, wrb, arb);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        d[k] = wra[k].value(); d[3 + k] = ara[k].value();
        d[6 + k] = wrb[k].value(); d[9 + k] = arb[k].value();
      }
    }
    sum64<12>(d, red);  // ends with a barrier: the next parts may reuse the shared memory
    if (threadIdx.x == 0) {
      double* q = partials + 8 * (size_t)part;
      for (int k = 0; k < 6; ++k) q[k] = d[k];
      if (two) {
        q += 8;
        for (int k = 0; k < 6; ++k) q[k] = d[6 + k];
      }
      sTicket = sNextTicket;
      for (int j = 0; j < 4; ++j) sDesc[j] = sNextDesc[j];
    }
    __syncthreads();
    part = sTicket;
  }
  locDecide(mv, c, st, partials, anyPend, smraw);
}

// p_new = w (first iteration) or w + beta p_old, the same expression for a
// row and for its neighbours
template <typename T>
__device__ __forceinline__ T pNew(bool first, T w, T b, T po) { return first ? w : w + b * po; }

// U > 1: the first U entries of a row have all their loads issued before the
// multiply-adds; U == 1: a plain loop.
template <typename T, int U>
__global__ void __launch_bounds__(kRowBlock, (U > 1 ? (sizeof(T) == 4 ? 3 : 2) : 4))
kLocSpmv(MeshView mv, PcgPtrs<T> p, DevState* st, double* partials) {
  p = casePcg(p, blockIdx.y, mv.nC);
  st += blockIdx.y;
  partials += (size_t)blockIdx.y * mv.caseRec;
  if (!st->pcgContinue) return;
  __shared__ double red[32 * 3];
  const int pb = st->pbuf;
  // the vectors never alias one another
  const T* __restrict__ po = pb ? p.p2 : p.p;
  T* __restrict__ pn = pb ? p.p : p.p2;
  const T* __restrict__ wv = p.w;
  const T* __restrict__ val = p.val;
  const T* __restrict__ dia = p.diag;
  const int* __restrict__ col = mv.col;
  const int* __restrict__ rp = mv.rowptr;
  T* __restrict__ qo = p.q;
  bool act[3], first[3];
  T b[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    act[k] = st->active[k] != 0; first[k] = st->nIter[k] == 0; b[k] = (T)st->beta[k];
  }
  Acc<T> a0, a1, a2;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < mv.nC; s += gridDim.x * blockDim.x) {
    const T dg = dia[s];
    const T v0 = pNew(first[0], wv[3 * s], b[0], po[3 * s]);
    const T v1 = pNew(first[1], wv[3 * s + 1], b[1], po[3 * s + 1]);
    const T v2 = pNew(first[2], wv[3 * s + 2], b[2], po[3 * s + 2]);
    T y0 = dg * v0, y1 = dg * v1, y2 = dg * v2;
    const int e0 = rp[s], e1 = rp[s + 1];
    int e = e0;
    if (U > 1) {
      int cl[U];
      T a[U], n0[U], n1[U], n2[U];
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (e0 + u < e1) { cl[u] = col[e0 + u]; a[u] = val[e0 + u]; }
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (e0 + u < e1) {
          n0[u] = pNew(first[0], wv[3 * cl[u]], b[0], po[3 * cl[u]]);
          n1[u] = pNew(first[1], wv[3 * cl[u] + 1], b[1], po[3 * cl[u] + 1]);
          n2[u] = pNew(first[2], wv[3 * cl[u] + 2], b[2], po[3 * cl[u] + 2]);
        }
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (e0 + u < e1) { y0 += a[u] * n0[u]; y1 += a[u] * n1[u]; y2 += a[u] * n2[u]; }
      e = e0 + U;
    }
    for (; e < e1; ++e) {
      const int c2 = col[e];
      const T a2 = val[e];
      y0 += a2 * pNew(first[0], wv[3 * c2], b[0], po[3 * c2]);
      y1 += a2 * pNew(first[1], wv[3 * c2 + 1], b[1], po[3 * c2 + 1]);
      y2 += a2 * pNew(first[2], wv[3 * c2 + 2], b[2], po[3 * c2 + 2]);
    }
    if (act[0]) { pn[3 * s] = v0; qo[3 * s] = y0; }
    if (act[1]) { pn[3 * s + 1] = v1; qo[3 * s + 1] = y1; }
    if (act[2]) { pn[3 * s + 2] = v2; qo[3 * s + 2] = y2; }
    a0.add(y0 * v0); a1.add(y1 * v1); a2.add(y2 * v2);
  }
  double acc[3] = {a0.value(), a1.value(), a2.value()};
  blockSum<3>(acc, red);
  if (threadIdx.x == 0) {
    double* q = partials + 8 * (size_t)blockIdx.x;
    q[0] = acc[0]; q[1] = acc[1]; q[2] = acc[2];
  }
  if (!lastBlockDone(&st->counter[6], gridDim.x)) return;
  double sum[3];
  reducePartials<3>(partials, 8, gridDim.x, sum, red);
  if (threadIdx.x != 0) return;
  st->counter[6] = 0;
  int any = 0;
  for (int k = 0; k < 3; ++k) {
    if (!st->active[k]) continue;
    st->wApA[k] = sum[k];
    if (fabs(sum[k]) / st->normFactor[k] < 1e-300) {  // checkSingularity: stop this component
      st->active[k] = 0;
      continue;
    }
    if (sum[k] <= 0) atomicOr(&st->status, kErrIndefinite);
    st->alpha[k] = st->wArA[k] / sum[k];
    st->pending[k] = 1;
    any = 1;
  }
  st->pbuf = pb ^ 1;
  st->pcgContinue = any;
}

// Split form of the second kernel (FP64 favours it: a neighbour's p_new is
// formed once instead of once per face): p_new = w + beta p_old ...
template <typename T>
__global__ void __launch_bounds__(kRowBlock)
kLocPUpdate(MeshView mv, PcgPtrs<T> p, const DevState* st) {
  p = casePcg(p, blockIdx.y, mv.nC);
  st += blockIdx.y;
  if (!st->pcgContinue) return;
  const int pb = st->pbuf;
  const T* __restrict__ po = pb ? p.p2 : p.p;
  T* __restrict__ pn = pb ? p.p : p.p2;
  const T* __restrict__ wv = p.w;
  bool act[3], first[3];
  T b[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    act[k] = st->active[k] != 0; first[k] = st->nIter[k] == 0; b[k] = (T)st->beta[k];
  }
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < mv.nC; s += gridDim.x * blockDim.x)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (act[k]) pn[3 * s + k] = pNew(first[k], wv[3 * s + k], b[k], po[3 * s + k]);
}

// ... then q = A p_new with the p.q sums and the same decisions as kLocSpmv.
template <typename T>
__global__ void __launch_bounds__(kRowBlock, 4)
kLocSpmvSplit(MeshView mv, PcgPtrs<T> p, DevState* st, double* partials) {
  p = casePcg(p, blockIdx.y, mv.nC);
  st += blockIdx.y;
  partials += (size_t)blockIdx.y * mv.caseRec;
  if (!st->pcgContinue) return;
  __shared__ double red[32 * 3];
  const int pb = st->pbuf;
  const T* __restrict__ pn = pb ? p.p : p.p2;
  const T* __restrict__ val = p.val;
  const T* __restrict__ dia = p.diag;
  const int* __restrict__ col = mv.col;
  const int* __restrict__ rp = mv.rowptr;
  T* __restrict__ qo = p.q;
  bool act[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) act[k] = st->active[k] != 0;
  Acc<T> a0, a1, a2;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < mv.nC; s += gridDim.x * blockDim.x) {
    const T dg = dia[s];
    const T v0 = pn[3 * s], v1 = pn[3 * s + 1], v2 = pn[3 * s + 2];
    T y0 = dg * v0, y1 = dg * v1, y2 = dg * v2;
    const int e1 = rp[s + 1];
    for (int e = rp[s]; e < e1; ++e) {
      const int c2 = col[e];
      const T a2 = val[e];
      y0 += a2 * pn[3 * c2]; y1 += a2 * pn[3 * c2 + 1]; y2 += a2 * pn[3 * c2 + 2];
    }
    if (act[0]) qo[3 * s] = y0;
    if (act[1]) qo[3 * s + 1] = y1;
    if (act[2]) qo[3 * s + 2] = y2;
    a0.add(y0 * v0); a1.add(y1 * v1); a2.add(y2 * v2);
  }
  double acc[3] = {a0.value(), a1.value(), a2.value()};
  blockSum<3>(acc, red);
  if (threadIdx.x == 0) {
    double* q = partials + 8 * (size_t)blockIdx.x;
    q[0] = acc[0]; q[1] = acc[1]; q[2] = acc[2];
  }
  if (!lastBlockDone(&st->counter[6], gridDim.x)) return;
  double sum[3];
  reducePartials<3>(partials, 8, gridDim.x, sum, red);
  if (threadIdx.x != 0) return;
  st->counter[6] = 0;
  int any = 0;
  for (int k = 0; k < 3; ++k) {
    if (!st->active[k]) continue;
    st->wApA[k] = sum[k];
    if (fabs(sum[k]) / st->normFactor[k] < 1e-300) {  // checkSingularity: stop this component
      st->active[k] = 0;
      continue;
    }
    if (sum[k] <= 0) atomicOr(&st->status, kErrIndefinite);
    st->alpha[k] = st->wArA[k] / sum[k];
    st->pending[k] = 1;
    any = 1;
  }
  st->pbuf = pb ^ 1;
  st->pcgContinue = any;
}

template <typename T, int NT, int RPT>
void launchPrecondV(const MeshView& mv, const Controls& c, const PcgPtrs<T>& p, DevState* st,
                    double* partials, int grid, cudaStream_t s, int nCases) {
  if (mv.locSlots)
    kLocPrecond<T, NT, RPT, true><<<dim3(grid, nCases), NT, localSmemBytes<T>(mv), s>>>(
        mv, c, p, st, partials);
  else
    kLocPrecond<T, NT, RPT, false><<<dim3(grid, nCases), NT, localSmemBytes<T>(mv), s>>>(
        mv, c, p, st, partials);
}

template <typename T>
size_t pairSmemBytes(const MeshView& mv) {
  return 2 * locRegionBytes<T>(mv);
}

template <typename T, int NT, int RPT>
void launchPrecondPair(const MeshView& mv, const Controls& c, const PcgPtrs<T>& p, DevState* st,
                       double* partials, int grid, cudaStream_t s, int nCases) {
  kLocPrecondPair<T, NT, RPT><<<dim3(grid, nCases), NT, pairSmemBytes<T>(mv), s>>>(mv, c, p, st,
                                                                                  partials);
}

template <typename T, int NT, int RPT, bool SLOT>
cudaError_t prepareK(const MeshView& mv, int* blocksPerSM) {
  const int sm = (int)localSmemBytes<T>(mv);
  cudaError_t e = setMaxDynamicSmem(kLocPrecond<T, NT, RPT, SLOT>);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, kLocPrecond<T, NT, RPT, SLOT>,
                                                       NT, sm);
}

template <typename T, int NT, int RPT>
cudaError_t prepareV(const MeshView& mv, int* blocksPerSM) {
  return mv.locSlots ? prepareK<T, NT, RPT, true>(mv, blocksPerSM)
                     : prepareK<T, NT, RPT, false>(mv, blocksPerSM);
}

template <typename T, int NT, int RPT>
cudaError_t preparePair(const MeshView& mv, int* blocksPerSM) {
  cudaError_t e = setMaxDynamicSmem(kLocPrecondPair<T, NT, RPT>);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, kLocPrecondPair<T, NT, RPT>, NT,
                                                       (int)pairSmemBytes<T>(mv));
}

}  // namespace

// Preconditioner variants.  Slot-table meshes: one part per CTA at a time
// (0) or two walked together (1); other meshes: 4 (FP32) or 2 (FP64) rows
// per thread in flight while streaming (0), or half that (1).  All give
// bit-identical results.  perf.part_threads reports 128 threads per CTA.
const int kLocVariantsNT[kLocNumNT] = {128, 128};
const int kLocVariantsU[kLocNumU] = {1, 6, 0};

template <typename T>
size_t localSmemBytes(const MeshView& mv) {
  return locRegionBytes<T>(mv);
}

template <typename T>
cudaError_t localPrepare(const MeshView& mv, int* blocksPerSM) {
  constexpr int R0 = sizeof(T) == 4 ? 4 : 2, R1 = sizeof(T) == 4 ? 2 : 1;
  cudaError_t e = prepareV<T, 128, R0>(mv, &blocksPerSM[0]);
  if (e != cudaSuccess) return e;
  if (mv.locSlots) return preparePair<T, 128, R0>(mv, &blocksPerSM[1]);
  return prepareV<T, 128, R1>(mv, &blocksPerSM[1]);
}

template <typename T>
void launchLocalGather(int n, const int* src, const double* rDa, T* lcoef, cudaStream_t s) {
  if (n > 0) kLocGather<T><<<(n + 255) / 256, 256, 0, s>>>(n, src, rDa, lcoef);
}

template <typename T>
void launchLocalPrecond(const MeshView& mv, const Controls& c, const PcgPtrs<T>& p, DevState* st,
                        double* partials, const LocalTuning& t, cudaStream_t s, int nCases) {
  constexpr int R0 = sizeof(T) == 4 ? 4 : 2, R1 = sizeof(T) == 4 ? 2 : 1;
  if (t.ntIdx == 1) {
    if (mv.locSlots) launchPrecondPair<T, 128, R0>(mv, c, p, st, partials, t.grid[1], s, nCases);
    else launchPrecondV<T, 128, R1>(mv, c, p, st, partials, t.grid[1], s, nCases);
  } else {
    launchPrecondV<T, 128, R0>(mv, c, p, st, partials, t.grid[0], s, nCases);
  }
}

template <typename T>
void launchLocalSpmv(const MeshView& mv, const PcgPtrs<T>& p, DevState* st, double* partials,
                     const LocalTuning& t, cudaStream_t s, int nCases) {
  const dim3 g(mv.rowGrid, nCases);
  if (t.uIdx == 2) {
    kLocPUpdate<T><<<g, kRowBlock, 0, s>>>(mv, p, st);
    kLocSpmvSplit<T><<<g, kRowBlock, 0, s>>>(mv, p, st, partials);
  } else if (t.uIdx == 1) {
    kLocSpmv<T, 6><<<g, kRowBlock, 0, s>>>(mv, p, st, partials);
  } else {
    kLocSpmv<T, 1><<<g, kRowBlock, 0, s>>>(mv, p, st, partials);
  }
}

template <typename T>
void launchLocalIteration(const MeshView& mv, const Controls& c, const PcgPtrs<T>& p,
                          DevState* st, double* partials, const LocalTuning& t, cudaStream_t s,
                          long long* launches, LaunchTimer* tm, int nCases) {
  {
    TimeScope ts(tm, S4G_K_LOC_PRECOND, s);
    launchLocalPrecond<T>(mv, c, p, st, partials, t, s, nCases);
  }
  {
    TimeScope ts(tm, S4G_K_LOC_SPMV, s);
    launchLocalSpmv<T>(mv, p, st, partials, t, s, nCases);
  }
  *launches += t.uIdx == 2 ? 3 : 2;
}

#define S4G_INSTANTIATE(T)                                                                      \
  template size_t localSmemBytes<T>(const MeshView&);                                           \
  template cudaError_t localPrepare<T>(const MeshView&, int*);                                  \
  template void launchLocalGather<T>(int, const int*, const double*, T*, cudaStream_t);          \
  template void launchLocalPrecond<T>(const MeshView&, const Controls&, const PcgPtrs<T>&,      \
                                      DevState*, double*, const LocalTuning&, cudaStream_t,     \
                                      int);                                                     \
  template void launchLocalSpmv<T>(const MeshView&, const PcgPtrs<T>&, DevState*, double*,      \
                                   const LocalTuning&, cudaStream_t, int);                      \
  template void launchLocalIteration<T>(const MeshView&, const Controls&, const PcgPtrs<T>&,    \
                                        DevState*, double*, const LocalTuning&, cudaStream_t,   \
                                        long long*, LaunchTimer*, int);
S4G_INSTANTIATE(double)
S4G_INSTANTIATE(float)
#undef S4G_INSTANTIATE

}  // namespace s4g
