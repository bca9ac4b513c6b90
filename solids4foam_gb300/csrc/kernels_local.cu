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
//   kLocPrecondSlots / kLocPrecond
//                r -= alpha q for the components whose iteration is
//                pending, sum|r| (the residual test of that iteration),
//                then w = M^-1 r per part and the w.r sums; the last CTA
//                decides convergence, beta and wArA.
//   kLocSpmv     the pending iteration's x += alpha p (from the p_old it
//                reads anyway), p_new = w + beta p_old and q = A p_new in
//                one pass (a neighbour's p_new is recomputed from its w and
//                p_old, so p is double-buffered), with the p.q sums; the
//                last CTA decides alpha (and the singularity stop).  The
//                x update of a solve's last iteration is applied by kApplyX
//                after the loop (DevState::xPend).
//
// The residual test of iteration n thus runs in the kernel that also
// preconditions for iteration n+1; when the test stops a component, that
// preconditioning is simply not used.  The arithmetic of every vector entry
// is the one of the separate kernels; only the order of the global sums
// differs.
//
// Variants.  The SpMV step runs fused with a plain or an unrolled entry
// loop, or split into a p-update pass and an SpMV; the preconditioner runs
// with 128 or 64 threads per part (generic tables) or on two grids (slot
// tables: every resident CTA, or the smallest grid that gives every CTA the
// same number of parts).  The autotuner
// (engine) times them on the mesh and keeps the fastest.  The SpMV variants
// sum in the same order (same grid and block); the preconditioner sums each
// part in a fixed order that depends neither on its block size nor on its
// grid, then the parts in groups of 32 in part order, then the groups in
// group order.  So all variants give bit-identical results.
//
// Part tables (HostPrep step 9): in-part entries per row, lower entries in
// CSR order then upper entries in reverse CSR order, coefficient rD_row*a_e
// and the column's row index inside the part (16 bits); per-row metadata
// (entry offset, lower and upper counts).  Both are padded per part so that
// they are staged with 16-byte cp.async copies while the CTA streams the
// residual update.  Hexahedral parts use fixed 3 + 3 slots per row instead
// (HostPrep::locSlots, kLocPrecondSlots).

#include <algorithm>

#include "kernels.cuh"
#include "pcg_common.cuh"

namespace s4g {
namespace {

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

// Shared memory of the slot-table kernel: coefficients, columns, w with the
// zero row, level starts (no row metadata, no residual copy).
template <typename T>
__device__ __forceinline__ LocSmem<T> slotSmem(const MeshView& mv, unsigned char* raw) {
  LocSmem<T> s;
  const int P = mv.maxRows, EL = mv.maxLocEntries;
  s.c = (T*)raw;                              // EL coefficients (EL % 8 == 0)
  s.m = nullptr;
  s.idx = (uint16_t*)(s.c + EL);              // EL local columns
  s.w = (T*)(s.idx + EL);                     // 3P + 3
  s.r = nullptr;
  s.lv = (int*)(s.w + 3 * P + 3);             // maxLevels + 1
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
// exact zero).
template <typename T>
__device__ __forceinline__ void slotApply(const LocSmem<T>& sm, const SlotRow<T>& row) {
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
}

// One substitution (DIR 0 forward, 1 backward) of kLocPrecondSlots: all 64
// threads, one row per thread with its slots in registers a level ahead
// and the level bounds two levels ahead (rows past the first 64 of a wide
// level are read at the level), so each level costs one round of
// shared-memory loads, the multiply-adds and a CTA barrier.
template <int DIR, typename T>
__device__ __forceinline__ void slotWalk(const LocSmem<T>& sm, int nL) {
  if (nL <= 0) return;
  constexpr int NW = 64;
  const int t = (int)threadIdx.x;
  auto lvl = [&](int q) { return DIR == 0 ? q : nL - 1 - q; };
  int lo = sm.lv[lvl(0)], hi = sm.lv[lvl(0) + 1];
  int lo1 = 0, hi1 = 0;
  if (nL > 1) { lo1 = sm.lv[lvl(1)]; hi1 = sm.lv[lvl(1) + 1]; }
  SlotRow<T> n0;
  slotPre<DIR>(sm, lo, hi, t, n0);
  for (int q = 0; q < nL; ++q) {
    const SlotRow<T> c0 = n0;
    const int clo = lo, chi = hi;
    lo = lo1; hi = hi1;
    if (q + 2 < nL) { lo1 = sm.lv[lvl(q + 2)]; hi1 = sm.lv[lvl(q + 2) + 1]; }
    if (q + 1 < nL) slotPre<DIR>(sm, lo, hi, t, n0);
    if (c0.i >= 0) slotApply(sm, c0);
    for (int off = t + NW; clo + off < chi; off += NW) {
      SlotRow<T> row;
      slotPre<DIR>(sm, clo, chi, off, row);
      slotApply(sm, row);
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void kLocGather(int n, const int* src, const double* rDa, T* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = src[i] >= 0 ? (T)rDa[src[i]] : T(0);
}

// Part records in groups of kLocGroup parts: the CTA whose part completes a
// group (the last to arrive on the group's counter) sums the group's records
// in part order by a fixed shuffle tree, and the last CTA of the launch sums
// the group records -- one round trip each instead of one CTA reading every
// part record at the end of the launch.
constexpr int kLocGroup = 32;

__device__ __forceinline__ int locGroupSize(int g, int nParts) {
  const int n = nParts - g * kLocGroup;
  return n < kLocGroup ? n : kLocGroup;
}

// Thread 0: the arrival of `part`'s record (written by this thread) on its
// group's counter; true if it completes the group.
__device__ __forceinline__ bool locArrive(unsigned* gcnt, int part, int nParts) {
  __threadfence();
  const int g = part / kLocGroup;
  return atomicAdd(&gcnt[g], 1u) + 1u == (unsigned)locGroupSize(g, nParts);
}

// One warp: the record (N values) of group g (lane j holds part g*32 + j),
// and the group's counter back to zero for the next launch.
template <int N = 6>
__device__ __forceinline__ void locGroupSum(const double* rec, double* grec, unsigned* gcnt, int g,
                                            int nParts) {
  const int lane = threadIdx.x & 31;
  const int part = g * kLocGroup + lane;
  __threadfence();
  double v[N];
#pragma unroll
  for (int k = 0; k < N; ++k) v[k] = part < nParts ? __ldcg(rec + 8 * (size_t)part + k) : 0.0;
#pragma unroll
  for (int k = 0; k < N; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) grec[8 * (size_t)g + k] = v[k];
    gcnt[g] = 0;
  }
}

// The last CTA: the sum of the group records in group order -- lane v of
// 64 sums groups v, v + 64, ..., then a fixed tree.  Result in thread 0.
template <int N>
__device__ __forceinline__ void locGroupsTotal(const double* grec, int nGroups, double (&S)[N],
                                               double* red) {
#pragma unroll
  for (int k = 0; k < N; ++k) S[k] = 0;
  if (threadIdx.x < 64)
    for (int g = threadIdx.x; g < nGroups; g += 64)
#pragma unroll
      for (int k = 0; k < N; ++k) S[k] += __ldcg(grec + 8 * (size_t)g + k);
  sum64<N>(S, red);
}

// End of a preconditioner launch, after the CTA's last part: thread 0
// reports that part on its group counter (warp 0 sums the group if that
// completes it); the last CTA sums the group records in group order -- lane
// v of 64 sums groups v, v + 64, ..., then a fixed tree -- and decides, per
// component, the residual test of the pending iteration, beta and wArA, and
// whether the loop goes on.  Block size >= 64.
__device__ __forceinline__ void locFinish(const MeshView& mv, const Controls& c, DevState* st,
                                          double* partials, int lastPart, bool anyPend,
                                          double* red, int* sGroup) {
  double* grec = partials + mv.locGrpOff;
  unsigned* gcnt = reinterpret_cast<unsigned*>(grec + 8 * (size_t)mv.locGroups);
  const int t = (int)threadIdx.x;
  if (t == 0)
    *sGroup = (lastPart >= 0 && locArrive(gcnt, lastPart, mv.nParts)) ? lastPart / kLocGroup : -1;
  __syncthreads();
  if (*sGroup >= 0 && t < 32) locGroupSum(partials, grec, gcnt, *sGroup, mv.nParts);
  if (!lastBlockDone(&st->counter[5], gridDim.x)) return;
  double S[6];
  locGroupsTotal<6>(grec, mv.locGroups, S, red);
  if (t != 0) return;
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

// Resident blocks the register budget is set for (NT threads, RPT rows per
// thread in flight at once in the streaming phase).  With 64 threads every
// thread walks; FP32 parts (about 31 KB of shared memory at 8^3 cells) then
// fit seven CTAs per SM, each walking its own part.
template <typename T, int NT, int RPT>
constexpr int locMinBlocks() {
  return NT == 64 ? (sizeof(T) == 4 ? 7 : 4) : (sizeof(T) == 4 ? 4 : (RPT >= 2 ? 3 : 4));
}

// The processor-local preconditioner of one PCG iteration: the pending
// update r -= alpha q, w = rD r, the forward and backward substitutions of
// each part inside one CTA, and the w.r and sum|r| sums.
//
// Streaming: each thread issues the loads of RPT rows at once (all the
// part's rows in one round trip when NT * RPT covers the part), while the
// part's tables arrive by 16-byte cp.async.  The updated residual and w go
// to shared memory.  Sums: per part, in a fixed order independent of NT
// and RPT (64 lanes over the rows, lane l summing rows l, l+64, ..., then a
// fixed tree), one record per part; the records are summed in groups of 32
// parts and the group records in group order (locFinish).  Every variant
// therefore gives bit-identical results.  Used for generic part tables;
// hexahedral parts with slot tables go to kLocPrecondSlots.
template <typename T, int NT, int RPT>
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
  const T* __restrict__ qg = p.q;
  const T* __restrict__ rDg = p.rD;
  T* __restrict__ rg = p.r;
  bool pend[3];
  T al[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) { pend[k] = st->pending[k] != 0; al[k] = (T)st->alpha[k]; }
  const bool anyPend = pend[0] || pend[1] || pend[2];
  // Parts come from a ticket counter: CTAs that finish early take more (no
  // tail of CTAs with one part more than the others); the next ticket and
  // its part's descriptor are fetched while the current part runs.
  __shared__ int sTicket, sNextTicket, sGroup;
  __shared__ int4 sDesc[2], sNextDesc[2];
  double* grec = partials + mv.locGrpOff;
  unsigned* gcnt = reinterpret_cast<unsigned*>(grec + 8 * (size_t)mv.locGroups);
  int prev = -1;
  if (threadIdx.x == 0) {
    const int t0 = (int)atomicAdd(&st->locTicket, 1u);
    sTicket = t0;
    if (t0 < mv.nParts) { sDesc[0] = mv.locDesc[2 * t0]; sDesc[1] = mv.locDesc[2 * t0 + 1]; }
  }
  __syncthreads();
  for (int part = sTicket; part < mv.nParts;) {
    const int4 dA = sDesc[0], dB = sDesc[1];
    const int pLo = dA.x, nR = dA.y, eLo = dA.z, nE = dA.w;
    const int mLo = dB.x, nM = dB.y, l0 = dB.z, nL = dB.w;
    // the next part's ticket and descriptor go straight to shared memory
    // (nothing of them stays in registers across the part)
    // and the previous part's record is reported on its group counter
    bool done = false;
    if (threadIdx.x == 0) {
      const int nt = (int)atomicAdd(&st->locTicket, 1u);
      if (prev >= 0) done = locArrive(gcnt, prev, mv.nParts);
      sNextTicket = nt;
      if (nt < mv.nParts) { sNextDesc[0] = mv.locDesc[2 * nt]; sNextDesc[1] = mv.locDesc[2 * nt + 1]; }
    }
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
    // pending update r -= alpha q (x += alpha p is the SpMV pass's): RPT
    // rows per thread with every load issued before any store; r and
    // w = rD r into shared memory
    for (int i0 = threadIdx.x; i0 < nR; i0 += RPT * NT) {
      T rv[RPT][3], qv[RPT][3], rd[RPT];
#pragma unroll
      for (int h = 0; h < RPT; ++h) {
        const int i = i0 + h * NT;
        if (i < nR) {
          const size_t g = 3 * (size_t)(pLo + i);
          rd[h] = rDg[pLo + i];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            rv[h][k] = rg[g + k];
            if (pend[k]) qv[h][k] = qg[g + k];
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
              rv[h][k] -= al[k] * qv[h][k];
              rg[g + k] = rv[h][k];
            }
            sm.r[3 * i + k] = rv[h][k];
            sm.w[3 * i + k] = rd[h] * rv[h][k];
          }
        }
      }
    }
    cpAsyncWaitAll();
    __syncthreads();
    // forward substitution: w_u -= sum_{l<u in part} (rD_u a_ul) w_l, then
    // backward substitution: w_l -= sum_{u>l in part} (rD_l a_lu) w_u
    T* __restrict__ wg = p.w + 3 * (size_t)pLo;
    double d6[6] = {0, 0, 0, 0, 0, 0};
    {
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
    if (threadIdx.x == 0) sGroup = done ? prev / kLocGroup : -1;
    sum64<6>(d6, red);  // ends with a barrier: the next part may reuse the shared memory
    if (threadIdx.x == 0) {
      double* q = partials + 8 * (size_t)part;
      for (int k = 0; k < 6; ++k) q[k] = d6[k];
      sTicket = sNextTicket;
      sDesc[0] = sNextDesc[0];
      sDesc[1] = sNextDesc[1];
    }
    __syncthreads();
    if (sGroup >= 0 && threadIdx.x < 32) locGroupSum(partials, grec, gcnt, sGroup, mv.nParts);
    prev = part;
    part = sTicket;
  }
  locFinish(mv, c, st, partials, prev, anyPend, red, &sGroup);
}

// The slot-table preconditioner (hexahedral parts, HostPrep::locSlots): 64
// threads per part, all of them walking.  Parts go to CTAs in a fixed
// stride (CTA b takes b, b + G, ...); the next part's descriptor arrives by
// cp.async with the current part's tables.  It streams r, q and rD (RPT
// rows per thread in flight), and a thread keeps the updated residual of its
// rows t, t + 64, ... (up to 8 rows) in registers, so the
// shared memory holds only the tables and w, and eight FP32 parts (five
// FP64) of 512 rows fit per SM.  After the walk w leaves in one coalesced
// pass and each thread sums w.r and |r| over its rows in row order, then a
// fixed tree: a part's record depends neither on the grid nor on RPT, so
// every variant gives bit-identical results.
template <typename T, int RPT>
__global__ void __launch_bounds__(64, (sizeof(T) == 4 ? 8 : 5))
kLocPrecondSlots(MeshView mv, Controls c, PcgPtrs<T> p, DevState* st, double* partials) {
  constexpr int NT = 64, KR = 8;
  p = casePcg(p, blockIdx.y, mv.nC);
  st += blockIdx.y;
  partials += (size_t)blockIdx.y * mv.caseRec;
  if (!st->pcgContinue) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  const LocSmem<T> sm = slotSmem<T>(mv, smraw);
  __shared__ double red[2 * 6];
  __shared__ __align__(16) int4 sDesc[2][2];
  __shared__ int sGroup;
  double* grec = partials + mv.locGrpOff;
  unsigned* gcnt = reinterpret_cast<unsigned*>(grec + 8 * (size_t)mv.locGroups);
  // the vectors never alias one another
  const T* __restrict__ qg = p.q;
  const T* __restrict__ rDg = p.rD;
  T* __restrict__ rg = p.r;
  bool pend[3];
  T al[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) { pend[k] = st->pending[k] != 0; al[k] = (T)st->alpha[k]; }
  const bool anyPend = pend[0] || pend[1] || pend[2];
  const int t = (int)threadIdx.x;
  const int nParts = mv.nParts;
  if (t < 3) sm.w[3 * mv.maxRows + t] = T(0);  // the zero row of the padded slots
  int part = (int)blockIdx.x;
  if (t == 0 && part < nParts) {
    cpAsync16(&sDesc[0][0], mv.locDesc + 2 * part);
    cpAsync16(&sDesc[0][1], mv.locDesc + 2 * part + 1);
  }
  cpAsyncWaitAll();
  __syncthreads();
  int prev = -1, buf = 0;
  for (; part < nParts; part += (int)gridDim.x, buf ^= 1) {
    const int4 dA = sDesc[buf][0], dB = sDesc[buf][1];
    const int pLo = dA.x, nR = dA.y, eLo = dA.z, nE = dA.w;
    const int l0 = dB.z, nL = dB.w;
    const int next = part + (int)gridDim.x;
    if (t == 0 && next < nParts) {
      cpAsync16(&sDesc[buf ^ 1][0], mv.locDesc + 2 * next);
      cpAsync16(&sDesc[buf ^ 1][1], mv.locDesc + 2 * next + 1);
    }
    // static part tables in flight while the vectors stream
    {
      const int nc = nE * (int)sizeof(T) / 16;
      const char* g = (const char*)(p.lcoef + eLo);
      for (int k = t; k < nc; k += NT) cpAsync16((char*)sm.c + 16 * k, g + 16 * k);
      const int ni = nE * 2 / 16;
      const char* gi = (const char*)(mv.locIdx + eLo);
      for (int k = t; k < ni; k += NT) cpAsync16((char*)sm.idx + 16 * k, gi + 16 * k);
    }
    for (int k = t; k <= nL; k += NT) sm.lv[k] = mv.lvlStart[l0 + k] - pLo;
    // pending update r -= alpha q and w = rD r, RPT rows per thread with
    // every load issued before any store (x += alpha p is the SpMV pass's).
    // Thread 0 reports the previous part's record on its group counter
    // while the first loads are in flight.
    bool done = false;
    T rK[KR][3];
    const bool regR = nR <= KR * NT;
    if (regR) {
#pragma unroll
      for (int it = 0; it < KR / RPT; ++it) {
        T qv[RPT][3], rd[RPT];
#pragma unroll
        for (int h = 0; h < RPT; ++h) {
          const int j = it * RPT + h, i = t + j * NT;
          if (i < nR) {
            const size_t g = 3 * (size_t)(pLo + i);
            rd[h] = rDg[pLo + i];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
              rK[j][k] = rg[g + k];
              if (pend[k]) qv[h][k] = qg[g + k];
            }
          }
        }
        if (it == 0 && t == 0 && prev >= 0) done = locArrive(gcnt, prev, nParts);
#pragma unroll
        for (int h = 0; h < RPT; ++h) {
          const int j = it * RPT + h, i = t + j * NT;
          if (i < nR) {
            const size_t g = 3 * (size_t)(pLo + i);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
              if (pend[k]) {
                rK[j][k] -= al[k] * qv[h][k];
                rg[g + k] = rK[j][k];
              }
              sm.w[3 * i + k] = rd[h] * rK[j][k];
            }
          }
        }
      }
    } else {
      if (t == 0 && prev >= 0) done = locArrive(gcnt, prev, nParts);
      for (int i0 = t; i0 < nR; i0 += RPT * NT) {
        T rv[RPT][3], qv[RPT][3], rd[RPT];
#pragma unroll
        for (int h = 0; h < RPT; ++h) {
          const int i = i0 + h * NT;
          if (i < nR) {
            const size_t g = 3 * (size_t)(pLo + i);
            rd[h] = rDg[pLo + i];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
              rv[h][k] = rg[g + k];
              if (pend[k]) qv[h][k] = qg[g + k];
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
                rv[h][k] -= al[k] * qv[h][k];
                rg[g + k] = rv[h][k];
              }
              sm.w[3 * i + k] = rd[h] * rv[h][k];
            }
          }
        }
      }
    }
    cpAsyncWaitAll();
    __syncthreads();
    // forward then backward substitution (each level ends with a barrier of
    // all 64 threads, so after the last one w is final for every thread)
    slotWalk<0>(sm, nL);
    slotWalk<1>(sm, nL);
    // w out in one coalesced pass; w.r and sum|r| over the thread's rows
    // t, t + 64, ... in row order
    T* __restrict__ wg = p.w + 3 * (size_t)pLo;
    for (int k = t; k < 3 * nR; k += NT) wg[k] = sm.w[k];
    Acc<T> wr[3], ar[3];
    if (regR) {
#pragma unroll
      for (int j = 0; j < KR; ++j) {
        const int i = t + j * NT;
        if (i < nR)
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            wr[k].add(sm.w[3 * i + k] * rK[j][k]);
            ar[k].add(fabs(rK[j][k]));
          }
      }
    } else {
      // each thread reads back the residual rows it wrote itself
      for (int i = t; i < nR; i += NT)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const T r = rg[3 * (size_t)(pLo + i) + k];
          wr[k].add(sm.w[3 * i + k] * r);
          ar[k].add(fabs(r));
        }
    }
    double d6[6];
#pragma unroll
    for (int k = 0; k < 3; ++k) { d6[k] = wr[k].value(); d6[3 + k] = ar[k].value(); }
    if (t == 0) sGroup = done ? prev / kLocGroup : -1;
    sum64<6>(d6, red);  // ends with a barrier: the next part may reuse the shared memory
    if (t == 0) {
      double* q = partials + 8 * (size_t)part;
#pragma unroll
      for (int k = 0; k < 6; ++k) q[k] = d6[k];
    }
    if (sGroup >= 0 && t < 32) locGroupSum(partials, grec, gcnt, sGroup, nParts);
    prev = part;
  }
  locFinish(mv, c, st, partials, prev, anyPend, red, &sGroup);
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
  T* __restrict__ xg = p.x;
  bool act[3], first[3], xp[3];
  T b[3], al[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    act[k] = st->active[k] != 0; first[k] = st->nIter[k] == 0; b[k] = (T)st->beta[k];
    xp[k] = st->xPend[k] != 0; al[k] = (T)st->alpha[k];
  }
  Acc<T> a0, a1, a2;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < mv.nC; s += gridDim.x * blockDim.x) {
    const T dg = dia[s];
    // the pending iteration's x += alpha p, from the p_old read here anyway
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (xp[k]) xg[3 * s + k] = xg[3 * s + k] + al[k] * po[3 * s + k];
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
    st->xPend[k] = 0;  // applied by this pass
    if (!st->active[k]) continue;
    st->wApA[k] = sum[k];
    if (fabs(sum[k]) / st->normFactor[k] < 1e-300) {  // checkSingularity: stop this component
      st->active[k] = 0;
      continue;
    }
    if (sum[k] <= 0) atomicOr(&st->status, kErrIndefinite);
    st->alpha[k] = st->wArA[k] / sum[k];
    st->pending[k] = 1;
    st->xPend[k] = 1;
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
  T* __restrict__ xg = p.x;
  bool act[3], first[3], xp[3];
  T b[3], al[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    act[k] = st->active[k] != 0; first[k] = st->nIter[k] == 0; b[k] = (T)st->beta[k];
    xp[k] = st->xPend[k] != 0; al[k] = (T)st->alpha[k];
  }
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < mv.nC; s += gridDim.x * blockDim.x)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      // the pending iteration's x += alpha p, from the p_old read here anyway
      if (xp[k]) xg[3 * s + k] = xg[3 * s + k] + al[k] * po[3 * s + k];
      if (act[k]) pn[3 * s + k] = pNew(first[k], wv[3 * s + k], b[k], po[3 * s + k]);
    }
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
    st->xPend[k] = 0;  // applied by this pass
    if (!st->active[k]) continue;
    st->wApA[k] = sum[k];
    if (fabs(sum[k]) / st->normFactor[k] < 1e-300) {  // checkSingularity: stop this component
      st->active[k] = 0;
      continue;
    }
    if (sum[k] <= 0) atomicOr(&st->status, kErrIndefinite);
    st->alpha[k] = st->wArA[k] / sum[k];
    st->pending[k] = 1;
    st->xPend[k] = 1;
    any = 1;
  }
  st->pbuf = pb ^ 1;
  st->pcgContinue = any;
}

// Generic tables: kLocPrecond with NT threads and RPT rows per thread in
// flight; slot tables: kLocPrecondSlots (64 threads) with RPTS.
template <typename T, int NT, int RPT, int RPTS>
void launchPrecondV(const MeshView& mv, const Controls& c, const PcgPtrs<T>& p, DevState* st,
                    double* partials, int grid, cudaStream_t s, int nCases) {
  if (mv.locSlots)
    kLocPrecondSlots<T, RPTS><<<dim3(grid, nCases), 64, localSmemBytes<T>(mv), s>>>(
        mv, c, p, st, partials);
  else
    kLocPrecond<T, NT, RPT><<<dim3(grid, nCases), NT, localSmemBytes<T>(mv), s>>>(
        mv, c, p, st, partials);
}

template <typename T, int NT, int RPT, int RPTS>
cudaError_t prepareV(const MeshView& mv, int* blocksPerSM) {
  const int sm = (int)localSmemBytes<T>(mv);
  if (mv.locSlots) {
    cudaError_t e = setMaxDynamicSmem(kLocPrecondSlots<T, RPTS>);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, kLocPrecondSlots<T, RPTS>, 64,
                                                         sm);
  }
  cudaError_t e = setMaxDynamicSmem(kLocPrecond<T, NT, RPT>);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, kLocPrecond<T, NT, RPT>,
                                                       NT, sm);
}

}  // namespace

// Preconditioner variants (threads per part x rows per thread in flight at
// once).  Generic tables: FP32 {128 x 4, 64 x 4}, FP64 {128 x 2, 64 x 2};
// the second of each pair has all its threads walking and half the threads
// per CTA, so more parts are walked at once per SM where shared memory
// allows.  Slot tables: 64 threads with 4 (FP32) or 2 (FP64) rows in
// flight, on a grid of every resident CTA or on the smallest grid that
// gives every CTA the same number of parts (no last wave of a few CTAs).  perf.part_threads reports the threads of the one in use.
const int kLocVariantsNT[kLocNumNT] = {128, 64};
const int kLocVariantsU[kLocNumU] = {1, 6, 0};

int localPartThreads(const MeshView& mv, int variant) {
  return mv.locSlots ? 64 : kLocVariantsNT[variant];
}

template <typename T>
size_t localSmemBytes(const MeshView& mv) {
  const size_t P = mv.maxRows, EL = mv.maxLocEntries, ML = mv.maxLocMeta;
  if (mv.locSlots)  // coefficients, columns, w with its zero row, level starts
    return sizeof(T) * (EL + 3 * P + 3) + 2 * EL + sizeof(int) * (mv.maxLevels + 1);
  const size_t tables = sizeof(T) * (EL + 6 * P + 3) + 4 * ML + 2 * EL + sizeof(int) * (mv.maxLevels + 1);
  return std::max(tables, (size_t)256 * 6 * sizeof(double));  // final reduction scratch
}

template <typename T>
cudaError_t localPrepare(const MeshView& mv, int* blocksPerSM) {
  cudaError_t e;
  if constexpr (sizeof(T) == 4) {
    e = prepareV<T, 128, 4, 4>(mv, &blocksPerSM[0]);
    return e != cudaSuccess ? e : prepareV<T, 64, 4, 4>(mv, &blocksPerSM[1]);
  } else {
    e = prepareV<T, 128, 2, 2>(mv, &blocksPerSM[0]);
    return e != cudaSuccess ? e : prepareV<T, 64, 2, 2>(mv, &blocksPerSM[1]);
  }
}

template <typename T>
void launchLocalGather(int n, const int* src, const double* rDa, T* lcoef, cudaStream_t s) {
  if (n > 0) kLocGather<T><<<(n + 255) / 256, 256, 0, s>>>(n, src, rDa, lcoef);
}

template <typename T>
void launchLocalPrecond(const MeshView& mv, const Controls& c, const PcgPtrs<T>& p, DevState* st,
                        double* partials, const LocalTuning& t, cudaStream_t s, int nCases) {
  if constexpr (sizeof(T) == 4) {
    if (t.ntIdx == 1) launchPrecondV<T, 64, 4, 4>(mv, c, p, st, partials, t.grid[1], s, nCases);
    else launchPrecondV<T, 128, 4, 4>(mv, c, p, st, partials, t.grid[0], s, nCases);
  } else {
    if (t.ntIdx == 1) launchPrecondV<T, 64, 2, 2>(mv, c, p, st, partials, t.grid[1], s, nCases);
    else launchPrecondV<T, 128, 2, 2>(mv, c, p, st, partials, t.grid[0], s, nCases);
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
