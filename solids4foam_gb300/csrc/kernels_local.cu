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
// Part tables (HostPrep step 9): in-part entries per row, lower entries in
// CSR order then upper entries in reverse CSR order, coefficient rD_row*a_e
// and the column's row index inside the part (16 bits); per-row metadata
// (entry offset, lower and upper counts).  Both are padded per part so that
// they are staged with 16-byte cp.async copies while the CTA streams the
// x/r update.

#include "kernels.cuh"
#include "pcg_common.cuh"

namespace s4g {
namespace {

constexpr int kLocBlock = 64;  // threads per part (levels of 8x8x8 parts hold <= 48 rows)

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
  s.w = (T*)(s.idx + EL);                     // 3P
  s.r = s.w + 3 * P;                          // 3P
  s.lv = (int*)(s.r + 3 * P);                 // maxLevels + 1
  return s;
}

template <typename T>
__global__ void kLocGather(int n, const int* src, const double* rDa, T* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = src[i] >= 0 ? (T)rDa[src[i]] : T(0);
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT)
kLocPrecond(MeshView mv, Controls c, PcgPtrs<T> p, DevState* st, double* partials) {
  if (!st->pcgContinue) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  const LocSmem<T> sm = locSmem<T>(mv, smraw);
  __shared__ double red[32 * 6];
  const T* pp = st->pbuf ? p.p2 : p.p;  // p of the pending iteration
  bool pend[3];
  T al[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) { pend[k] = st->pending[k] != 0; al[k] = (T)st->alpha[k]; }
  const bool anyPend = pend[0] || pend[1] || pend[2];
  Acc<T> wr[3], ar[3];
  for (int part = blockIdx.x; part < mv.nParts; part += gridDim.x) {
    const int pLo = mv.partStart[part], nR = mv.partStart[part + 1] - pLo;
    const int eLo = mv.locEntStart[part], nE = mv.locEntStart[part + 1] - eLo;
    const int mLo = mv.locMetaStart[part], nM = mv.locMetaStart[part + 1] - mLo;
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
    const int l0 = mv.lvlOff[part], nL = mv.lvlOff[part + 1] - l0;
    for (int k = threadIdx.x; k <= nL; k += NT) sm.lv[k] = mv.lvlStart[l0 + k] - pLo;
    // pending update and residual sums; w starts as rD r
    for (int i = threadIdx.x; i < nR; i += NT) {
      const size_t g = 3 * (size_t)(pLo + i);
      const T rd = p.rD[pLo + i];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        T rv = p.r[g + k];
        if (pend[k]) {
          p.x[g + k] += al[k] * pp[g + k];
          rv -= al[k] * p.q[g + k];
          p.r[g + k] = rv;
        }
        ar[k].add(fabs(rv));
        sm.r[3 * i + k] = rv;
        sm.w[3 * i + k] = rd * rv;
      }
    }
    cpAsyncWaitAll();
    __syncthreads();
    // forward substitution: w_u -= sum_{l<u in part} (rD_u a_ul) w_l
    for (int l = 0; l < nL; ++l) {
      for (int i = sm.lv[l] + threadIdx.x; i < sm.lv[l + 1]; i += NT) {
        const uint32_t m = sm.m[i];
        const int j0 = m & 0xffff, j1 = j0 + ((m >> 16) & 0xff);
        T v0 = sm.w[3 * i], v1 = sm.w[3 * i + 1], v2 = sm.w[3 * i + 2];
        for (int j = j0; j < j1; ++j) {
          const int q = sm.idx[j];
          const T a = sm.c[j];
          v0 -= a * sm.w[3 * q]; v1 -= a * sm.w[3 * q + 1]; v2 -= a * sm.w[3 * q + 2];
        }
        sm.w[3 * i] = v0; sm.w[3 * i + 1] = v1; sm.w[3 * i + 2] = v2;
      }
      __syncthreads();
    }
    // backward substitution: w_l -= sum_{u>l in part} (rD_l a_lu) w_u
    for (int l = nL - 1; l >= 0; --l) {
      for (int i = sm.lv[l] + threadIdx.x; i < sm.lv[l + 1]; i += NT) {
        const uint32_t m = sm.m[i];
        const int j0 = (m & 0xffff) + ((m >> 16) & 0xff), j1 = j0 + (m >> 24);
        T v0 = sm.w[3 * i], v1 = sm.w[3 * i + 1], v2 = sm.w[3 * i + 2];
        for (int j = j0; j < j1; ++j) {
          const int q = sm.idx[j];
          const T a = sm.c[j];
          v0 -= a * sm.w[3 * q]; v1 -= a * sm.w[3 * q + 1]; v2 -= a * sm.w[3 * q + 2];
        }
        sm.w[3 * i] = v0; sm.w[3 * i + 1] = v1; sm.w[3 * i + 2] = v2;
        wr[0].add(v0 * sm.r[3 * i]); wr[1].add(v1 * sm.r[3 * i + 1]); wr[2].add(v2 * sm.r[3 * i + 2]);
      }
      __syncthreads();
    }
    T* wg = p.w + 3 * (size_t)pLo;
    for (int k = threadIdx.x; k < 3 * nR; k += NT) wg[k] = sm.w[k];
    __syncthreads();  // the next part reuses the shared memory
  }
  double acc[6] = {wr[0].value(), wr[1].value(), wr[2].value(),
                   ar[0].value(), ar[1].value(), ar[2].value()};
  blockSum<6>(acc, red);
  if (threadIdx.x == 0) {
    double* q = partials + 8 * (size_t)blockIdx.x;
    for (int k = 0; k < 6; ++k) q[k] = acc[k];
  }
  if (!lastBlockDone(&st->counter[5], gridDim.x)) return;
  double S[6];
  reducePartials<6>(partials, 8, gridDim.x, S, red);
  if (threadIdx.x != 0) return;
  st->counter[5] = 0;
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

// p_new = w (first iteration) or w + beta p_old, the same expression for a
// row and for its neighbours
template <typename T>
__device__ __forceinline__ T pNew(bool first, T w, T b, T po) { return first ? w : w + b * po; }

template <typename T>
__global__ void __launch_bounds__(kRowBlock)
kLocSpmv(MeshView mv, PcgPtrs<T> p, DevState* st, double* partials) {
  if (!st->pcgContinue) return;
  __shared__ double red[32 * 3];
  const int pb = st->pbuf;
  const T* po = pb ? p.p2 : p.p;
  T* pn = pb ? p.p : p.p2;
  bool act[3], first[3];
  T b[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    act[k] = st->active[k] != 0; first[k] = st->nIter[k] == 0; b[k] = (T)st->beta[k];
  }
  Acc<T> a0, a1, a2;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < mv.nC; s += gridDim.x * blockDim.x) {
    const T dg = p.diag[s];
    const T v0 = pNew(first[0], p.w[3 * s], b[0], po[3 * s]);
    const T v1 = pNew(first[1], p.w[3 * s + 1], b[1], po[3 * s + 1]);
    const T v2 = pNew(first[2], p.w[3 * s + 2], b[2], po[3 * s + 2]);
    T y0 = dg * v0, y1 = dg * v1, y2 = dg * v2;
    const int e1 = mv.rowptr[s + 1];
    for (int e = mv.rowptr[s]; e < e1; ++e) {
      const int cl = mv.col[e];
      const T a = p.val[e];
      y0 += a * pNew(first[0], p.w[3 * cl], b[0], po[3 * cl]);
      y1 += a * pNew(first[1], p.w[3 * cl + 1], b[1], po[3 * cl + 1]);
      y2 += a * pNew(first[2], p.w[3 * cl + 2], b[2], po[3 * cl + 2]);
    }
    if (act[0]) { pn[3 * s] = v0; p.q[3 * s] = y0; }
    if (act[1]) { pn[3 * s + 1] = v1; p.q[3 * s + 1] = y1; }
    if (act[2]) { pn[3 * s + 2] = v2; p.q[3 * s + 2] = y2; }
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

}  // namespace

template <typename T>
size_t localSmemBytes(const MeshView& mv) {
  const size_t P = mv.maxRows, EL = mv.maxLocEntries, ML = mv.maxLocMeta;
  return sizeof(T) * (EL + 6 * P) + 4 * ML + 2 * EL + sizeof(int) * (mv.maxLevels + 1);
}

template <typename T>
cudaError_t localPrepare(const MeshView& mv, int* blocksPerSM) {
  const int sm = (int)localSmemBytes<T>(mv);
  cudaError_t e = cudaFuncSetAttribute(kLocPrecond<T, kLocBlock>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, kLocPrecond<T, kLocBlock>,
                                                       kLocBlock, sm);
}

template <typename T>
void launchLocalGather(int n, const int* src, const double* rDa, T* lcoef, cudaStream_t s) {
  if (n > 0) kLocGather<T><<<(n + 255) / 256, 256, 0, s>>>(n, src, rDa, lcoef);
}

template <typename T>
void launchLocalIteration(const MeshView& mv, const Controls& c, const PcgPtrs<T>& p,
                          DevState* st, double* partials, int grid, cudaStream_t s,
                          long long* launches, LaunchTimer* tm) {
  {
    TimeScope ts(tm, S4G_K_LOC_PRECOND, s);
    kLocPrecond<T, kLocBlock><<<grid, kLocBlock, localSmemBytes<T>(mv), s>>>(mv, c, p, st, partials);
  }
  {
    TimeScope ts(tm, S4G_K_LOC_SPMV, s);
    kLocSpmv<T><<<mv.rowGrid, kRowBlock, 0, s>>>(mv, p, st, partials);
  }
  *launches += 2;
}

#define S4G_INSTANTIATE(T)                                                                      \
  template size_t localSmemBytes<T>(const MeshView&);                                           \
  template cudaError_t localPrepare<T>(const MeshView&, int*);                                  \
  template void launchLocalGather<T>(int, const int*, const double*, T*, cudaStream_t);          \
  template void launchLocalIteration<T>(const MeshView&, const Controls&, const PcgPtrs<T>&,    \
                                        DevState*, double*, int, cudaStream_t, long long*,      \
                                        LaunchTimer*);
S4G_INSTANTIATE(double)
S4G_INSTANTIATE(float)
#undef S4G_INSTANTIATE

}  // namespace s4g
