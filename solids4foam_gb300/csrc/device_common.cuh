// Device-side structures and small helpers shared by the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace s4g {

constexpr int kRowBlock = 256;        // threads per block of the row kernels
constexpr int kSweepBlock = 128;      // threads per block of the DIC sweeps
constexpr int kSpinLimit = 1 << 22;   // bounded waits: default polls before giving up

// status bits of DevState::status
constexpr unsigned kErrTimeout = 1u;
constexpr unsigned kErrNaN = 2u;
constexpr unsigned kErrIndefinite = 4u;

// Read-only view of the uploaded mesh (storage order), passed by value.
struct MeshView {
  int nC, nI, nB, nParts, subdomains;
  int emptyDir;        // 2-D: 1, 2, 3 for an x, y, z empty direction; 0: 3-D
  const int* rowptr; const int* col; const int* fidx;      // CSR, fidx ~f for neighbour side
  const int* fown; const int* fnei;                        // internal faces
  const double* fS; const double* fmagS; const double* fw; const double* fdelta;
  const double* C;                                         // [nC][3]
  const double* invDd;                                     // [nC][6]
  const int* browptr; const int* btype;                    // boundary faces by cell
  const double* bS; const double* bmagS; const double* bn; const double* bk;
  const double* bdelta; const double* bls;
  const double* lsv;                                       // [2 nI][3] per CSR entry
  const double* bval; const double* bpress;                // BC data [nB][3], [nB]
  const double* brelax;                                    // [nB] traction relaxationFactor
  const int* partStart; const int* lvlOff; const int* lvlStart;
  const int* upPtr; const int* upIdx; const int* dnPtr; const int* dnIdx;
  // shared-memory staging of the sweeps (see HostPrep)
  const int* haloFPtr; const int* haloFIdx; const int* haloBPtr; const int* haloBIdx;
  const int* slot;
  const int* lowCnt;   // lower entries per row
  int maxRows, maxHalo, maxEntries, maxLevels;
  int rowGrid;         // blocks of the grid-stride row kernels
  int spinLimit;       // polls of a bounded wait before it gives up (kErrTimeout)
  // processor-local DIC tables (see HostPrep)
  const int* locEntStart; const int* locSrc; const uint16_t* locIdx;
  const int* locMetaStart; const uint32_t* locMeta;
  const int4* locDesc;   // [nParts][2] part descriptors
  int maxLocEntries, maxLocMeta;
  int locSlots;          // 1: fixed-slot in-part tables (see HostPrep::locSlots)
  // batched load cases: a launch's blockIdx.y is the case; per-case data
  // lies caseRec doubles (reduction records) or one field size apart
  long caseRec;
  // within a case's records: the group records of the processor-local
  // preconditioner (8 doubles per group of 32 parts) start locGrpOff
  // doubles in, followed by the groups' arrival counters (unsigned)
  long locGrpOff;
  int locGroups;
};

// Batched launches: the case's boundary values (bval [case][nB][3],
// bpress [case][nB]).
__device__ __forceinline__ void caseView(MeshView& mv, int cs) {
  mv.bval += 3 * (size_t)cs * mv.nB;
  mv.bpress += (size_t)cs * mv.nB;
}

// Material and solver constants of a solve.
struct Controls {
  int law;               // 0 linear elastic, 1 neo-Hookean
  int tl;                // 0 linear geometry; total Lagrangian: 1 incremental
                         // (solves DD), 2 total (solves D)
  double mu, K, lambda, impK, rImpK;
  double gamma, gammaS;  // impKf and RhieChow gamma on internal faces
  double loadFactor;
  double tol, relTol;
  int maxIter;
  int nCorr;
  double solTol, altTol, matTol;
  int precond;           // 0 DIC, 1 diagonal
  double fieldRelax;     // relaxField "fixed" factor (1: none)
  int aitken;            // relaxField "Aitken" (fieldRelax is then 1)
  double aitkenA0;       // Aitken: the factor of an increment's first corrector
};

// Mutable solver state in device memory.  Scalars that steer the loops are
// decided on the device; the host only reads them back.
struct DevState {
  // outer corrector loop
  int iCorr;             // index of the corrector in progress
  int outerContinue;
  int converged;
  int nCorrDone;
  int dcur;              // which D buffer is current
  int lastMaxIters;
  long long totalLinIters;
  double xbar[3];        // gAverage of each displacement component
  double relRes, initResMag;
  double maxJ, minJ;     // TL
  int enforceLinear;
  int caseLive;          // the corrector loop of this case is still running
  // PCG (three independent component solves)
  int pcgIter;
  int pcgContinue;
  int active[3];
  int nIter[3];
  double normFactor[3], initRes[3], finalRes[3];
  double wArA[3], wApA[3], alpha[3], beta[3];
  // fused (processor-local DIC) iteration: an update x += alpha p,
  // r -= alpha q is pending per component; which p buffer is the newest
  int pending[3];
  int pbuf;
  // x += alpha p of the pending iteration, not yet applied to x: the next
  // SpMV pass applies it (it reads that p anyway), or kApplyX after the loop
  int xPend[3];
  unsigned locTicket;    // next part of the processor-local preconditioner
  // error bits
  unsigned status;
  // last-block counters (one per kernel kind)
  unsigned counter[16];
  // sweep control
  unsigned ticket[2], ctasDone[2], partsDone[2], epoch[2];
  // device-resident loop (conditional graph nodes): iterations of the PCG
  // loop of the corrector in progress and correctors of the graph launch
  unsigned loopPcg, loopOuter;
};

// The dynamic shared-memory limit of a kernel is a process-wide attribute:
// it is set to the device's opt-in maximum (not to one mesh's need), so
// that meshes of different sizes, uploaded in any order or from several
// threads, can all launch.  Occupancy follows the size each launch asks for.
template <typename K>
inline cudaError_t setMaxDynamicSmem(K kernel) {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              optin - (int)fa.sharedSizeBytes);
}

// ---- memory-order helpers --------------------------------------------------
__device__ __forceinline__ unsigned ldAcquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ldRelaxed(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void fenceAcqRel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ void stRelease(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ---- small vector/tensor algebra (OpenFOAM conventions) -------------------
struct V3 { double x, y, z; };
struct T9 { double xx, xy, xz, yx, yy, yz, zx, zy, zz; };
struct S6 { double xx, xy, xz, yy, yz, zz; };

__device__ __forceinline__ V3 ldV(const double* a, long i) { return {a[3 * i], a[3 * i + 1], a[3 * i + 2]}; }
// vectors of the PCG value type (double or float) as FP64
template <typename T>
__device__ __forceinline__ V3 ldVT(const T* a, long i) {
  return {(double)a[3 * i], (double)a[3 * i + 1], (double)a[3 * i + 2]};
}
template <typename T>
__device__ __forceinline__ void stVT(T* a, long i, V3 v) {
  a[3 * i] = (T)v.x; a[3 * i + 1] = (T)v.y; a[3 * i + 2] = (T)v.z;
}
__device__ __forceinline__ void stV(double* a, long i, V3 v) { a[3 * i] = v.x; a[3 * i + 1] = v.y; a[3 * i + 2] = v.z; }
__device__ __forceinline__ T9 ldT(const double* a, long i) {
  const double* p = a + 9 * i;
  return {p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8]};
}
__device__ __forceinline__ void stT(double* a, long i, const T9& t) {
  double* p = a + 9 * i;
  p[0] = t.xx; p[1] = t.xy; p[2] = t.xz; p[3] = t.yx; p[4] = t.yy; p[5] = t.yz;
  p[6] = t.zx; p[7] = t.zy; p[8] = t.zz;
}
__device__ __forceinline__ S6 ldS(const double* a, long i) {
  const double* p = a + 6 * i;
  return {p[0], p[1], p[2], p[3], p[4], p[5]};
}
__device__ __forceinline__ void stS(double* a, long i, const S6& s) {
  double* p = a + 6 * i;
  p[0] = s.xx; p[1] = s.xy; p[2] = s.xz; p[3] = s.yy; p[4] = s.yz; p[5] = s.zz;
}
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double magSqr(V3 a) { return dot(a, a); }
__device__ __forceinline__ double mag(V3 a) { return sqrt(dot(a, a)); }
__device__ __forceinline__ T9 zeroT() { return {0, 0, 0, 0, 0, 0, 0, 0, 0}; }
__device__ __forceinline__ T9 operator+(const T9& a, const T9& b) {
  return {a.xx + b.xx, a.xy + b.xy, a.xz + b.xz, a.yx + b.yx, a.yy + b.yy,
          a.yz + b.yz, a.zx + b.zx, a.zy + b.zy, a.zz + b.zz};
}
__device__ __forceinline__ T9 operator-(const T9& a, const T9& b) {
  return {a.xx - b.xx, a.xy - b.xy, a.xz - b.xz, a.yx - b.yx, a.yy - b.yy,
          a.yz - b.yz, a.zx - b.zx, a.zy - b.zy, a.zz - b.zz};
}
__device__ __forceinline__ T9 operator*(double s, const T9& a) {
  return {s * a.xx, s * a.xy, s * a.xz, s * a.yx, s * a.yy, s * a.yz,
          s * a.zx, s * a.zy, s * a.zz};
}
__device__ __forceinline__ T9 outer(V3 a, V3 b) {
  return {a.x * b.x, a.x * b.y, a.x * b.z, a.y * b.x, a.y * b.y,
          a.y * b.z, a.z * b.x, a.z * b.y, a.z * b.z};
}
__device__ __forceinline__ V3 dotVT(V3 v, const T9& t) {
  return {v.x * t.xx + v.y * t.yx + v.z * t.zx,
          v.x * t.xy + v.y * t.yy + v.z * t.zy,
          v.x * t.xz + v.y * t.yz + v.z * t.zz};
}
__device__ __forceinline__ V3 dotVS(V3 v, const S6& s) {
  return {v.x * s.xx + v.y * s.xy + v.z * s.xz,
          v.x * s.xy + v.y * s.yy + v.z * s.yz,
          v.x * s.xz + v.y * s.yz + v.z * s.zz};
}
__device__ __forceinline__ T9 transposeT(const T9& t) {
  return {t.xx, t.yx, t.zx, t.xy, t.yy, t.zy, t.xz, t.yz, t.zz};
}
__device__ __forceinline__ T9 dotTT(const T9& a, const T9& b) {
  return {a.xx * b.xx + a.xy * b.yx + a.xz * b.zx, a.xx * b.xy + a.xy * b.yy + a.xz * b.zy,
          a.xx * b.xz + a.xy * b.yz + a.xz * b.zz, a.yx * b.xx + a.yy * b.yx + a.yz * b.zx,
          a.yx * b.xy + a.yy * b.yy + a.yz * b.zy, a.yx * b.xz + a.yy * b.yz + a.yz * b.zz,
          a.zx * b.xx + a.zy * b.yx + a.zz * b.zx, a.zx * b.xy + a.zy * b.yy + a.zz * b.zy,
          a.zx * b.xz + a.zy * b.yz + a.zz * b.zz};
}
__device__ __forceinline__ double detT(const T9& t) {
  return t.xx * (t.yy * t.zz - t.yz * t.zy) - t.xy * (t.yx * t.zz - t.yz * t.zx) +
         t.xz * (t.yx * t.zy - t.yy * t.zx);
}
__device__ __forceinline__ T9 invT(const T9& t) {
  double d = detT(t);
  T9 c = {t.yy * t.zz - t.yz * t.zy, t.xz * t.zy - t.xy * t.zz, t.xy * t.yz - t.xz * t.yy,
          t.yz * t.zx - t.yx * t.zz, t.xx * t.zz - t.xz * t.zx, t.xz * t.yx - t.xx * t.yz,
          t.yx * t.zy - t.yy * t.zx, t.xy * t.zx - t.xx * t.zy, t.xx * t.yy - t.xy * t.yx};
  return (1.0 / d) * c;
}
__device__ __forceinline__ S6 symmT(const T9& t) {
  return {t.xx, 0.5 * (t.xy + t.yx), 0.5 * (t.xz + t.zx), t.yy, 0.5 * (t.yz + t.zy), t.zz};
}
__device__ __forceinline__ T9 fromS(const S6& s) {
  return {s.xx, s.xy, s.xz, s.xy, s.yy, s.yz, s.xz, s.yz, s.zz};
}
__device__ __forceinline__ double trS(const S6& s) { return s.xx + s.yy + s.zz; }
__device__ __forceinline__ double trT(const T9& t) { return t.xx + t.yy + t.zz; }
__device__ __forceinline__ S6 devS(const S6& s) {
  double m = trS(s) / 3.0;
  return {s.xx - m, s.xy, s.xz, s.yy - m, s.yz, s.zz - m};
}
__device__ __forceinline__ S6 operator+(const S6& a, const S6& b) {
  return {a.xx + b.xx, a.xy + b.xy, a.xz + b.xz, a.yy + b.yy, a.yz + b.yz, a.zz + b.zz};
}
__device__ __forceinline__ S6 operator*(double s, const S6& a) {
  return {s * a.xx, s * a.xy, s * a.xz, s * a.yy, s * a.yz, s * a.zz};
}
__device__ __forceinline__ S6 addI(const S6& a, double s) {
  return {a.xx + s, a.xy, a.xz, a.yy + s, a.yz, a.zz + s};
}
__device__ __forceinline__ S6 invS(const S6& s) {
  double d = s.xx * (s.yy * s.zz - s.yz * s.yz) - s.xy * (s.xy * s.zz - s.yz * s.xz) +
             s.xz * (s.xy * s.yz - s.yy * s.xz);
  S6 c = {s.yy * s.zz - s.yz * s.yz, s.xz * s.yz - s.xy * s.zz, s.xy * s.yz - s.xz * s.yy,
          s.xx * s.zz - s.xz * s.xz, s.xy * s.xz - s.xx * s.yz, s.xx * s.yy - s.xy * s.xy};
  return (1.0 / d) * c;
}

// Deterministic block sum of N values (fixed shuffle tree, fixed warp order).
// Result valid in thread 0.
template <int N>
__device__ __forceinline__ void blockSum(double (&v)[N], double* smem /* [32*N] */) {
#pragma unroll
  for (int k = 0; k < N; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; ++k) smem[wid * N + k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      double s = 0;
      for (int w = 0; w < nw; ++w) s += smem[w * N + k];
      v[k] = s;
    }
  }
  __syncthreads();
}

template <int N>
__device__ __forceinline__ void blockMax(double (&v)[N], double* smem) {
#pragma unroll
  for (int k = 0; k < N; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] = fmax(v[k], __shfl_down_sync(0xffffffffu, v[k], o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; ++k) smem[wid * N + k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      double s = smem[k];
      for (int w = 1; w < nw; ++w) s = fmax(s, smem[w * N + k]);
      v[k] = s;
    }
  }
  __syncthreads();
}

// Fixed-order reduction of `count` partial records (stride doubles apart,
// N values each) by the whole block: thread t sums records t, t+B, ... in
// order, then a fixed shuffle/warp tree.  Result valid in thread 0.
template <int N>
__device__ __forceinline__ void reducePartials(const double* partials, int stride, int count,
                                               double (&out)[N], double* smem) {
#pragma unroll
  for (int k = 0; k < N; ++k) out[k] = 0;
  for (int q = threadIdx.x; q < count; q += blockDim.x)
#pragma unroll
    for (int k = 0; k < N; ++k) out[k] += __ldcg(partials + (size_t)stride * q + k);
  blockSum<N>(out, smem);
}

// Sum of N values over the first 64 threads (two warps) by a fixed tree,
// whatever the block size.  Result valid in thread 0; needs blockDim >= 64.
template <int N>
__device__ __forceinline__ void sum64(double (&v)[N], double* smem /* [2*N] */) {
  if (threadIdx.x < 64) {
#pragma unroll
    for (int k = 0; k < N; ++k)
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if (threadIdx.x == 32)
#pragma unroll
      for (int k = 0; k < N; ++k) smem[k] = v[k];
  }
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] += smem[k];
  __syncthreads();
}

// reducePartials with 64 fixed virtual lanes: the summation order depends on
// `count` only, not on the block size of the kernel that reduces.
template <int N>
__device__ __forceinline__ void reducePartials64(const double* partials, int stride, int count,
                                                 double (&out)[N], double* smem) {
#pragma unroll
  for (int k = 0; k < N; ++k) out[k] = 0;
  if (threadIdx.x < 64)
    for (int q = threadIdx.x; q < count; q += 64)
#pragma unroll
      for (int k = 0; k < N; ++k) out[k] += __ldcg(partials + (size_t)stride * q + k);
  sum64<N>(out, smem);
}

// Fixed-order sum of `count` records of N values (`stride` doubles apart)
// over 256 virtual lanes: lane v sums records v, v+256, ... in order (four
// loads in flight), then lanes v, v+32, ..., v+224 are summed in order and
// the 32 results by a fixed shuffle tree.  The order depends on `count`
// only, and any block size works.  scratch: 256*N doubles of shared memory.
// Result valid in thread 0.
template <int N>
__device__ __forceinline__ void reduceRecords(const double* rec, int stride, int count,
                                              double (&out)[N], double* scratch) {
  for (int v = threadIdx.x; v < 256; v += blockDim.x) {
    double a[N];
#pragma unroll
    for (int k = 0; k < N; ++k) a[k] = 0;
    int q = v;
    for (; q + 3 * 256 < count; q += 4 * 256) {
      double t[4][N];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int k = 0; k < N; ++k) t[u][k] = __ldcg(rec + (size_t)stride * (q + 256 * u) + k);
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int k = 0; k < N; ++k) a[k] += t[u][k];
    }
    for (; q < count; q += 256)
#pragma unroll
      for (int k = 0; k < N; ++k) a[k] += __ldcg(rec + (size_t)stride * q + k);
#pragma unroll
    for (int k = 0; k < N; ++k) scratch[v * N + k] = a[k];
  }
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      double b = 0;
      for (int j = 0; j < 8; ++j) b += scratch[(threadIdx.x + 32 * j) * N + k];
      for (int o = 16; o > 0; o >>= 1) b += __shfl_down_sync(0xffffffffu, b, o);
      out[k] = b;
    }
  }
  __syncthreads();
}

template <int N>
__device__ __forceinline__ void reducePartialsMax(const double* partials, int stride, int count,
                                                  double (&out)[N], double* smem) {
#pragma unroll
  for (int k = 0; k < N; ++k) out[k] = -1e300;
  for (int q = threadIdx.x; q < count; q += blockDim.x)
#pragma unroll
    for (int k = 0; k < N; ++k) out[k] = fmax(out[k], __ldcg(partials + (size_t)stride * q + k));
  blockMax<N>(out, smem);
}

// Thread 0 has written the block's partial record; it publishes it with one
// gpu-scope fence and takes a ticket.  True in all threads of the block that
// arrived last (which then reads every block's record).
__device__ __forceinline__ bool lastBlockDone(unsigned* counter, unsigned total) {
  __shared__ int amLast;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    amLast = (atomicAdd(counter, 1u) == total - 1);
  }
  __syncthreads();
  if (amLast) __threadfence();
  return amLast != 0;
}

// Grid of the row kernels: a few resident blocks per SM, rows in a
// grid-stride loop, so the per-launch finalize reads few partial records.
constexpr int kRowBlocksPerSM = 4;

}  // namespace s4g
