// y = A x together with the column products x.Ax, without allocating.
//
// Some callers cannot allocate memory at the moment they need an operator
// product: a host loop that has handed every free byte of the device to
// other work (a server that admits solves by their memory footprint), a
// real-time or latency-bound caller that must not enter the CUDA allocator
// (which can synchronise the device and take locks), or code running while
// an allocation would be unsafe.  This entry point serves them: it works in
// the mesh's existing work vectors and in one fixed scratch block that lives
// in static device memory, so it calls no cudaMalloc, cudaFree or other
// allocating routine, on the device or the host.
//
// Scratch.  gScratch holds one partial record per block (at most
// kNaMaxBlocks blocks of kNaBlock rows: meshes of up to 262,144 cells; a
// larger mesh is rejected with S4G_BAD_ARG), the result and a block counter.
// Only the counter must be zero when a call starts; static device memory
// starts at zero, the last block of every call sets it back to zero, and the
// host also zeroes it with cudaMemsetAsync before each launch, so a call
// that failed half-way cannot poison the next one.  The partial records need
// no initial value (each block writes its own before the last one reads).
//
// One scratch block per device serves every mesh and context of the process:
// calls that overlap in time on the same device -- from two host threads, or
// on two streams without an ordering between them -- race on it and give
// wrong results.  Callers must order such calls.
//
// Set-up.  The first call on a device looks up the scratch's device address
// with cudaGetSymbolAddress, with that device current, and keeps it; later
// calls reuse it.  Make that first call before any stream capture begins.

#include <mutex>
#include <string>

#include "kernels.cuh"

namespace s4g {
namespace {

constexpr int kNaBlock = 256;
constexpr int kNaMaxBlocks = 1024;  // 262,144 cells
constexpr int kNaMaxDevices = 64;

struct NoAllocScratch {
  double partial[kNaMaxBlocks][4];
  double result[4];
  unsigned counter;
};

// 32.8 KB of static device memory
static __device__ __align__(256) NoAllocScratch gScratch;

std::mutex gSetupMutex;
NoAllocScratch* gScratchPtr[kNaMaxDevices] = {};

// caller order [n][k] -> storage order [n][3] (unused columns zero)
__global__ void kToStorage(int n, int k, const int* c2s, const double* x, double* xs) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const long s = c2s[c];
  for (int j = 0; j < 3; ++j) xs[3 * s + j] = j < k ? x[(long)k * c + j] : 0.0;
}

// storage order [n][3] -> caller order [n][k]
__global__ void kFromStorage(int n, int k, const int* c2s, const double* ys, double* y) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const long s = c2s[c];
  for (int j = 0; j < k; ++j) y[(long)k * c + j] = ys[3 * s + j];
}

// One row per thread: y = A x (the amul of the PCG), and per block the
// x.y sums of the three columns; the last block reduces the records in a
// fixed order into the result and resets the counter.
__global__ void __launch_bounds__(kNaBlock)
kAmulDot(MeshView mv, const double* val, const double* diag, const double* x, double* y,
         NoAllocScratch* sc) {
  __shared__ double red[32 * 3];
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[3] = {0, 0, 0};
  if (s < mv.nC) {
    double a[3];
    for (int j = 0; j < 3; ++j) a[j] = diag[s] * x[3 * s + j];
    for (int e = mv.rowptr[s]; e < mv.rowptr[s + 1]; ++e) {
      const int cl = mv.col[e];
      for (int j = 0; j < 3; ++j) a[j] += val[e] * x[3 * cl + j];
    }
    for (int j = 0; j < 3; ++j) {
      y[3 * s + j] = a[j];
      acc[j] = x[3 * s + j] * a[j];
    }
  }
  blockSum<3>(acc, red);
  if (threadIdx.x == 0)
    for (int j = 0; j < 3; ++j) sc->partial[blockIdx.x][j] = acc[j];
  if (!lastBlockDone(&sc->counter, gridDim.x)) return;
  double sum[3];
  reducePartials<3>(&sc->partial[0][0], 4, gridDim.x, sum, red);
  if (threadIdx.x != 0) return;
  for (int j = 0; j < 3; ++j) sc->result[j] = sum[j];
  sc->counter = 0;
}

}  // namespace

s4g_status opAmulDotNoAlloc(const MeshView& mv, const int* c2s, const double* val,
                            const double* diag, double* work0, double* work1, int device,
                            cudaStream_t s, int k, const double* x, double* y, double* xAx,
                            std::string& err) {
  if (k < 1 || k > 3 || !x || !y || !xAx) {
    err = "k must be 1..3 and x, y, xAx non-null";
    return S4G_BAD_ARG;
  }
  if (mv.nC > kNaMaxBlocks * kNaBlock) {
    err = "mesh has " + std::to_string(mv.nC) + " cells; s4g_op_amul_dot_noalloc serves at most " +
          std::to_string(kNaMaxBlocks * kNaBlock) + " (its static scratch is fixed)";
    return S4G_BAD_ARG;
  }
  if (device < 0 || device >= kNaMaxDevices) {
    err = "device index out of range for the no-allocation scratch";
    return S4G_BAD_ARG;
  }
  NoAllocScratch* sc = nullptr;
  {
    std::lock_guard<std::mutex> lock(gSetupMutex);
    if (!gScratchPtr[device]) {
      cudaError_t e = cudaGetSymbolAddress((void**)&gScratchPtr[device], gScratch);
      if (e != cudaSuccess) {
        gScratchPtr[device] = nullptr;
        err = std::string("cudaGetSymbolAddress of the scratch: ") + cudaGetErrorString(e);
        return S4G_CUDA_ERROR;
      }
    }
    sc = gScratchPtr[device];
  }
  const int n = mv.nC;
  const int g = (n + kNaBlock - 1) / kNaBlock;
  auto fail = [&](cudaError_t e, const char* what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return S4G_CUDA_ERROR;
  };
  cudaError_t e = cudaMemcpyAsync(work1, x, sizeof(double) * (size_t)k * n, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail(e, "copy of x");
  kToStorage<<<g, kNaBlock, 0, s>>>(n, k, c2s, work1, work0);
  e = cudaMemsetAsync(&sc->counter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return fail(e, "reset of the scratch counter");
  kAmulDot<<<g, kNaBlock, 0, s>>>(mv, val, diag, work0, work1, sc);
  kFromStorage<<<g, kNaBlock, 0, s>>>(n, k, c2s, work1, work0);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(e, "launch");
  e = cudaMemcpyAsync(y, work0, sizeof(double) * (size_t)k * n, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return fail(e, "copy of y");
  e = cudaMemcpyAsync(xAx, sc->result, sizeof(double) * k, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return fail(e, "copy of x.Ax");
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(e, "synchronise");
  return S4G_OK;
}

}  // namespace s4g
