// Helpers shared by the PCG kernels.
#pragma once

#include "device_common.cuh"

namespace s4g {

// Asynchronous global->shared copies (LDGSTS): a part's static data is put in
// flight at once and waited for with one hardware wait.
template <int BYTES>
__device__ __forceinline__ void cpAsync(void* sm, const void* gm) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(sm);
  if (BYTES == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gm) : "memory");
  else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gm) : "memory");
}
template <typename T>
__device__ __forceinline__ void cpAsyncT(T* sm, const T* gm) { cpAsync<sizeof(T)>(sm, gm); }
__device__ __forceinline__ void cpAsyncWaitAll() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_all;" ::: "memory");
}

// Sum of T values: plain for double; Neumaier-compensated for float.
template <typename T> struct Acc;
template <> struct Acc<double> {
  double s = 0;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double value() const { return s; }
};
template <> struct Acc<float> {
  float s = 0, c = 0;
  __device__ __forceinline__ void add(float x) {
    const float t = s + x;
    c += (fabsf(s) >= fabsf(x)) ? (s - t) + x : (x - t) + s;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// 16-byte asynchronous global->shared copy that bypasses L1 (data read once).
__device__ __forceinline__ void cpAsync16(void* sm, const void* gm) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(sm);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gm) : "memory");
}

}  // namespace s4g
