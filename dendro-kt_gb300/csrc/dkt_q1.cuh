// Value arithmetic shared by the Q1 leaf kernels (dkt_q1fx.cu, dkt_tile.cu).
#pragma once
#include <cstdint>

namespace dkt {

// Value arithmetic of the Q1 leaf kernel.  FixedArith: exact int64 fixed
// point (halving = arithmetic shift, mode scaling = the high word of a
// 128-bit product, integer atomics).  F32Arith: binary32 (halving and mode
// scaling rounded, float atomics), the inner operator of the mixed-precision
// solver.
struct FixedArith {
  using T = long long;
  __device__ static __forceinline__ T half_sum(T a, T b) { return (a + b) >> 1; }
  __device__ static __forceinline__ T half(T a) { return a >> 1; }
  // floor(v * m / 2^64): every per-mode factor is stored as m = round(f * 2^64)
  __device__ static __forceinline__ T scale(T v, const void *f, int idx)
  {
    return __mul64hi(v, __ldg(static_cast<const long long *>(f) + idx));
  }
  // factor staged in shared memory
  struct Factor { long long m; };
  __device__ static __forceinline__ Factor load_factor(const void *f, int idx)
  {
    return Factor{static_cast<const long long *>(f)[idx]};
  }
  __device__ static __forceinline__ T apply(T v, const Factor &q) { return __mul64hi(v, q.m); }
  __device__ static __forceinline__ void add(T *y, T v) { atomicAdd((unsigned long long *) y, (unsigned long long) v); }
};
struct F32Arith {
  using T = float;
  __device__ static __forceinline__ T half_sum(T a, T b) { return (a + b) * 0.5f; }
  __device__ static __forceinline__ T half(T a) { return a * 0.5f; }
  __device__ static __forceinline__ T scale(T v, const void *f, int idx)
  {
    return v * __ldg(static_cast<const float *>(f) + idx);
  }
  struct Factor { float m; };
  __device__ static __forceinline__ Factor load_factor(const void *f, int idx)
  {
    return Factor{static_cast<const float *>(f)[idx]};
  }
  __device__ static __forceinline__ T apply(T v, const Factor &q) { return v * q.m; }
  __device__ static __forceinline__ void add(T *y, T v) { atomicAdd(y, v); }
};

}  // namespace dkt
