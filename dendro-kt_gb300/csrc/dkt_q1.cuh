// Value arithmetic shared by the Q1 leaf kernels (dkt_q1fx.cu, dkt_tile.cu).
#pragma once
#include <cstdint>

namespace dkt {

__device__ __forceinline__ long long mulshift(long long v, long long m, int e)
{
  // floor(v * m / 2^e) with a 128-bit intermediate, 1 <= e <= 126
  const long long hi = __mul64hi(v, m);
  const unsigned long long lo = (unsigned long long) v * (unsigned long long) m;
  if (e >= 64) return hi >> (e - 64);
  return (long long) ((lo >> e) | ((unsigned long long) hi << (64 - e)));
}

// Value arithmetic of the Q1 leaf kernel.  FixedArith: exact int64 fixed
// point (halving = arithmetic shift, mode scaling = 128-bit multiply-shift,
// integer atomics).  F32Arith: binary32 (halving and mode scaling rounded,
// float atomics), the inner operator of the mixed-precision solver.
// floor(v * m / 2^e) for 64 <= e <= 126 (every per-mode factor has e >= 64):
// the high word of the 128-bit product, shifted.
__device__ __forceinline__ long long mulshift_hi(long long v, long long m, int e)
{
  return __mul64hi(v, m) >> (e - 64);
}

struct FixedArith {
  using T = long long;
  __device__ static __forceinline__ T half_sum(T a, T b) { return (a + b) >> 1; }
  __device__ static __forceinline__ T half(T a) { return a >> 1; }
  __device__ static __forceinline__ T scale(T v, const void *f, const int *fe, int idx)
  {
    return mulshift(v, __ldg(static_cast<const long long *>(f) + idx), __ldg(fe + idx));
  }
  // factor staged in shared memory: mantissa and exponent
  struct Factor { long long m; int e; };
  __device__ static __forceinline__ Factor load_factor(const void *f, const int *fe, int idx)
  {
    return Factor{static_cast<const long long *>(f)[idx], fe[idx]};
  }
  __device__ static __forceinline__ T apply(T v, const Factor &q) { return mulshift_hi(v, q.m, q.e); }
  __device__ static __forceinline__ void add(T *y, T v) { atomicAdd((unsigned long long *) y, (unsigned long long) v); }
};
struct F32Arith {
  using T = float;
  __device__ static __forceinline__ T half_sum(T a, T b) { return (a + b) * 0.5f; }
  __device__ static __forceinline__ T half(T a) { return a * 0.5f; }
  __device__ static __forceinline__ T scale(T v, const void *f, const int *, int idx)
  {
    return v * __ldg(static_cast<const float *>(f) + idx);
  }
  struct Factor { float m; };
  __device__ static __forceinline__ Factor load_factor(const void *f, const int *, int idx)
  {
    return Factor{static_cast<const float *>(f)[idx]};
  }
  __device__ static __forceinline__ T apply(T v, const Factor &q) { return v * q.m; }
  __device__ static __forceinline__ void add(T *y, T v) { atomicAdd(y, v); }
};

}  // namespace dkt
