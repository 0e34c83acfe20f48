// Device primitives for the integer side of the path: a stable LSD radix
// sort over 64- or 128-bit keys, exclusive scans, stream compaction and
// binary search.  All hand-written for sm_103a; no library sort or scan.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <atomic>
#include <map>
#include <mutex>
#include <utility>
#include <vector>
#include <stdexcept>
#include <string>

namespace dkt {

#define DKT_CUDA(call)                                                                      \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " at " \
                               + __FILE__ + ":" + std::to_string(__LINE__));                \
  } while (0)

inline void check_launch(const char *what)
{
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw std::runtime_error(std::string("launch ") + what + ": " + cudaGetErrorString(e));
}

// 128-bit key; hi word compared first.
struct Key128 {
  uint64_t lo, hi;
};
__host__ __device__ inline bool key_less(const Key128 &a, const Key128 &b)
{
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__host__ __device__ inline bool key_eq(const Key128 &a, const Key128 &b) { return a.hi == b.hi && a.lo == b.lo; }

template <typename K> __device__ __forceinline__ unsigned key_digit(const K &k, int shift);
template <> __device__ __forceinline__ unsigned key_digit<uint64_t>(const uint64_t &k, int shift)
{
  return (unsigned) (k >> shift) & 0xFFu;
}
template <> __device__ __forceinline__ unsigned key_digit<Key128>(const Key128 &k, int shift)
{
  if (shift >= 64) return (unsigned) (k.hi >> (shift - 64)) & 0xFFu;
  if (shift > 56) return (unsigned) ((k.lo >> shift) | (k.hi << (64 - shift))) & 0xFFu;
  return (unsigned) (k.lo >> shift) & 0xFFu;
}

// Device buffer with RAII.
// Raises (never lowers) a kernel's dynamic shared-memory limit.  The limit is
// per function and shared by all host threads, so a thread that lowered it
// could make another thread's launch with a larger size fail; only raising
// it, under a lock, keeps every concurrent launch within the limit.
template <typename F>
inline void ensure_dyn_smem(F *kfn, size_t bytes)
{
  if (bytes <= 48 * 1024) return;
  static std::mutex m;
  static std::map<std::pair<int, const void *>, size_t> cur;
  int dev = 0;
  DKT_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(m);
  size_t &c = cur[{dev, reinterpret_cast<const void *>(kfn)}];
  if (bytes > c) {
    DKT_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes));
    c = bytes;
  }
}

// Device bytes held through DBuf by the calling host thread (current and
// peak); a served request reads its own footprint from it.
struct MemCounter {
  int64_t cur = 0, peak = 0;
};
inline MemCounter &mem_counter()
{
  static thread_local MemCounter m;
  return m;
}

// The device's default memory pool keeps freed blocks for reuse instead of
// returning them to the driver at every synchronisation (set once per device).
inline void keep_pool_memory()
{
  static std::atomic<unsigned long long> done{0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
  const unsigned long long bit = 1ull << dev;
  if (done.load() & bit) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done.fetch_or(bit);
}

template <typename T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  DBuf() = default;
  explicit DBuf(size_t count) { alloc(count); }
  void alloc(size_t count)
  {
    free();
    n = count;
    if (count) {
      // Stream-ordered allocation on the calling thread's default stream:
      // unlike cudaMalloc/cudaFree it never synchronises the whole device,
      // so threads serving different requests keep the GPU busy together.
      // The sync makes the block usable on any stream at once.
      keep_pool_memory();
      DKT_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&p), count * sizeof(T), cudaStreamPerThread));
      DKT_CUDA(cudaStreamSynchronize(cudaStreamPerThread));
      MemCounter &m = mem_counter();
      m.cur += (int64_t) (count * sizeof(T));
      if (m.cur > m.peak) m.peak = m.cur;
    }
  }
  void free()
  {
    if (p) {
      // no work on any stream may still use the block (every path in this
      // library synchronises its streams before its buffers go)
      cudaFreeAsync(p, cudaStreamPerThread);
      mem_counter().cur -= (int64_t) (n * sizeof(T));
    }
    p = nullptr;
    n = 0;
  }
  ~DBuf() { free(); }
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DBuf &operator=(DBuf &&o) noexcept
  {
    if (this != &o) { free(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  void upload(const T *h, size_t count, cudaStream_t s = 0)
  {
    if (count > n) alloc(count);
    if (count) DKT_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  std::vector<T> download(size_t count, cudaStream_t s = 0) const
  {
    std::vector<T> h(count);
    if (count) DKT_CUDA(cudaMemcpyAsync(h.data(), p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    if (count) DKT_CUDA(cudaStreamSynchronize(s));
    return h;
  }
};

// ---------------------------------------------------------------------------
// Exclusive scan (uint32 or uint64), three phases, recursive over block sums.
// ---------------------------------------------------------------------------
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename T>
__global__ void scan_tiles_kernel(const T *__restrict__ in, T *__restrict__ out, T *__restrict__ sums, size_t n)
{
  __shared__ T warp_tot[SCAN_THREADS / 32];
  const size_t base = (size_t) blockIdx.x * SCAN_TILE + (size_t) threadIdx.x * SCAN_ITEMS;
  T v[SCAN_ITEMS];
  T acc = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    T x = (base + i < n) ? in[base + i] : (T) 0;
    v[i] = acc;
    acc += x;
  }
  // inclusive warp scan of per-thread totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T incl = acc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    T w = (lane < SCAN_THREADS / 32) ? warp_tot[lane] : (T) 0;
    T wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < SCAN_THREADS / 32) warp_tot[lane] = wi - w;
    if (lane == SCAN_THREADS / 32 - 1 && sums) sums[blockIdx.x] = wi;
  }
  __syncthreads();
  const T off = warp_tot[warp] + (incl - acc);
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++)
    if (base + i < n) out[base + i] = v[i] + off;
}

template <typename T>
__global__ void scan_add_kernel(T *__restrict__ out, const T *__restrict__ sums, size_t n)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += sums[i / SCAN_TILE];
}

// out[i] = sum_{j<i} in[j]; returns nothing (total via out[n-1]+in[n-1]).
template <typename T>
void exclusive_scan(const T *in, T *out, size_t n, cudaStream_t s)
{
  if (n == 0) return;
  const size_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles == 1) {
    scan_tiles_kernel<T><<<1, SCAN_THREADS, 0, s>>>(in, out, nullptr, n);
    check_launch("scan");
    return;
  }
  DBuf<T> sums(tiles), sums_scan(tiles);
  scan_tiles_kernel<T><<<(unsigned) tiles, SCAN_THREADS, 0, s>>>(in, out, sums.p, n);
  check_launch("scan");
  exclusive_scan<T>(sums.p, sums_scan.p, tiles, s);
  scan_add_kernel<T><<<(unsigned) ((n + 255) / 256), 256, 0, s>>>(out, sums_scan.p, n);
  check_launch("scan_add");
  DKT_CUDA(cudaStreamSynchronize(s));   // sums buffers are freed on return
}

// Exclusive scan that also returns the total on the host.
template <typename T>
T exclusive_scan_total(const T *in, T *out, size_t n, cudaStream_t s)
{
  if (n == 0) return 0;
  exclusive_scan<T>(in, out, n, s);
  T a = 0, b = 0;
  DKT_CUDA(cudaMemcpyAsync(&a, out + n - 1, sizeof(T), cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaMemcpyAsync(&b, in + n - 1, sizeof(T), cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaStreamSynchronize(s));
  return a + b;
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits.  Tile = 256 threads x 16 rounds; the
// element of round r, warp w, lane l is tile index r*256 + w*32 + l, and its
// rank among equal digits in the tile is built from __match_any_sync counts,
// which keeps equal digits in index order (stability).
// ---------------------------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;

template <typename K>
__global__ void radix_hist_kernel(const K *__restrict__ keys, uint32_t *__restrict__ counts, size_t n, int shift,
                                  unsigned ntiles)
{
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const size_t base = (size_t) blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ROUNDS; r++) {
    const size_t i = base + (size_t) r * RS_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&h[key_digit<K>(keys[i], shift)], 1u);
  }
  __syncthreads();
  counts[(size_t) threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

template <typename K, typename V>
__global__ void radix_scatter_kernel(const K *__restrict__ kin, K *__restrict__ kout, const V *__restrict__ vin,
                                     V *__restrict__ vout, const uint32_t *__restrict__ offs, size_t n, int shift,
                                     unsigned ntiles)
{
  __shared__ uint32_t running[256];
  __shared__ uint32_t cnt[RS_THREADS / 32][256];
  __shared__ uint32_t gbase[256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  running[threadIdx.x] = 0;
  gbase[threadIdx.x] = offs[(size_t) threadIdx.x * ntiles + blockIdx.x];
  const size_t base = (size_t) blockIdx.x * RS_TILE;
  const unsigned lt = (1u << lane) - 1u;
  for (int r = 0; r < RS_ROUNDS; r++) {
#pragma unroll
    for (int w = 0; w < RS_THREADS / 32; w++) cnt[w][threadIdx.x] = 0;
    __syncthreads();
    const size_t i = base + (size_t) r * RS_THREADS + threadIdx.x;
    const bool valid = i < n;
    K k;
    unsigned dg = 256;   // sentinel for invalid lanes, never matches a real digit
    if (valid) { k = kin[i]; dg = key_digit<K>(k, shift); }
    const unsigned m = __match_any_sync(0xffffffffu, dg);
    const unsigned lrank = __popc(m & lt);
    if (valid && lrank == 0) cnt[warp][dg] = __popc(m);
    __syncthreads();
    {
      uint32_t p = running[threadIdx.x];
#pragma unroll
      for (int w = 0; w < RS_THREADS / 32; w++) {
        uint32_t t = cnt[w][threadIdx.x];
        cnt[w][threadIdx.x] = p;
        p += t;
      }
      running[threadIdx.x] = p;
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = gbase[dg] + cnt[warp][dg] + lrank;
      kout[pos] = k;
      if (vout) vout[pos] = vin[i];
    }
    __syncthreads();
  }
}

// Sorts (keys, values) by the key bits [0, nbits).  Keys and values are
// sorted in place (double-buffered internally).  values may be null.
template <typename K, typename V>
void radix_sort_pairs(K *keys, V *vals, size_t n, int nbits, cudaStream_t s)
{
  if (n <= 1) return;
  const unsigned ntiles = (unsigned) ((n + RS_TILE - 1) / RS_TILE);
  DBuf<K> k2(n);
  DBuf<V> v2(vals ? n : 0);
  DBuf<uint32_t> counts((size_t) 256 * ntiles), offs((size_t) 256 * ntiles);
  K *ka = keys, *kb = k2.p;
  V *va = vals, *vb = v2.p;
  const int passes = (nbits + 7) / 8;
  for (int ps = 0; ps < passes; ps++) {
    const int shift = ps * 8;
    radix_hist_kernel<K><<<ntiles, RS_THREADS, 0, s>>>(ka, counts.p, n, shift, ntiles);
    check_launch("radix_hist");
    exclusive_scan<uint32_t>(counts.p, offs.p, (size_t) 256 * ntiles, s);
    radix_scatter_kernel<K, V><<<ntiles, RS_THREADS, 0, s>>>(ka, kb, va, vb, offs.p, n, shift, ntiles);
    check_launch("radix_scatter");
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    DKT_CUDA(cudaMemcpyAsync(keys, ka, n * sizeof(K), cudaMemcpyDeviceToDevice, s));
    if (vals) DKT_CUDA(cudaMemcpyAsync(vals, va, n * sizeof(V), cudaMemcpyDeviceToDevice, s));
  }
  DKT_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------------
// Compaction helpers.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void scatter_if_kernel(const T *__restrict__ in, const uint32_t *__restrict__ flag,
                                  const uint32_t *__restrict__ pos, T *__restrict__ out, size_t n)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flag[i]) out[pos[i]] = in[i];
}

// Lower bound of key in sorted[0, n).
__device__ __forceinline__ int64_t lower_bound_u64(const uint64_t *__restrict__ sorted, int64_t n, uint64_t key)
{
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (sorted[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

inline unsigned grid_for(size_t n, unsigned threads = 256)
{
  return (unsigned) ((n + threads - 1) / threads);
}

}  // namespace dkt
