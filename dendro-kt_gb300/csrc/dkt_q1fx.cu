// Linear-element (Q1) leaf kernel in exact 64-bit fixed point.
//
// GB300 executes FP64 at about 1/58 of its FP32 rate (0.63 T FMA/s measured),
// so a dense FP64 nPe x nPe product per leaf is compute bound far below the
// HBM roof.  For the built-in Q1 operators every elemental matrix is diagonal
// in the Hadamard basis: the 1D reference mass [[2,1],[1,2]]/3 and stiffness
// [[1,-1],[-1,1]]/2 both equal H diag(.) H with H = [[1,1],[1,-1]], so
//     K_L = H^(x)d  diag(D_L)  H^(x)d,
//     D_L[s] = alpha_L * sum_a lk(s_a) prod_{b!=a} lm(s_b) + beta_L * prod_b lm(s_b),
// lm = (1/2, 1/6), lk = (0, 1/2) (identity: D = 2^-d).  The leaf work is then
// two Walsh-Hadamard transforms (additions), one scaling per mode and, for
// hanging leaves, the child interpolation and its transpose (halvings) --
// all done on int64 fixed-point values, accumulated with integer atomics.
// Integer addition is associative, so the product is bitwise deterministic
// whatever the launch order.
//
// Scales: x is stored as xq = round(x * 2^sx) with |xq| <= 2^(60-dim); the
// per-mode factors carry 2^c so that every contribution stays below
// 2^(54-dim) and a node can absorb 256 of them; y = yq * 2^-(sx+c).
#include <algorithm>
#include <cmath>
#include <type_traits>
#include "dkt_internal.cuh"
#include "dkt_q1.cuh"

namespace dkt {

// One thread per four lexicographic ranks of a leaf (2^dim / 4 lanes per
// leaf): butterflies along axes 0 and 1 stay in registers, along the higher
// axes they are warp shuffles between the lanes of the leaf.  Each lane reads
// its four node indices with one 16-byte load.  In fixed point the integer
// steps are the same as evaluating the leaf sequentially, so results are
// bit-identical.
template <typename T>
__device__ __forceinline__ void bfly_reg(T *v, int d)
{
  // axis d in {0, 1} inside the thread's four ranks
#pragma unroll
  for (int k = 0; k < 4; k++) {
    if (k & (1 << d)) continue;
    const T a = v[k], b = v[k | (1 << d)];
    v[k] = a + b;
    v[k | (1 << d)] = a - b;
  }
}

// A contribution of a level-L leaf (fixed point: in level L's unit) added
// into node n, whose sum is in the unit of its coarsest contributing level
// lam[n] <= L: floor(v / 2^(kappa (L - lam[n]))).
template <typename AR>
__device__ __forceinline__ void add_to_node(typename AR::T *yq, int n, typename AR::T v, int L,
                                            const uint8_t *__restrict__ lam, int kappa)
{
  if constexpr (std::is_same<AR, FixedArith>::value) {
    if (lam) v >>= kappa * (L - (int) __ldg(lam + n));
  }
  AR::add(yq + n, v);
}

template <int DIM, typename AR>
__global__ void __launch_bounds__(256) k_matvec_q1(
    const int32_t *__restrict__ e2n, const uint32_t *__restrict__ info, const int32_t *__restrict__ hidx,
    const int32_t *__restrict__ p2n, const uint32_t *__restrict__ fill, int64_t n_leaf, int64_t n_hang,
    const void *__restrict__ fm, const typename AR::T *__restrict__ xq,
    typename AR::T *__restrict__ yq, const int32_t *__restrict__ hzoff, const int32_t *__restrict__ hztab,
    const typename AR::T *__restrict__ stvq, int conforming, const uint8_t *__restrict__ lam, int kappa, int nlev,
    const int32_t *__restrict__ leaf_list = nullptr, int64_t n_list = 0)
{
  using T = typename AR::T;
  constexpr int NPE = 1 << DIM, LPL = NPE / 4;
  const int64_t tid = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t li = tid / LPL;
  // every leaf, or only the leaves of leaf_list
  const bool valid = leaf_list ? li < n_list : li < n_leaf;
  const int64_t i = leaf_list ? (valid ? (int64_t) __ldg(leaf_list + li) : 0) : li;
  const int sub = (int) (tid % LPL);
  const int rb = sub * 4;                      // first rank of this lane
  const uint32_t inf = valid ? __ldg(info + i) : 0u;
  const int L = inf & 0xFFu;
  const unsigned child = (inf >> 8) & 0xFFu;
  const bool hang = (inf >> 16) & 1u;
  int4 e = make_int4(-1, -1, -1, -1);
  if (valid) e = __ldg(reinterpret_cast<const int4 *>(e2n + i * NPE + rb));
  const int nd[4] = {e.x, e.y, e.z, e.w};
  T v[4];
#pragma unroll
  for (int k = 0; k < 4; k++) v[k] = nd[k] >= 0 ? __ldg(xq + nd[k]) : T(0);
  int64_t h = 0;
  uint32_t fmask = 0xFFFFu;
  int pn[4] = {-1, -1, -1, -1};
  const bool grp_hang = (LPL > 1) ? (bool) __any_sync(0xffffffffu, hang) : hang;
  if (grp_hang) {
    T xp[4] = {T(0), T(0), T(0), T(0)};
    if (hang) {
      h = __ldg(hidx + i);
      fmask = __ldg(fill + h * 3);
      const int4 pq = __ldg(reinterpret_cast<const int4 *>(p2n + h * NPE + rb));
      pn[0] = pq.x; pn[1] = pq.y; pn[2] = pq.z; pn[3] = pq.w;
      const int32_t hz = hzoff ? __ldg(hzoff + h) : -1;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        if (pn[k] >= 0) xp[k] = __ldg(xq + pn[k]);
        else if (hz >= 0) {
          const int32_t id = __ldg(hztab + (int64_t) hz * NPE + rb + k);
          if (id >= 0) xp[k] = __ldg(stvq + id);
        }
      }
    }
    // parent -> child interpolation
#pragma unroll
    for (int d = 0; d < 2; d++) {
      const bool cb = (child >> d) & 1u;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        if (k & (1 << d)) continue;
        const T m = AR::half_sum(xp[k], xp[k | (1 << d)]);
        if (cb) xp[k] = m; else xp[k | (1 << d)] = m;
      }
    }
#pragma unroll
    for (int d = 2; d < DIM; d++) {
      const bool cb = (child >> d) & 1u;
      const bool mine = (sub >> (d - 2)) & 1;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const T o = __shfl_xor_sync(0xffffffffu, xp[k], 1 << (d - 2));
        if (mine != cb) xp[k] = AR::half_sum(xp[k], o);
      }
    }
    if (hang) {
#pragma unroll
      for (int k = 0; k < 4; k++)
        if (!((fmask >> (rb + k)) & 1u)) v[k] = xp[k];
    }
  }
  // Walsh-Hadamard transform, per-mode scaling, transform back
  bfly_reg<T>(v, 0);
  bfly_reg<T>(v, 1);
#pragma unroll
  for (int d = 2; d < DIM; d++) {
    const bool mine = (sub >> (d - 2)) & 1;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const T o = __shfl_xor_sync(0xffffffffu, v[k], 1 << (d - 2));
      v[k] = mine ? (o - v[k]) : (v[k] + o);
    }
  }
  if (valid) {
    // fixed point: the factors of the leaf's own level unit (row L of the
    // per-unit table); binary32: one row per level
    const int frow = std::is_same<AR, FixedArith>::value ? (L * nlev + L) * NPE : L * NPE;
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = AR::scale(v[k], fm, frow + rb + k);
  }
  bfly_reg<T>(v, 0);
  bfly_reg<T>(v, 1);
#pragma unroll
  for (int d = 2; d < DIM; d++) {
    const bool mine = (sub >> (d - 2)) & 1;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const T o = __shfl_xor_sync(0xffffffffu, v[k], 1 << (d - 2));
      v[k] = mine ? (o - v[k]) : (v[k] + o);
    }
  }
#pragma unroll
  for (int k = 0; k < 4; k++)
    if (nd[k] >= 0) add_to_node<AR>(yq, nd[k], v[k], L, lam, kappa);
  if (grp_hang) {
    // transpose of the interpolation on the unfilled ranks, into the parent nodes
    T z[4];
#pragma unroll
    for (int k = 0; k < 4; k++) z[k] = (hang && !((fmask >> (rb + k)) & 1u)) ? v[k] : T(0);
#pragma unroll
    for (int d = 0; d < 2; d++) {
      const bool cb = (child >> d) & 1u;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        if (k & (1 << d)) continue;
        const T a = z[k], b = z[k | (1 << d)];
        if (cb) { z[k] = AR::half(a); z[k | (1 << d)] = b + AR::half(a); }
        else { z[k] = a + AR::half(b); z[k | (1 << d)] = AR::half(b); }
      }
    }
#pragma unroll
    for (int d = 2; d < DIM; d++) {
      const bool cb = (child >> d) & 1u;
      const bool mine = (sub >> (d - 2)) & 1;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const T o = __shfl_xor_sync(0xffffffffu, z[k], 1 << (d - 2));
        z[k] = (mine == cb) ? z[k] + AR::half(o) : AR::half(z[k]);
      }
    }
    if (hang) {
#pragma unroll
      for (int k = 0; k < 4; k++)
        if (pn[k] >= 0 && (conforming || !((fmask >> (rb + k)) & 1u))) add_to_node<AR>(yq, pn[k], z[k], L, lam, kappa);
    }
  }
}

// The passes between FP64 and fixed point run on the integer pipes: GB300
// executes FP64 (and FP64 conversions) at a small fraction of its integer
// rate, enough to make these memory-bound passes compute-bound otherwise.

// max |x|: the largest bit pattern of |x| (non-negative doubles order as
// integers): grid-stride loads four apart, a block reduction, one atomic per block.
__global__ void __launch_bounds__(256) k_absmax(const double *__restrict__ x, int64_t n,
                                                unsigned long long *__restrict__ out)
{
  __shared__ unsigned long long sh[8];
  constexpr unsigned long long ABS = 0x7FFFFFFFFFFFFFFFull;
  const unsigned long long *xb = reinterpret_cast<const unsigned long long *>(x);
  unsigned long long m = 0;
  const int64_t stride = (int64_t) gridDim.x * blockDim.x;
  const int64_t tid = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if ((reinterpret_cast<uintptr_t>(x) & 15u) == 0) {
    // 16-byte loads over the pairs, four in flight
    const ulonglong2 *x2 = reinterpret_cast<const ulonglong2 *>(x);
    const int64_t n2 = n >> 1;
    int64_t i = tid;
    for (; i + 3 * stride < n2; i += 4 * stride) {
      const ulonglong2 a = __ldg(x2 + i), b = __ldg(x2 + i + stride), c = __ldg(x2 + i + 2 * stride),
                       d = __ldg(x2 + i + 3 * stride);
      m = max(m, max(max(a.x & ABS, a.y & ABS), max(b.x & ABS, b.y & ABS)));
      m = max(m, max(max(c.x & ABS, c.y & ABS), max(d.x & ABS, d.y & ABS)));
    }
    for (; i < n2; i += stride) {
      const ulonglong2 a = __ldg(x2 + i);
      m = max(m, max(a.x & ABS, a.y & ABS));
    }
    if (tid == 0 && (n & 1)) m = max(m, xb[n - 1] & ABS);
  } else {
    // an 8-byte-aligned view (e.g. an offset slice): scalar loads
    for (int64_t i = tid; i < n; i += stride) m = max(m, xb[i] & ABS);
  }
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int) (blockDim.x >> 5); w++) m = max(m, sh[w]);
    atomicMax(out, m);
  }
}

// sx from max|x|: xq = round(x * 2^sx) keeps |xq| <= 2^bx
__device__ __forceinline__ int fixed_exponent(const unsigned long long *amax, int bx)
{
  const unsigned long long b = *amax;
  if (b == 0) return bx;
  const int ef = (int) (b >> 52);                       // biased exponent (|x| finite)
  const int e = ef == 0 ? -1010 - __clzll(b) : ef - 1022;   // max|x| < 2^e, as frexp
  return bx - e;
}

// x * 2^k as two exact power-of-two products (|k| <= 2046); ldexp(x, k)
__device__ __forceinline__ double scale2(double x, int k)
{
  const int h = k / 2;
  return (x * __longlong_as_double((long long) (1023 + h) << 52)) *
         __longlong_as_double((long long) (1023 + (k - h)) << 52);
}

// round(x * 2^sx) to nearest even, in integer arithmetic (|result| < 2^63)
__device__ __forceinline__ long long fixed_from_double(double x, int sx)
{
  const unsigned long long b = (unsigned long long) __double_as_longlong(x);
  const int ef = (int) ((b >> 52) & 0x7FF);
  unsigned long long m = b & ((1ull << 52) - 1);
  int e;                                                // |x| = m * 2^e
  if (ef == 0) e = -1074;
  else { m |= 1ull << 52; e = ef - 1075; }
  const int k = e + sx;
  unsigned long long q;
  if (m == 0 || k < -63) q = 0;
  else if (k >= 0) q = m << k;
  else {
    const int r = -k;
    q = m >> r;
    const unsigned long long rem = m & ((1ull << r) - 1), half = 1ull << (r - 1);
    if (rem > half || (rem == half && (q & 1ull))) q++;
  }
  return (b >> 63) ? -(long long) q : (long long) q;
}

// (double) v * 2^sh: the int64 -> double rounding (to nearest even) and the
// exponent, in integer arithmetic; results outside the normal range take
// the FP64 path
__device__ __forceinline__ double double_from_fixed(long long v, int sh)
{
  if (v == 0) return 0.0;
  const bool neg = v < 0;
  const unsigned long long a = neg ? 0ull - (unsigned long long) v : (unsigned long long) v;
  const int msb = 63 - __clzll(a);
  unsigned long long m;
  int e = msb;
  if (msb <= 52) {
    m = a << (52 - msb);
  } else {
    const int r = msb - 52;
    m = a >> r;
    const unsigned long long rem = a & ((1ull << r) - 1), half = 1ull << (r - 1);
    if (rem > half || (rem == half && (m & 1ull))) {
      m++;
      if (m == (1ull << 53)) { m >>= 1; e++; }
    }
  }
  const int be = e + sh + 1023;
  if (be <= 0 || be >= 2047) return scale2((double) v, sh);
  return __longlong_as_double((long long) (((unsigned long long) neg << 63) | ((unsigned long long) be << 52) |
                                           (m & ((1ull << 52) - 1))));
}

// The conversion passes take two elements per thread, with one 16-byte load
// and store when the caller's vector is 16-byte aligned (twice the bytes in
// flight of one 8-byte element per thread); thread t does elements 2t, 2t+1.
inline unsigned pair_grid(int64_t n) { return grid_for((n + 1) / 2); }

// xq = round(x * 2^sx)
__global__ void k_to_fixed(const double *__restrict__ x, long long *__restrict__ xq, int64_t n,
                           const unsigned long long *__restrict__ amax, int *__restrict__ sx_out, int bx)
{
  const int sx = fixed_exponent(amax, bx);
  const int64_t i = 2 * ((int64_t) blockIdx.x * blockDim.x + threadIdx.x);
  if (i == 0) *sx_out = sx;
  if (i + 1 < n && (reinterpret_cast<uintptr_t>(x) & 15u) == 0) {
    const double2 v = __ldg(reinterpret_cast<const double2 *>(x + i));
    reinterpret_cast<longlong2 *>(xq)[i >> 1] = make_longlong2(fixed_from_double(v.x, sx), fixed_from_double(v.y, sx));
  } else {
    if (i < n) xq[i] = fixed_from_double(x[i], sx);
    if (i + 1 < n) xq[i + 1] = fixed_from_double(x[i + 1], sx);
  }
}

// round(v / DIV), halves away from zero (DIV a compile-time constant: a
// multiply-high, no division instruction)
template <int DIV>
__device__ __forceinline__ long long div_round(long long v)
{
  if constexpr (DIV == 1) return v;
  const unsigned long long a = v < 0 ? 0ull - (unsigned long long) v : (unsigned long long) v;
  const long long q = (long long) ((a + DIV / 2) / (unsigned long long) DIV);
  return v < 0 ? -q : q;
}

// y = round(yq / DIV) * 2^-(sx + c + kappa lam[i]): the dyadic scaling leaves
// 3^dim times the product in yq (DIV = 3^dim), the per-mode factors the
// product itself; node i's sum is in the unit of its level lam[i] (lam
// null: one unit)
template <int DIV>
__global__ void k_from_fixed(const long long *__restrict__ yq, double *__restrict__ y, int64_t n,
                             const int *__restrict__ sx, int c, const uint8_t *__restrict__ lam, int kappa)
{
  const int sh = -(*sx + c);
  const int64_t i = 2 * ((int64_t) blockIdx.x * blockDim.x + threadIdx.x);
  if (i + 1 < n && (reinterpret_cast<uintptr_t>(y) & 15u) == 0) {
    const longlong2 v = reinterpret_cast<const longlong2 *>(yq)[i >> 1];
    int s0 = sh, s1 = sh;
    if (lam) {
      const uchar2 l = reinterpret_cast<const uchar2 *>(lam)[i >> 1];
      s0 -= kappa * l.x;
      s1 -= kappa * l.y;
    }
    reinterpret_cast<double2 *>(y)[i >> 1] =
        make_double2(double_from_fixed(div_round<DIV>(v.x), s0), double_from_fixed(div_round<DIV>(v.y), s1));
  } else {
    if (i < n) y[i] = double_from_fixed(div_round<DIV>(yq[i]), sh - (lam ? kappa * lam[i] : 0));
    if (i + 1 < n) y[i + 1] = double_from_fixed(div_round<DIV>(yq[i + 1]), sh - (lam ? kappa * lam[i + 1] : 0));
  }
}

__global__ void k_zero_ids_ll(long long *__restrict__ v, const uint32_t *__restrict__ ids, int64_t nb)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nb) v[ids[i]] = 0;
}
__global__ void k_zero_ids_d(double *__restrict__ v, const uint32_t *__restrict__ ids, int64_t nb)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nb) v[ids[i]] = 0.0;
}
__global__ void k_min_level(const uint32_t *__restrict__ info, int64_t n, int *__restrict__ out)
{
  int m = 255;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x)
    m = min(m, (int) (info[i] & 0xFFu));
  atomicMin(out, m);
}

// lam[n] = the coarsest level of a leaf that adds into node n (its own
// ranks, and the parent ranks of the hanging leaves)
__global__ void k_node_minlev(const int32_t *__restrict__ e2n, const uint32_t *__restrict__ info,
                              const int32_t *__restrict__ hidx, const int32_t *__restrict__ p2n, int64_t n_leaf,
                              int npe, uint32_t *__restrict__ lam)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_leaf) return;
  const uint32_t inf = info[i];
  const uint32_t L = inf & 0xFFu;
  for (int k = 0; k < npe; k++) {
    const int32_t n = e2n[i * npe + k];
    if (n >= 0) atomicMin(lam + n, L);
  }
  if ((inf >> 16) & 1u) {
    const int64_t h = hidx[i];
    for (int k = 0; k < npe; k++) {
      const int32_t n = p2n[h * npe + k];
      if (n >= 0) atomicMin(lam + n, L);
    }
  }
}
__global__ void k_lam_narrow(const uint32_t *__restrict__ in, uint8_t *__restrict__ out, int64_t n, uint32_t dflt)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (uint8_t) (in[i] == 0xFFFFFFFFu ? dflt : in[i]);
}

void stale_eval(Plan &pl, const double *x, const long long *xq, cudaStream_t s);

// Host setup of the per-(level, mode) factors.  Returns false when the
// operator is not one of the diagonalisable Q1 built-ins.
//
// Fixed-point units.  The built-in operators are K_L = alpha_L A + beta_L B
// (A the Laplacian, B the mass); on the unit cube alpha_L and beta_L are
// powers of two that fall by 2^kappa per level (kappa = dim - 2 for the
// Laplacian, dim for the mass).  One unit for every level would leave the
// finest levels' contributions 2^(kappa (L - lmin)) smaller than the unit's
// scale -- some forty bits at level 8 in 4D instead of fifty.  So each level L
// has its own unit, 2^(-kappa L) times the level-0 unit: a node keeps its sum
// in the unit of the coarsest level adding into it (fx_lam), a tile computes
// in the unit of its coarsest leaf level tau (tl_tau) and converts each node
// sum once when it flushes it, and the per-leaf kernel computes in its leaf's
// own unit.  fx_fm holds the multiply-high factors of every (unit level tau,
// leaf level L >= tau, mode): row tau is a tile's factor table.
bool q1fx_setup(Plan &pl, cudaStream_t s)
{
  if (pl.order != 1 || pl.op.kind == OP_CUSTOM || pl.n_leaf == 0) return false;
  const int dim = pl.dim, NPE = 1 << dim, nlev = pl.md + 1;
  DBuf<int> dmin(1);
  const int init = 255;
  DKT_CUDA(cudaMemcpyAsync(dmin.p, &init, sizeof(int), cudaMemcpyHostToDevice, s));
  k_min_level<<<304, 256, 0, s>>>(pl.info.p, pl.n_leaf, dmin.p);
  check_launch("min_level");
  int lmin = 0;
  DKT_CUDA(cudaMemcpyAsync(&lmin, dmin.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaStreamSynchronize(s));
  // D_L[s]: the element matrix of level L in the Hadamard basis
  std::vector<double> D((size_t) nlev * NPE, 0.0);
  double maxD = 0.0;
  for (int L = 0; L < nlev; L++)
    for (int sidx = 0; sidx < NPE; sidx++) {
      double v;
      if (pl.op.kind == OP_IDENTITY) v = std::ldexp(1.0, -dim);
      else {
        double lapl = 0.0, mass = 1.0;
        for (int a = 0; a < dim; a++) {
          double t = ((sidx >> a) & 1) ? 0.5 : 0.0;
          for (int b = 0; b < dim; b++)
            if (b != a) t *= ((sidx >> b) & 1) ? (1.0 / 6.0) : 0.5;
          lapl += t;
          mass *= ((sidx >> a) & 1) ? (1.0 / 6.0) : 0.5;
        }
        v = pl.op.alpha[L] * lapl + pl.op.beta[L] * mass;
      }
      D[(size_t) L * NPE + sidx] = v;
      if (L >= lmin) maxD = std::max(maxD, std::fabs(v));
    }
  if (!(maxD > 0.0)) return false;
  // In the Hadamard basis 6^dim D_L[s] = C1(k) alpha_L + C2(k) beta_L with
  // k = popcount(s), C1(k) = k 3^(dim-k+1), C2(k) = 3^(dim-k) (integers).
  int p3 = 1;
  for (int a = 0; a < dim; a++) p3 *= 3;
  std::vector<double> C1(dim + 1), C2(dim + 1);
  for (int k = 0; k <= dim; k++) {
    int t = 1;
    for (int a = 0; a < dim - k; a++) t *= 3;
    C2[k] = t;
    C1[k] = k == 0 ? 0.0 : (double) k * t * 3;
  }
  // Dyadic operators: every alpha_L, beta_L (L >= lmin) a power of two or zero.
  const int kind = pl.op.kind;
  bool dy = kind == OP_LAPMASS || kind == OP_LAPLACE || kind == OP_MASS || kind == OP_HEAT || kind == OP_HEATVEC;
  int mode = 0;
  std::vector<int> ea(nlev, 0), eb(nlev, 0);
  auto pow2 = [](double v, int &e) {   // v = 2^e exactly
    int q = 0;
    const double m = std::frexp(v, &q);
    e = q - 1;
    return m == 0.5;
  };
  for (int L = lmin; L < nlev && dy; L++) {
    const double al = pl.op.alpha[L], be = pl.op.beta[L];
    if (al != 0.0) { mode |= 1; dy = dy && al > 0.0 && pow2(al, ea[L]); }
    if (be != 0.0) { mode |= 2; dy = dy && be > 0.0 && pow2(be, eb[L]); }
  }
  dy = dy && mode != 0;
  if (dy) {
    // the integer form against D computed directly
    for (int L = lmin; L < nlev; L++)
      for (int sidx = 0; sidx < NPE; sidx++) {
        const int k = __builtin_popcount(sidx);
        const double e = (C1[k] * pl.op.alpha[L] + C2[k] * pl.op.beta[L]) / std::ldexp((double) p3, dim);
        const double d = D[(size_t) L * NPE + sidx];
        if (std::fabs(e - d) > 1e-15 * std::fabs(d)) dy = false;
      }
  }
  // kappa: the level exponent of the leading term
  int kappa = 0;
  if (dy && lmin + 1 < nlev) {
    const std::vector<int> &ex = (mode & 1) ? ea : eb;
    kappa = ex[lmin] - ex[lmin + 1];
    for (int L = lmin; L + 1 < nlev; L++)
      if (ex[L] - ex[L + 1] != kappa) kappa = -1;
    if (kappa < 0 || kappa > 4) kappa = 0;
  }
  // Per level the scaled factors F_L[s] (6^dim D_L[s] when dyadic, else
  // D_L[s]); unit exponents cp + kappa L keep F_L 2^(cp + kappa L) below
  // 2^-6 for every level and mode (dyadic), or below 2^(-6-dim) (one unit).
  auto F = [&](int L, int sidx) {
    return dy ? C1[__builtin_popcount(sidx)] * pl.op.alpha[L] + C2[__builtin_popcount(sidx)] * pl.op.beta[L]
              : D[(size_t) L * NPE + sidx];
  };
  double g = 0.0;
  for (int L = lmin; L < nlev; L++)
    for (int sidx = 0; sidx < NPE; sidx++) g = std::max(g, std::ldexp(std::fabs(F(L, sidx)), kappa * L));
  int eg = 0;
  std::frexp(g, &eg);                        // g < 2^eg
  const int cp = dy ? -6 - eg : -6 - dim - eg;
  // fm[(tau nlev + L) NPE + s] = round(F_L[s] 2^(cp + kappa tau + 64)) < 2^58
  // for lmin <= tau <= L (0 elsewhere): a transformed value (below
  // 2^(bx + dim)) times the factor, high word, stays below 2^(bx + dim - 6)
  std::vector<long long> fm((size_t) nlev * nlev * NPE, 0);
  for (int tau = lmin; tau < nlev; tau++)
    for (int L = tau; L < nlev; L++)
      for (int sidx = 0; sidx < NPE; sidx++)
        fm[((size_t) tau * nlev + L) * NPE + sidx] =
            (long long) std::llround(std::ldexp(F(L, sidx), cp + kappa * tau + 64));
  // Dyadic scaling in the tiled kernel: the mode value w of a level-L leaf
  // in a tile of unit level tau becomes
  //   (C1(k) w + (C2(k) w >> d_L)) >> (s_L - kappa tau)       (both terms)
  //   (C(k) w) >> (s_L - kappa tau)                          (one term)
  // with every shift below 32 (two-instruction shifts); otherwise the
  // multiply-high factors are used.
  std::vector<uint32_t> sh(nlev, 0u);
  int sc_mode = 0;
  if (dy) {
    sc_mode = mode;
    for (int L = lmin; L < nlev && sc_mode; L++) {
      const int e_lead = (mode & 1) ? ea[L] : eb[L];   // the leading term's exponent
      const int sl = -(e_lead + cp);
      const int dl = (mode == 3) ? ea[L] - eb[L] : 0;
      // the coarsest unit a level-L leaf can be computed in is level lmin's
      if (sl - kappa * L < 0 || sl - kappa * lmin > 31 || dl < 0 || dl > 31 || (mode == 3 && dl < 1)) sc_mode = 0;
      sh[L] = (uint32_t) sl | ((uint32_t) dl << 8);
    }
  }
  pl.fx_shift.upload(sh.data(), sh.size(), s);
  pl.fx_fm.upload(fm.data(), fm.size(), s);
  pl.fx_scale = sc_mode;
  pl.fx_div = dy ? p3 : 1;
  pl.fx_bx = dy ? 60 - 2 * dim : 60 - dim;
  pl.fx_c = dy ? cp + dim : cp;
  pl.fx_kappa = kappa;
  if (kappa > 0) {
    DBuf<uint32_t> lam32(pl.n_nodes);
    DKT_CUDA(cudaMemsetAsync(lam32.p, 0xFF, pl.n_nodes * sizeof(uint32_t), s));
    k_node_minlev<<<grid_for(pl.n_leaf), 256, 0, s>>>(pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.n_leaf, NPE,
                                                      lam32.p);
    pl.fx_lam.alloc(pl.n_nodes);
    k_lam_narrow<<<grid_for(pl.n_nodes), 256, 0, s>>>(lam32.p, pl.fx_lam.p, pl.n_nodes, (uint32_t) lmin);
    check_launch("node_levels");
    DKT_CUDA(cudaStreamSynchronize(s));
  }
  std::vector<float> f32(D.size());
  for (size_t k = 0; k < D.size(); k++) f32[k] = (float) D[k];
  pl.f32_f.upload(f32.data(), f32.size(), s);
  pl.f32_ready = !pl.st_ready || pl.st_n_runs == 0;
  pl.xq.alloc(pl.n_nodes);
  pl.yq.alloc(pl.n_nodes);
  pl.fx_amax.alloc(1);
  pl.fx_sx.alloc(1);
  pl.fx_ready = true;
  return true;
}

void tiled_fixed(Plan &pl, bool skip_stale, cudaStream_t s);
void tiled_f32(Plan &pl, const float *x, float *y, cudaStream_t s);

// The leaves that read stale slots, after the chain (per-leaf kernel).
template <int DIM>
static void launch_q1fx_stale_leaves(Plan &pl, cudaStream_t s)
{
  const unsigned threads = 256;
  k_matvec_q1<DIM, FixedArith><<<grid_for(pl.st_n_hleaf * ((1 << DIM) / 4), threads), threads, 0, s>>>(
      pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.fill.p, pl.n_leaf, pl.n_hang, pl.fx_fm.p, pl.xq.p,
      pl.yq.p, pl.st_hzoff.p, pl.st_hztab.p, pl.st_vq.p, pl.conforming ? 1 : 0,
      pl.fx_kappa > 0 ? pl.fx_lam.p : nullptr, pl.fx_kappa, pl.md + 1, pl.st_hleaves.p, pl.st_n_hleaf);
  check_launch("matvec_q1fx_stale_leaves");
  pl.n_launch++;
}

template <int DIM>
static void launch_q1fx(Plan &pl, bool skip_stale, cudaStream_t s)
{
  const unsigned threads = 256;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (pl.timing) {
    DKT_CUDA(cudaEventCreate(&e0));
    DKT_CUDA(cudaEventCreate(&e1));
    DKT_CUDA(cudaEventRecord(e0, s));
  }
  if (pl.tl_ready) tiled_fixed(pl, skip_stale, s);
  else k_matvec_q1<DIM, FixedArith><<<grid_for(pl.n_leaf * ((1 << DIM) / 4), threads), threads, 0, s>>>(
      pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.fill.p, pl.n_leaf, pl.n_hang, pl.fx_fm.p,
      pl.xq.p, pl.yq.p, pl.st_ready ? pl.st_hzoff.p : nullptr, pl.st_hztab.p, pl.st_vq.p, pl.conforming ? 1 : 0,
      pl.fx_kappa > 0 ? pl.fx_lam.p : nullptr, pl.fx_kappa, pl.md + 1);
  if (!pl.tl_ready) {
    check_launch("matvec_q1fx");
    pl.n_launch++;
  }
  if (pl.timing) {
    DKT_CUDA(cudaEventRecord(e1, s));
    pl.ev.push_back(e0);
    pl.ev.push_back(e1);
    pl.timed_launches++;
  }
}

template <int DIM>
static void launch_q1f32(Plan &pl, const float *x, float *y, cudaStream_t s)
{
  const unsigned threads = 256;
  if (pl.tl_ready) { tiled_f32(pl, x, y, s); return; }
  k_matvec_q1<DIM, F32Arith><<<grid_for(pl.n_leaf * ((1 << DIM) / 4), threads), threads, 0, s>>>(
      pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.fill.p, pl.n_leaf, pl.n_hang, pl.f32_f.p, x, y,
      nullptr, nullptr, nullptr, pl.conforming ? 1 : 0, nullptr, 0, pl.md + 1);
  check_launch("matvec_q1f32");
  pl.n_launch++;
}

__global__ void k_zero_ids_f(float *__restrict__ v, const uint32_t *__restrict__ ids, int64_t nb)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nb) v[ids[i]] = 0.0f;
}

// Binary32 product with the built-in operator of the plan (Q1 here, Q2 in
// dkt_q2sf.cu).  bc_in / bc_out zero the
// domain-boundary entries of the input (through a scratch copy) and of the
// output, as feMatrix::matVec does for the operators with boundary steps.
void q2sf_f32(Plan &pl, const float *x, float *y, cudaStream_t s);

void q1f32_apply(Plan &pl, const float *x, float *y, bool bc_in, bool bc_out, cudaStream_t s)
{
  if (!pl.f32_ready)
    throw std::runtime_error("binary32 product needs a Q1 or Q2 built-in operator without stale parent reads");
  const int64_t n = pl.n_nodes;
  if (bc_in && pl.n_bdry > 0) {
    if (pl.x32.n < (size_t) n) pl.x32.alloc(n);
    DKT_CUDA(cudaMemcpyAsync(pl.x32.p, x, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    k_zero_ids_f<<<grid_for(pl.n_bdry), 256, 0, s>>>(pl.x32.p, pl.bdry.p, pl.n_bdry);
    check_launch("zero_in_f32");
    pl.n_launch++;
    x = pl.x32.p;
  }
  if (pl.order == 2) {
    q2sf_f32(pl, x, y, s);
  } else {
    DKT_CUDA(cudaMemsetAsync(y, 0, n * sizeof(float), s));
    switch (pl.dim) {
      case 2: launch_q1f32<2>(pl, x, y, s); break;
      case 3: launch_q1f32<3>(pl, x, y, s); break;
      case 4: launch_q1f32<4>(pl, x, y, s); break;
      default: throw std::runtime_error("unsupported dim");
    }
  }
  if (bc_out && pl.n_bdry > 0) {
    k_zero_ids_f<<<grid_for(pl.n_bdry), 256, 0, s>>>(y, pl.bdry.p, pl.n_bdry);
    check_launch("zero_out_f32");
    pl.n_launch++;
  }
}

__global__ void k_scale(double *__restrict__ v, int64_t n, double a)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] *= a;
}
void scale_vector(double *v, int64_t n, double a, cudaStream_t s)
{
  k_scale<<<grid_for(n), 256, 0, s>>>(v, n, a);
  check_launch("scale");
}


// fem::matvec / feMatrix::matVec through the fixed-point path.  `bc` applies
// the pre/post boundary zeroing.
// The side stream of the stale-buffer chain and its fork/join events, made on
// first use.  Highest priority: the chain's few, long, latency-bound blocks
// start at once and the leaf kernel fills the rest of the machine around them.
void ensure_side_stream(Plan &pl)
{
  if (pl.st_stream) return;
  int lo = 0, hi = 0;
  DKT_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
  DKT_CUDA(cudaStreamCreateWithPriority(&pl.st_stream, cudaStreamNonBlocking, hi));
  DKT_CUDA(cudaEventCreateWithFlags(&pl.st_fork, cudaEventDisableTiming));
  DKT_CUDA(cudaEventCreateWithFlags(&pl.st_join, cudaEventDisableTiming));
}

void q1fx_matvec(Plan &pl, const double *x, double *y, double scale, bool bc, cudaStream_t s)
{
  const int64_t n = pl.n_nodes;
  DKT_CUDA(cudaMemsetAsync(pl.fx_amax.p, 0, sizeof(unsigned long long), s));
  k_absmax<<<std::max<unsigned>(1u, std::min<unsigned>(grid_for(n, 1024), 152 * 8)), 256, 0, s>>>(x, n, pl.fx_amax.p);
  k_to_fixed<<<pair_grid(n), 256, 0, s>>>(x, pl.xq.p, n, pl.fx_amax.p, pl.fx_sx.p, pl.fx_bx);
  check_launch("to_fixed");
  pl.n_launch += 2;
  if (bc && pl.n_bdry > 0) {
    k_zero_ids_ll<<<grid_for(pl.n_bdry), 256, 0, s>>>(pl.xq.p, pl.bdry.p, pl.n_bdry);
    check_launch("zero_in");
    pl.n_launch++;
  }
  DKT_CUDA(cudaMemsetAsync(pl.yq.p, 0, n * sizeof(long long), s));
  // With tiles, the stale-buffer chain runs on a side stream while the tiled
  // kernel does every leaf that does not read stale slots; those few leaves
  // follow once the chain has joined.
  const bool split = pl.tl_ready && pl.st_ready && pl.st_n_runs > 0 && pl.st_n_hleaf > 0;
  if (split) {
    ensure_side_stream(pl);
    DKT_CUDA(cudaEventRecord(pl.st_fork, s));
    DKT_CUDA(cudaStreamWaitEvent(pl.st_stream, pl.st_fork, 0));
    stale_eval(pl, nullptr, pl.xq.p, pl.st_stream);
    DKT_CUDA(cudaEventRecord(pl.st_join, pl.st_stream));
  } else {
    stale_eval(pl, nullptr, pl.xq.p, s);
  }
  switch (pl.dim) {
    case 2: launch_q1fx<2>(pl, split, s); break;
    case 3: launch_q1fx<3>(pl, split, s); break;
    case 4: launch_q1fx<4>(pl, split, s); break;
    default: throw std::runtime_error("unsupported dim");
  }
  if (split) {
    DKT_CUDA(cudaStreamWaitEvent(s, pl.st_join, 0));
    switch (pl.dim) {
      case 2: launch_q1fx_stale_leaves<2>(pl, s); break;
      case 3: launch_q1fx_stale_leaves<3>(pl, s); break;
      case 4: launch_q1fx_stale_leaves<4>(pl, s); break;
    }
  }
  const uint8_t *lam = pl.fx_kappa > 0 ? pl.fx_lam.p : nullptr;
  switch (pl.fx_div) {
#define DKT_FROM(D) \
  case D: k_from_fixed<D><<<pair_grid(n), 256, 0, s>>>(pl.yq.p, y, n, pl.fx_sx.p, pl.fx_c, lam, pl.fx_kappa); break;
    DKT_FROM(1) DKT_FROM(9) DKT_FROM(27) DKT_FROM(81)
#undef DKT_FROM
    default: throw std::runtime_error("unsupported fixed-point divisor");
  }
  check_launch("from_fixed");
  pl.n_launch++;
  if (bc && pl.n_bdry > 0) {
    k_zero_ids_d<<<grid_for(pl.n_bdry), 256, 0, s>>>(y, pl.bdry.p, pl.n_bdry);
    check_launch("zero_out");
    pl.n_launch++;
  }
  if (scale != 1.0 && pl.op.uses_scale) {
    // the built-in operators are linear in scale
    scale_vector(y, n, scale, s);
    pl.n_launch++;
  }
}

}  // namespace dkt
