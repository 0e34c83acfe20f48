// Sum-factorised leaf kernel for the order-2 built-in operators.
//
// Every Q2 built-in operator (HeatMat<3>, Laplacian + mass, Laplacian, mass,
// HeatVec<3>) is a Kronecker sum of the 1D mass M1 and stiffness K1:
//   K_L = alpha_L sum_t (M1 x .. x K1_t x .. x M1) + beta_L (M1 x .. x M1).
// With M1 = T^T T and K1 = T^T diag(lam) T (q2_factors), this is
//   K_L = (T x .. x T)^T diag(D_L) (T x .. x T),
//   D_L[r] = alpha_L sum_t lam[digit_t(r)] + beta_L,
// so the elemental product of fem::matvec (matvec.h:467-468) becomes a 1D
// transform along every axis, a diagonal scaling and the transposed
// transforms: 2 d 3^(d-1) 4 + 3^d FP64 operations instead of the 2 (3^d)^2
// of the dense contraction (4D: 945 against 13,122).  The
// transform is used in its unit-diagonal form U = diag(1/T_kk) T, rows
// (1, u01, 1), (u10, 1, u10), (-1, 0, 1), whose line products take four
// operations; the row scales move into D.  The child interpolation
// of hanging leaves (IKD_Parent2Child / IKD_Child2Parent, refel.h:214-271) is
// applied the same way with its exact sparsity (two of three rows copy a
// parent node).  FP64 on this part runs at about 2 FMA per clock per SM, so
// operation count is what bounds the kernel.
//
// Three threads work on one leaf, each holding 3^(d-1) of its values, in one
// of two layouts (split by the last-axis index or by the first-axis index);
// every 1D operator runs in the layout where its axis is local to a thread,
// and the values change layout through shared memory (two exchanges per
// leaf, four for a hanging leaf).  A warp takes ten leaves (lanes 30 and 31
// idle).  Leaves run in an order with the hanging
// leaves first (stable), so almost every warp is uniform in whether it runs
// the interpolation.
#include <algorithm>
#include <type_traits>
#include "dkt_host.h"
#include "dkt_internal.cuh"

namespace dkt {

template <typename V>
struct SfCoef {
  // unit-diagonal transform U = diag(1/T_kk) T, rows (1, u01, 1), (u10, 1, u10), (-1, 0, 1)
  V u01, u10;
  // middle row of the child-0 interpolation: y1 = pa x0 + pb x1 + pc x2
  V pa, pb, pc;
};

template <int DIM>
struct SfDim {
  static constexpr int NV = DIM == 2 ? 3 : (DIM == 3 ? 9 : 27);   // values per thread
  static constexpr int NPE = 3 * NV;
};

// Line operators on (a, b, c) along one axis, in place.
// U: 4 operations per line
template <typename V>
__device__ __forceinline__ void line_t(V &a, V &b, V &c, const SfCoef<V> &k)
{
  const V s = a + c;
  const V e0 = fma(k.u01, b, s), e1 = fma(k.u10, s, b), o = c - a;
  a = e0;
  b = e1;
  c = o;
}
// U^T: 4 operations per line
template <typename V>
__device__ __forceinline__ void line_tt(V &a, V &b, V &c, const SfCoef<V> &k)
{
  const V e = fma(k.u10, b, a), m = fma(k.u01, a, b);
  a = e - c;
  b = m;
  c = e + c;
}
// parent -> child (forward interpolation), child bit cb along this axis
template <typename V>
__device__ __forceinline__ void line_p(V &a, V &b, V &c, const SfCoef<V> &k, bool cb)
{
  const V y0 = cb ? b : a, y2 = cb ? c : b;
  const V y1 = fma(k.pc, cb ? a : c, fma(k.pb, b, k.pa * (cb ? c : a)));
  a = y0;
  b = y1;
  c = y2;
}
// child -> parent (transposed interpolation)
template <typename V>
__device__ __forceinline__ void line_pt(V &a, V &b, V &c, const SfCoef<V> &k, bool cb)
{
  const V lo = fma(k.pa, b, cb ? c : a), mid = fma(k.pb, b, cb ? a : c), hi = k.pc * b;
  a = cb ? hi : lo;
  b = mid;
  c = cb ? lo : hi;
}

// Two layouts of a leaf's 3^d values over its three threads.  Layout A:
// thread k holds the ranks k*NV + j, j < NV (last-axis digit k), so axes
// 0..d-2 are local; layout B: thread k holds the ranks k + 3 j (first-axis
// digit k), so axes 1..d-1 are local.  Every 1D operator is applied where
// its axis is local; the values change layout through a per-leaf buffer in
// shared memory.
template <int DIM, int AX, typename V, typename Op>
__device__ __forceinline__ void axis_a(V (&v)[SfDim<DIM>::NV], Op op)
{
  static_assert(AX >= 0 && AX <= DIM - 2, "axis not local in layout A");
  constexpr int s = AX == 0 ? 1 : (AX == 1 ? 3 : 9);
#pragma unroll
  for (int j = 0; j < SfDim<DIM>::NV; j++)
    if ((j / s) % 3 == 0) op(AX, v[j], v[j + s], v[j + 2 * s]);
}
template <int DIM, int AX, typename V, typename Op>
__device__ __forceinline__ void axis_b(V (&v)[SfDim<DIM>::NV], Op op)
{
  static_assert(AX >= 1 && AX <= DIM - 1, "axis not local in layout B");
  constexpr int s = AX == 1 ? 1 : (AX == 2 ? 3 : 9);
#pragma unroll
  for (int j = 0; j < SfDim<DIM>::NV; j++)
    if ((j / s) % 3 == 0) op(AX, v[j], v[j + s], v[j + 2 * s]);
}
template <int DIM, typename V, typename Op>
__device__ __forceinline__ void axes_a_all(V (&v)[SfDim<DIM>::NV], Op op)
{
  axis_a<DIM, 0>(v, op);
  if constexpr (DIM >= 3) axis_a<DIM, 1>(v, op);
  if constexpr (DIM >= 4) axis_a<DIM, 2>(v, op);
}
template <int DIM, typename V, typename Op>
__device__ __forceinline__ void axes_b_all(V (&v)[SfDim<DIM>::NV], Op op)
{
  axis_b<DIM, 1>(v, op);
  if constexpr (DIM >= 3) axis_b<DIM, 2>(v, op);
  if constexpr (DIM >= 4) axis_b<DIM, 3>(v, op);
}
// A -> B and B -> A through the leaf's buffer; idle lanes only synchronise.
template <int NV, typename V>
__device__ __forceinline__ void to_b(V (&v)[NV], V *buf, int k, bool act)
{
  if (act) {
#pragma unroll
    for (int j = 0; j < NV; j++) buf[k * NV + j] = v[j];
  }
  __syncwarp();
  if (act) {
#pragma unroll
    for (int j = 0; j < NV; j++) v[j] = buf[k + 3 * j];
  }
  __syncwarp();
}
template <int NV, typename V>
__device__ __forceinline__ void to_a(V (&v)[NV], V *buf, int k, bool act)
{
  if (act) {
#pragma unroll
    for (int j = 0; j < NV; j++) buf[k + 3 * j] = v[j];
  }
  __syncwarp();
  if (act) {
#pragma unroll
    for (int j = 0; j < NV; j++) v[j] = buf[k * NV + j];
  }
  __syncwarp();
}

// V = double: the FP64 product; V = float: the binary32 product (inner
// operator of the mixed-precision solver; plans without stale reads).
template <int DIM, typename V>
__global__ void __launch_bounds__(128, std::is_same<V, float>::value ? 6 : 3) k_matvec_q2sf(
    const int32_t *__restrict__ e2n, const uint32_t *__restrict__ info, const int32_t *__restrict__ hidx,
    const int32_t *__restrict__ p2n, const uint32_t *__restrict__ fill, const int32_t *__restrict__ order,
    int64_t n_leaf, SfCoef<V> cf, const V *__restrict__ Dtab, const V *__restrict__ x, V *__restrict__ y,
    V scale, const int32_t *__restrict__ hzoff, const int32_t *__restrict__ hztab,
    const double *__restrict__ stv, int conforming)
{
  constexpr int NV = SfDim<DIM>::NV, NPE = SfDim<DIM>::NPE;
  __shared__ V sbuf[4 * 10 * NPE];   // one buffer per leaf of the block (blockDim 128)
  const int lane = threadIdx.x & 31, slot = lane / 3, k = lane - 3 * slot;
  const int warp = threadIdx.x >> 5;
  const int64_t t = ((int64_t) blockIdx.x * 4 + warp) * 10 + slot;
  const bool act = slot < 10;                 // lanes 30, 31 are idle
  const bool valid = act && t < n_leaf;
  V *buf = sbuf + (warp * 10 + (act ? slot : 0)) * NPE;
  const int64_t i = valid ? (int64_t) order[t] : 0;
  const uint32_t inf = valid ? info[i] : 0u;
  const int L = inf & 0xFFu;
  const unsigned child = (inf >> 8) & 0xFFu;
  const bool hang = valid && ((inf >> 16) & 1u);

  // own values in layout B
  V u[NV];
  const int32_t *er = e2n + i * NPE;
#pragma unroll
  for (int j = 0; j < NV; j++) {
    const int32_t nd = valid ? er[k + 3 * j] : -1;
    u[j] = nd >= 0 ? x[nd] : V(0);
  }
  const bool any_h = __any_sync(0xffffffffu, hang);
  uint32_t fA = 0, fB = 0;   // fill bits of the thread's ranks in layout A and in layout B
  int64_t h = 0;
  if (any_h) {
    V v[NV];
    if (hang) {
      h = hidx[i];
      const uint32_t w0 = fill[h * 3], w1 = fill[h * 3 + 1], w2 = fill[h * 3 + 2];
      const int b0 = k * NV, sh = b0 & 31;   // ranks b0 .. b0+NV-1 lie in words b0>>5 and b0>>5 + 1
      const uint64_t two = (b0 >> 5) == 0 ? ((uint64_t) w0 | ((uint64_t) w1 << 32))
                                          : ((uint64_t) w1 | ((uint64_t) w2 << 32));
      fA = (uint32_t) (two >> sh) & ((1u << NV) - 1u);
#pragma unroll
      for (int j = 0; j < NV; j++) {
        const int r = k + 3 * j;
        const uint32_t w = r < 32 ? w0 : (r < 64 ? w1 : w2);
        fB |= ((w >> (r & 31)) & 1u) << j;
      }
      const int32_t hz = hzoff ? hzoff[h] : -1;   // slots read from the emulated static buffer
      const int32_t *pr = p2n + h * NPE + k * NV;
#pragma unroll
      for (int j = 0; j < NV; j++) {
        const int32_t pn = pr[j];
        V val = V(0);
        if (pn >= 0) val = x[pn];
        else if (hz >= 0) {
          const int32_t id = hztab[(int64_t) hz * NPE + k * NV + j];
          if (id >= 0) val = (V) stv[id];
        }
        v[j] = val;
      }
    } else {
#pragma unroll
      for (int j = 0; j < NV; j++) v[j] = V(0);
    }
    // parent -> child: axes 0..d-2 in layout A, the last axis in layout B
    auto ip = [&](int ax, V &a, V &b, V &c) { line_p(a, b, c, cf, (child >> ax) & 1u); };
    axes_a_all<DIM>(v, ip);
    to_b<NV>(v, buf, k, act);
    axis_b<DIM, DIM - 1>(v, ip);
    if (hang) {
#pragma unroll
      for (int j = 0; j < NV; j++)
        if (!((fB >> j) & 1u)) u[j] = v[j];
    }
  }
  // forward transform: axes 1..d-1 in B, axis 0 in A
  auto tf = [&](int, V &a, V &b, V &c) { line_t(a, b, c, cf); };
  axes_b_all<DIM>(u, tf);
  to_a<NV>(u, buf, k, act);
  axis_a<DIM, 0>(u, tf);
  // diagonal of level L (layout A: ranks k*NV + j)
  const V *Dl = Dtab + (int64_t) L * NPE + k * NV;
  if (scale == V(1)) {
#pragma unroll
    for (int j = 0; j < NV; j++) u[j] *= __ldg(Dl + j);
  } else {
#pragma unroll
    for (int j = 0; j < NV; j++) u[j] *= scale * __ldg(Dl + j);
  }
  // transposed transform: axes 0..d-2 in A, the last axis in B
  auto tt = [&](int, V &a, V &b, V &c) { line_tt(a, b, c, cf); };
  axes_a_all<DIM>(u, tt);
  to_b<NV>(u, buf, k, act);
  axis_b<DIM, DIM - 1>(u, tt);
  if (valid) {
#pragma unroll
    for (int j = 0; j < NV; j++) {
      const int32_t nd = er[k + 3 * j];
      if (nd >= 0) atomicAdd(y + nd, u[j]);
    }
  }
  if (any_h) {
    // zero the filled ranks, interpolate back to the parent (matvec.h:482-522):
    // axes 1..d-1 in B, axis 0 in A
#pragma unroll
    for (int j = 0; j < NV; j++)
      if (!hang || ((fB >> j) & 1u)) u[j] = V(0);
    auto pt = [&](int ax, V &a, V &b, V &c) { line_pt(a, b, c, cf, (child >> ax) & 1u); };
    axes_b_all<DIM>(u, pt);
    to_a<NV>(u, buf, k, act);
    axis_a<DIM, 0>(u, pt);
    if (hang) {
      const int32_t *pr = p2n + h * NPE + k * NV;
#pragma unroll
      for (int j = 0; j < NV; j++) {
        const int32_t pn = pr[j];
        // the reference masks parent slot q by the leaf's fill bit q
        if (pn >= 0 && (conforming || !((fA >> j) & 1u))) atomicAdd(y + pn, u[j]);
      }
    }
  }
}

// Leaf classes of the main launch: 0 hanging, 1 not hanging, 2 left out
// (reads stale slots, done after the chain when the product is split).
__global__ void k_leaf_class(const uint32_t *__restrict__ info, uint32_t *__restrict__ f0, uint32_t *__restrict__ f1,
                             int64_t n, int drop_stale)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t v = info[i];
  const bool out = drop_stale && ((v >> 27) & 1u);
  f0[i] = (!out && ((v >> 16) & 1u)) ? 1u : 0u;
  f1[i] = (!out && !((v >> 16) & 1u)) ? 1u : 0u;
}
// Stable order with the hanging leaves first: the scan of class 0, then n_h +
// the scan of class 1.
__global__ void k_order_hanging_first(const uint32_t *__restrict__ f0, const uint32_t *__restrict__ p0,
                                      const uint32_t *__restrict__ f1, const uint32_t *__restrict__ p1, int64_t n,
                                      int64_t n_h, int32_t *__restrict__ order)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (f0[i]) order[p0[i]] = (int32_t) i;
  else if (f1[i]) order[n_h + (int64_t) p1[i]] = (int32_t) i;
}

// Plan-time setup: the order-2 factors, the per-level diagonals D_L and the
// leaf order.  Returns false (dense kernel) for other orders, the identity
// and custom operators, or if the 1D operators lack the expected structure.
bool q2sf_setup(Plan &pl, cudaStream_t s)
{
  pl.sf_ready = false;
  const int k = pl.op.kind;
  if (pl.order != 2 || k == OP_IDENTITY || k == OP_CUSTOM || pl.n_leaf == 0) return false;
  double T[9], lam[3], pint[3];
  if (!q2_factors(T, lam, pint)) return false;
  const int dim = pl.dim, npe = pl.npe, nlev = pl.md + 1;
  // D_L[r] = alpha_L sum_t lam[digit_t(r)] + beta_L, times prod_t T_kk^2 for
  // the kernel's unit-diagonal transform U = diag(1/T_kk) T (so that
  // (x T)^T diag(D) (x T) = (x U)^T diag(D prod T_kk^2) (x U)).  T and lam are
  // checked against the dense tables of the plan's operator below.
  std::vector<double> D((size_t) nlev * npe);
  for (int l = 0; l < nlev; l++)
    for (int r = 0; r < npe; r++) {
      long double sl = 0.0L, f = 1.0L;
      int rr = r;
      for (int d = 0; d < dim; d++) {
        sl += lam[rr % 3];
        f *= (long double) T[(rr % 3) * 4] * T[(rr % 3) * 4];
        rr /= 3;
      }
      D[(size_t) l * npe + r] = (double) (((long double) pl.op.alpha[l] * sl + pl.op.beta[l]) * f);
    }
  {
    // (T x..x T)^T diag(D_0 unit) (T x..x T) against A and B separately
    std::vector<double> TT((size_t) npe * npe);
    for (int r = 0; r < npe; r++)
      for (int c = 0; c < npe; c++) {
        double v = 1.0;
        int rr = r, cc = c;
        for (int d = 0; d < dim; d++) { v *= T[(rr % 3) * 3 + (cc % 3)]; rr /= 3; cc /= 3; }
        TT[(size_t) r * npe + c] = v;
      }
    double err = 0.0, mx = 0.0;
    for (int term = 0; term < 2; term++) {
      const std::vector<double> &coef = term == 0 ? pl.op.alpha : pl.op.beta;
      if (std::all_of(coef.begin(), coef.end(), [](double c) { return c == 0.0; })) continue;   // term unused
      const std::vector<double> &ref = term == 0 ? pl.op.A : pl.op.B;
      for (int r = 0; r < npe; r++)
        for (int c = 0; c < npe; c++) {
          double v = 0.0;
          for (int m = 0; m < npe; m++) {
            double dm = 1.0;
            if (term == 0) {
              dm = 0.0;
              int mm = m;
              for (int d = 0; d < dim; d++) { dm += lam[mm % 3]; mm /= 3; }
            }
            v += TT[(size_t) m * npe + r] * dm * TT[(size_t) m * npe + c];
          }
          const double want = ref[(size_t) r * npe + c];
          err = std::max(err, std::fabs(v - want));
          mx = std::max(mx, std::fabs(want));
        }
    }
    if (!(err <= 1e-13 * mx)) return false;
  }
  pl.sf_D.upload(D.data(), D.size(), s);
  {
    std::vector<float> D32(D.begin(), D.end());
    pl.sf_D32.upload(D32.data(), D32.size(), s);
  }
  std::copy(T, T + 9, pl.sf_T);
  std::copy(pint, pint + 3, pl.sf_pint);
  // With stale parent reads the chain runs on a side stream during the main
  // launch, which leaves out the leaves that read its values.
  pl.sf_split = pl.st_ready && pl.st_n_runs > 0 && pl.st_n_hleaf > 0;
  DBuf<uint32_t> f0(pl.n_leaf), p0(pl.n_leaf), f1(pl.n_leaf), p1(pl.n_leaf);
  k_leaf_class<<<grid_for(pl.n_leaf), 256, 0, s>>>(pl.info.p, f0.p, f1.p, pl.n_leaf, pl.sf_split ? 1 : 0);
  const int64_t nh = (int64_t) exclusive_scan_total<uint32_t>(f0.p, p0.p, pl.n_leaf, s);
  const int64_t nn = (int64_t) exclusive_scan_total<uint32_t>(f1.p, p1.p, pl.n_leaf, s);
  pl.sf_n_main = nh + nn;
  if (pl.sf_n_main + (pl.sf_split ? pl.st_n_hleaf : 0) != pl.n_leaf) throw std::runtime_error("q2sf leaf classes");
  pl.sf_order.alloc(std::max<int64_t>(pl.sf_n_main, 1));
  k_order_hanging_first<<<grid_for(pl.n_leaf), 256, 0, s>>>(f0.p, p0.p, f1.p, p1.p, pl.n_leaf, nh, pl.sf_order.p);
  check_launch("q2sf_order");
  DKT_CUDA(cudaStreamSynchronize(s));
  pl.sf_ready = true;
  // the binary32 product (inner operator of the mixed solver) needs no stale reads
  pl.f32_ready = !pl.st_ready || pl.st_n_runs == 0;
  return true;
}

template <typename V> static const V *sf_table(const Plan &pl);
template <> const double *sf_table<double>(const Plan &pl) { return pl.sf_D.p; }
template <> const float *sf_table<float>(const Plan &pl) { return pl.sf_D32.p; }

// stale: the launch covers leaves that may read stale slots
template <int DIM, typename V>
static void launch_sf(Plan &pl, const int32_t *order, int64_t n, const V *x, V *y, double scale, bool stale,
                      cudaStream_t s)
{
  if (n == 0) return;
  SfCoef<V> cf;
  cf.u01 = (V) (pl.sf_T[1] / pl.sf_T[0]);
  cf.u10 = (V) (pl.sf_T[3] / pl.sf_T[4]);
  cf.pa = (V) pl.sf_pint[0]; cf.pb = (V) pl.sf_pint[1]; cf.pc = (V) pl.sf_pint[2];
  const bool fp64 = std::is_same<V, double>::value;
  const int64_t per_block = 4 * 10;   // 4 warps of 10 leaves
  const unsigned blocks = (unsigned) ((n + per_block - 1) / per_block);
  k_matvec_q2sf<DIM, V><<<blocks, 128, 0, s>>>(pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.fill.p, order,
                                               n, cf, sf_table<V>(pl), x, y, (V) (pl.op.uses_scale ? scale : 1.0),
                                               (fp64 && stale && pl.st_ready) ? pl.st_hzoff.p : nullptr, pl.st_hztab.p,
                                               pl.st_v.p, pl.conforming ? 1 : 0);
  check_launch("matvec_q2sf");
}

template <typename V>
static void launch_sf_dim(Plan &pl, const int32_t *order, int64_t n, const V *x, V *y, double scale, bool stale,
                          cudaStream_t s)
{
  switch (pl.dim) {
    case 2: launch_sf<2, V>(pl, order, n, x, y, scale, stale, s); break;
    case 3: launch_sf<3, V>(pl, order, n, x, y, scale, stale, s); break;
    case 4: launch_sf<4, V>(pl, order, n, x, y, scale, stale, s); break;
    default: throw std::runtime_error("unsupported dim");
  }
  if (n > 0) pl.n_launch++;
}

// Binary32 product y = A x (y zeroed here), the order-2 counterpart of the
// Q1 binary32 kernels: same leaf order, float values, float atomics.
void q2sf_f32(Plan &pl, const float *x, float *y, cudaStream_t s)
{
  if (!pl.sf_ready || !pl.f32_ready) throw std::runtime_error("binary32 Q2 product needs a plan without stale reads");
  DKT_CUDA(cudaMemsetAsync(y, 0, pl.n_nodes * sizeof(float), s));
  launch_sf_dim<float>(pl, pl.sf_order.p, pl.sf_n_main, x, y, 1.0, false, s);
}

void stale_eval(Plan &pl, const double *x, const long long *xq, cudaStream_t s);
void ensure_side_stream(Plan &pl);

// fem::matvec with the sum-factorised kernel; y has been zeroed.  With stale
// parent reads, the static-buffer chain runs on the high-priority side stream
// while the main launch does every leaf that does not read its values; those
// leaves follow once the chain has joined.  Only the main launch is timed.
void q2sf_matvec(Plan &pl, const double *x, double *y, double scale, cudaStream_t s)
{
  if (pl.sf_split) {
    ensure_side_stream(pl);
    DKT_CUDA(cudaEventRecord(pl.st_fork, s));
    DKT_CUDA(cudaStreamWaitEvent(pl.st_stream, pl.st_fork, 0));
    stale_eval(pl, x, nullptr, pl.st_stream);
    DKT_CUDA(cudaEventRecord(pl.st_join, pl.st_stream));
  } else {
    stale_eval(pl, x, nullptr, s);
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (pl.timing) {
    DKT_CUDA(cudaEventCreate(&e0));
    DKT_CUDA(cudaEventCreate(&e1));
    DKT_CUDA(cudaEventRecord(e0, s));
  }
  // split: the main launch leaves out every leaf that reads stale slots
  launch_sf_dim<double>(pl, pl.sf_order.p, pl.sf_n_main, x, y, scale, !pl.sf_split, s);
  if (pl.timing) {
    DKT_CUDA(cudaEventRecord(e1, s));
    pl.ev.push_back(e0);
    pl.ev.push_back(e1);
    pl.timed_launches++;
  }
  if (pl.sf_split) {
    DKT_CUDA(cudaStreamWaitEvent(s, pl.st_join, 0));
    launch_sf_dim<double>(pl, pl.st_hleaves.p, pl.st_n_hleaf, x, y, scale, true, s);
  }
}

}  // namespace dkt
