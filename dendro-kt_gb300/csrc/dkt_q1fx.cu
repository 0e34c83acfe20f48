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
#include <cmath>
#include "dkt_internal.cuh"

namespace dkt {

__device__ __forceinline__ long long mulshift(long long v, long long m, int e)
{
  // floor(v * m / 2^e) with a 128-bit intermediate, 1 <= e <= 126
  const long long hi = __mul64hi(v, m);
  const unsigned long long lo = (unsigned long long) v * (unsigned long long) m;
  if (e >= 64) return hi >> (e - 64);
  return (long long) ((lo >> e) | ((unsigned long long) hi << (64 - e)));
}

// In-place Walsh-Hadamard transform over DIM axes (rank bit d = axis d).
template <int DIM>
__device__ __forceinline__ void wht(long long *u)
{
  constexpr int NPE = 1 << DIM;
#pragma unroll
  for (int d = 0; d < DIM; d++) {
#pragma unroll
    for (int r = 0; r < NPE; r++) {
      if (r & (1 << d)) continue;
      const long long a = u[r], b = u[r | (1 << d)];
      u[r] = a + b;
      u[r | (1 << d)] = a - b;
    }
  }
}

// Parent -> child interpolation of Q1 (IKD_Parent2Child with ip_1D_{0,1}):
// along an axis where the child bit is 0, child node 0 takes parent node 0
// and child node 1 the mean; mirrored when the bit is 1.
template <int DIM>
__device__ __forceinline__ void p2c(long long *v, unsigned child)
{
  constexpr int NPE = 1 << DIM;
#pragma unroll
  for (int d = 0; d < DIM; d++) {
    const bool hi = (child >> d) & 1u;
#pragma unroll
    for (int r = 0; r < NPE; r++) {
      if (r & (1 << d)) continue;
      const long long a = v[r], b = v[r | (1 << d)];
      const long long m = (a + b) >> 1;
      if (hi) v[r] = m; else v[r | (1 << d)] = m;
    }
  }
}

// Transpose (IKD_Child2Parent with ipT_1D_{0,1}).
template <int DIM>
__device__ __forceinline__ void c2p(long long *v, unsigned child)
{
  constexpr int NPE = 1 << DIM;
#pragma unroll
  for (int d = 0; d < DIM; d++) {
    const bool hi = (child >> d) & 1u;
#pragma unroll
    for (int r = 0; r < NPE; r++) {
      if (r & (1 << d)) continue;
      const long long a = v[r], b = v[r | (1 << d)];
      if (hi) { v[r] = a >> 1; v[r | (1 << d)] = b + (a >> 1); }
      else { v[r] = a + (b >> 1); v[r | (1 << d)] = b >> 1; }
    }
  }
}

template <int DIM>
__global__ void __launch_bounds__(256) k_matvec_q1fx(
    const int32_t *__restrict__ e2n, const uint32_t *__restrict__ info, const int32_t *__restrict__ hidx,
    const int32_t *__restrict__ p2n, const uint32_t *__restrict__ fill, int64_t n_leaf, int64_t n_hang,
    const long long *__restrict__ fm, const int *__restrict__ fe, const long long *__restrict__ xq,
    unsigned long long *__restrict__ yq)
{
  constexpr int NPE = 1 << DIM;
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_leaf) return;
  const uint32_t inf = info[i];
  const int L = inf & 0xFFu;
  const unsigned child = (inf >> 8) & 0xFFu;
  const bool hang = (inf >> 16) & 1u;
  long long u[NPE];
  int32_t nd[NPE];
#pragma unroll
  for (int r = 0; r < NPE; r++) {
    nd[r] = e2n[(int64_t) r * n_leaf + i];
    u[r] = nd[r] >= 0 ? __ldg(xq + nd[r]) : 0ll;
  }
  int64_t h = 0;
  uint32_t fmask = 0;
  if (hang) {
    h = hidx[i];
    fmask = fill[h];
    long long xp[NPE];
#pragma unroll
    for (int q = 0; q < NPE; q++) {
      const int32_t pn = p2n[(int64_t) q * n_hang + h];
      xp[q] = pn >= 0 ? __ldg(xq + pn) : 0ll;
    }
    p2c<DIM>(xp, child);
#pragma unroll
    for (int r = 0; r < NPE; r++)
      if (!((fmask >> r) & 1u)) u[r] = xp[r];
  }
  wht<DIM>(u);
#pragma unroll
  for (int s = 0; s < NPE; s++) u[s] = mulshift(u[s], fm[L * NPE + s], fe[L * NPE + s]);
  wht<DIM>(u);
#pragma unroll
  for (int r = 0; r < NPE; r++)
    if (nd[r] >= 0) atomicAdd(yq + nd[r], (unsigned long long) u[r]);
  if (hang) {
#pragma unroll
    for (int r = 0; r < NPE; r++)
      if ((fmask >> r) & 1u) u[r] = 0;
    c2p<DIM>(u, child);
#pragma unroll
    for (int q = 0; q < NPE; q++) {
      const int32_t pn = p2n[(int64_t) q * n_hang + h];
      if (pn >= 0 && !((fmask >> q) & 1u)) atomicAdd(yq + pn, (unsigned long long) u[q]);
    }
  }
}

// max |x| (as the bit pattern of a non-negative double, so integer atomicMax orders it)
__global__ void k_absmax(const double *__restrict__ x, int64_t n, unsigned long long *__restrict__ out)
{
  double m = 0.0;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x)
    m = fmax(m, fabs(x[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long) __double_as_longlong(m));
}

// xq = round(x * 2^sx), sx from max|x| (device scalar); boundary entries zeroed
// when ids are given (feMatrix pre-matvec).
__global__ void k_to_fixed(const double *__restrict__ x, long long *__restrict__ xq, int64_t n,
                           const unsigned long long *__restrict__ amax, int *__restrict__ sx_out, int dim)
{
  const double m = __longlong_as_double((long long) *amax);
  int e = 0;
  if (m > 0.0) frexp(m, &e);   // m < 2^e
  const int sx = (60 - dim) - e;
  if (blockIdx.x == 0 && threadIdx.x == 0) *sx_out = sx;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x)
    xq[i] = __double2ll_rn(ldexp(x[i], sx));
}

__global__ void k_from_fixed(const long long *__restrict__ yq, double *__restrict__ y, int64_t n,
                             const int *__restrict__ sx, int c)
{
  const int sh = -(*sx + c);
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x)
    y[i] = ldexp((double) yq[i], sh);
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

// Host setup of the per-(level, mode) factors.  Returns false when the
// operator is not one of the diagonalisable Q1 built-ins.
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
  int emax = 0;
  std::frexp(maxD, &emax);                    // maxD < 2^emax
  const int c = -6 - dim - emax;             // max factor < 2^(-6-dim)
  std::vector<long long> fm((size_t) nlev * NPE);
  std::vector<int> fe((size_t) nlev * NPE);
  for (size_t k = 0; k < D.size(); k++) {
    const double f = std::ldexp(D[k], c);
    if (f == 0.0) { fm[k] = 0; fe[k] = 1; continue; }
    int ef = 0;
    std::frexp(f, &ef);                       // f < 2^ef, ef <= -6-dim
    const int e = 62 - ef;                    // fm = f * 2^e < 2^62
    fe[k] = std::min(e, 126);
    fm[k] = (long long) std::llround(std::ldexp(f, fe[k]));
  }
  pl.fx_c = c;
  pl.fx_fm.upload(fm.data(), fm.size(), s);
  pl.fx_fe.upload(fe.data(), fe.size(), s);
  pl.xq.alloc(pl.n_nodes);
  pl.yq.alloc(pl.n_nodes);
  pl.fx_amax.alloc(1);
  pl.fx_sx.alloc(1);
  pl.fx_ready = true;
  return true;
}

template <int DIM>
static void launch_q1fx(Plan &pl, cudaStream_t s)
{
  const unsigned threads = 256;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (pl.timing) {
    DKT_CUDA(cudaEventCreate(&e0));
    DKT_CUDA(cudaEventCreate(&e1));
    DKT_CUDA(cudaEventRecord(e0, s));
  }
  k_matvec_q1fx<DIM><<<grid_for(pl.n_leaf, threads), threads, 0, s>>>(
      pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.fill.p, pl.n_leaf, pl.n_hang, pl.fx_fm.p, pl.fx_fe.p,
      (const long long *) pl.xq.p, (unsigned long long *) pl.yq.p);
  check_launch("matvec_q1fx");
  if (pl.timing) {
    DKT_CUDA(cudaEventRecord(e1, s));
    pl.ev.push_back(e0);
    pl.ev.push_back(e1);
    pl.timed_launches++;
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
void q1fx_matvec(Plan &pl, const double *x, double *y, double scale, bool bc, cudaStream_t s)
{
  const int64_t n = pl.n_nodes;
  DKT_CUDA(cudaMemsetAsync(pl.fx_amax.p, 0, sizeof(unsigned long long), s));
  k_absmax<<<608, 256, 0, s>>>(x, n, pl.fx_amax.p);
  k_to_fixed<<<608, 256, 0, s>>>(x, pl.xq.p, n, pl.fx_amax.p, pl.fx_sx.p, pl.dim);
  check_launch("to_fixed");
  if (bc && pl.n_bdry > 0) {
    k_zero_ids_ll<<<grid_for(pl.n_bdry), 256, 0, s>>>(pl.xq.p, pl.bdry.p, pl.n_bdry);
    check_launch("zero_in");
  }
  DKT_CUDA(cudaMemsetAsync(pl.yq.p, 0, n * sizeof(long long), s));
  switch (pl.dim) {
    case 2: launch_q1fx<2>(pl, s); break;
    case 3: launch_q1fx<3>(pl, s); break;
    case 4: launch_q1fx<4>(pl, s); break;
    default: throw std::runtime_error("unsupported dim");
  }
  k_from_fixed<<<608, 256, 0, s>>>(pl.yq.p, y, n, pl.fx_sx.p, pl.fx_c);
  check_launch("from_fixed");
  if (bc && pl.n_bdry > 0) {
    k_zero_ids_d<<<grid_for(pl.n_bdry), 256, 0, s>>>(y, pl.bdry.p, pl.n_bdry);
    check_launch("zero_out");
  }
  if (scale != 1.0 && pl.op.uses_scale) {
    // the built-in operators are linear in scale
    scale_vector(y, n, scale, s);
  }
}

}  // namespace dkt
