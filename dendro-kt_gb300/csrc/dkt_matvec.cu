// Fused leaf kernel of the flattened fem::matvec (FEM/include/matvec.h:368-528):
// per leaf visit it gathers the element's nodal values (matvec.h:380-400),
// interpolates missing ranks from the parent's level-(L-1) nodes with
// IKD_Parent2Child (matvec.h:402-457, FEM/include/refel.h:214-238), applies the
// elemental operator (eleOp, matvec.h:467-468), scatter-adds the outputs to the
// element's nodes (the leaf copy-out plus bottom_up, matvec.h:470-480, 202-216),
// and for hanging leaves zeroes the filled ranks, applies IKD_Child2Parent and
// adds the result to the parent nodes whose rank is unfilled in the leaf mask
// (matvec.h:482-522).
#include <mutex>
#include <string>
#include "dkt_internal.cuh"

namespace dkt {

template <int DIM, int M>
struct Pow {
  static constexpr int v = M * Pow<DIM - 1, M>::v;
};
template <int M>
struct Pow<0, M> {
  static constexpr int v = 1;
};

// In-place tensor apply of the child interpolation along every axis.
// forward:   y_j = sum_k ip[k*M + j] x_k   (parent -> child)
// transpose: y_j = sum_k ip[j*M + k] x_k   (child -> parent)
template <int DIM, int M, bool TRANSPOSE>
__host__ __device__ __forceinline__ void interp(double *v, const double *__restrict__ ip, unsigned child)
{
  constexpr int NPE = Pow<DIM, M>::v;
  constexpr int UR = NPE <= 16 ? NPE : 1;
#pragma unroll
  for (int d = 0; d < DIM; d++) {
    const double *A = ip + ((child >> d) & 1u) * M * M;
    int stride = 1;
#pragma unroll
    for (int a = 0; a < d; a++) stride *= M;
    double t[NPE];
#pragma unroll UR
    for (int idx = 0; idx < NPE; idx++) {
      const int j = (idx / stride) % M;
      const int base = idx - j * stride;
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < M; k++) s += (TRANSPOSE ? A[j * M + k] : A[k * M + j]) * v[base + k * stride];
      t[idx] = s;
    }
#pragma unroll UR
    for (int idx = 0; idx < NPE; idx++) v[idx] = t[idx];
  }
}

__host__ __device__ __forceinline__ void accum(double *p, double v)
{
#ifdef __CUDA_ARCH__
  atomicAdd(p, v);
#else
  *p += v;
#endif
}

// One leaf visit: gather, parent interpolation, elemental operator, scatter
// and the hanging transpose.  sA/sB/sip point at the staged operator and
// interpolation tables.
template <int DIM, int P, bool CUSTOM>
__host__ __device__ __forceinline__ void leaf_body(
    int64_t i, const int32_t *__restrict__ e2n, const uint32_t *__restrict__ info, const int32_t *__restrict__ hidx,
    const int32_t *__restrict__ p2n, const uint32_t *__restrict__ fill, int64_t n_leaf, int64_t n_hang,
    const double *sA, const double *sB, const double *__restrict__ alpha, const double *__restrict__ beta,
    const double *__restrict__ table, const double *sip, const double *__restrict__ x, double *__restrict__ y,
    double scale, const int32_t *__restrict__ hzoff, const int32_t *__restrict__ hztab,
    const double *__restrict__ stv, int conforming)
{
  constexpr int M = P + 1, NPE = Pow<DIM, M>::v;
  constexpr int UR = NPE <= 16 ? NPE : 1;
  const uint32_t inf = info[i];
  const int L = inf & 0xFFu;
  const unsigned child = (inf >> 8) & 0xFFu;
  const bool hang = (inf >> 16) & 1u;
  double u[NPE];
  int32_t nd[NPE];
#pragma unroll UR
  for (int r = 0; r < NPE; r++) {
    nd[r] = e2n[(int64_t) i * NPE + r];
    u[r] = nd[r] >= 0 ? x[nd[r]] : 0.0;
  }
  int64_t h = 0;
  uint32_t fm[3] = {0, 0, 0};
  if (hang) {
    h = hidx[i];
    for (int w = 0; w < 3; w++) fm[w] = fill[(int64_t) h * 3 + w];
    double xp[NPE];
    const int32_t hz = hzoff ? hzoff[h] : -1;   // slots this leaf reads from the static buffer
#pragma unroll UR
    for (int q = 0; q < NPE; q++) {
      const int32_t pn = p2n[(int64_t) h * NPE + q];
      double v = 0.0;
      if (pn >= 0) v = x[pn];
      else if (hz >= 0) {
        const int32_t id = hztab[(int64_t) hz * NPE + q];
        if (id >= 0) v = stv[id];
      }
      xp[q] = v;
    }
    interp<DIM, M, false>(xp, sip, child);
#pragma unroll UR
    for (int r = 0; r < NPE; r++)
      if (!((fm[r >> 5] >> (r & 31)) & 1u)) u[r] = xp[r];
  }
  double out[NPE];
  if (CUSTOM) {
    const double *K = table + (int64_t) L * NPE * NPE;
#pragma unroll UR
    for (int r = 0; r < NPE; r++) {
      double s = 0.0;
#pragma unroll UR
      for (int c = 0; c < NPE; c++) s += K[r * NPE + c] * u[c];
      out[r] = scale * s;
    }
  } else {
    const double a = alpha[L] * scale, b = beta[L] * scale;
#pragma unroll UR
    for (int r = 0; r < NPE; r++) {
      double sa = 0.0, sb = 0.0;
#pragma unroll UR
      for (int c = 0; c < NPE; c++) { sa += sA[r * NPE + c] * u[c]; sb += sB[r * NPE + c] * u[c]; }
      out[r] = a * sa + b * sb;
    }
  }
#pragma unroll UR
  for (int r = 0; r < NPE; r++)
    if (nd[r] >= 0) accum(&y[nd[r]], out[r]);
  if (hang) {
#pragma unroll UR
    for (int r = 0; r < NPE; r++)
      if ((fm[r >> 5] >> (r & 31)) & 1u) out[r] = 0.0;
    interp<DIM, M, true>(out, sip, child);
#pragma unroll UR
    for (int q = 0; q < NPE; q++) {
      const int32_t pn = p2n[(int64_t) h * NPE + q];
      if (pn >= 0 && (conforming || !((fm[q >> 5] >> (q & 31)) & 1u))) accum(&y[pn], out[q]);
    }
  }
}

template <int DIM, int P, bool CUSTOM>
__global__ void __launch_bounds__(128) k_matvec_leaf(
    const int32_t *__restrict__ e2n, const uint32_t *__restrict__ info, const int32_t *__restrict__ hidx,
    const int32_t *__restrict__ p2n, const uint32_t *__restrict__ fill, int64_t n_leaf, int64_t n_hang,
    const double *__restrict__ gA, const double *__restrict__ gB, const double *__restrict__ alpha,
    const double *__restrict__ beta, const double *__restrict__ table, const double *__restrict__ gip,
    const double *__restrict__ x, double *__restrict__ y, double scale, const int32_t *__restrict__ hzoff,
    const int32_t *__restrict__ hztab, const double *__restrict__ stv, int conforming)
{
  constexpr int M = P + 1, NPE = Pow<DIM, M>::v;
  constexpr int UR = NPE <= 16 ? NPE : 1;
  extern __shared__ double sm[];
  // custom operators keep no A/B in shared memory: the interpolation tables
  // then start at the beginning of the dynamic allocation
  double *sA = sm, *sB = sm + NPE * NPE, *sip = CUSTOM ? sm : sm + 2 * NPE * NPE;
  if (!CUSTOM) {
    for (int t = threadIdx.x; t < NPE * NPE; t += blockDim.x) { sA[t] = gA[t]; sB[t] = gB[t]; }
  }
  for (int t = threadIdx.x; t < 2 * M * M; t += blockDim.x) sip[t] = gip[t];
  __syncthreads();
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_leaf) return;
  leaf_body<DIM, P, CUSTOM>(i, e2n, info, hidx, p2n, fill, n_leaf, n_hang, sA, sB, alpha, beta, table, sip, x, y,
                            scale, hzoff, hztab, stv, conforming);
}

__global__ void k_zero_at(double *__restrict__ v, const uint32_t *__restrict__ ids, int64_t nb)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nb) v[ids[i]] = 0.0;
}

#define ST_ARGS (pl.st_ready ? pl.st_hzoff.p : nullptr), pl.st_hztab.p, pl.st_v.p, (pl.conforming ? 1 : 0)

void stale_eval(Plan &pl, const double *x, const long long *xq, cudaStream_t s);

template <int DIM, int P>
static void launch_leaf(Plan &pl, const double *x, double *y, double scale, cudaStream_t s)
{
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (pl.timing) {
    DKT_CUDA(cudaEventCreate(&e0));
    DKT_CUDA(cudaEventCreate(&e1));
    DKT_CUDA(cudaEventRecord(e0, s));
  }
  constexpr int M = P + 1, NPE = Pow<DIM, M>::v;
  const bool custom = pl.op.kind == OP_CUSTOM;
  const size_t smem = (size_t) (custom ? 0 : 2 * NPE * NPE) * sizeof(double) + 2 * M * M * sizeof(double) + 16;
  const unsigned threads = 128;
  const unsigned blocks = grid_for(pl.n_leaf, threads);
  if (custom) {
    auto kfn = k_matvec_leaf<DIM, P, true>;
    kfn<<<blocks, threads, smem, s>>>(pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.fill.p, pl.n_leaf, pl.n_hang,
                                      nullptr, nullptr, nullptr, nullptr, pl.opTable.p, pl.ip.p, x, y, scale, ST_ARGS);
  } else {
    auto kfn = k_matvec_leaf<DIM, P, false>;
    ensure_dyn_smem(kfn, smem);
    kfn<<<blocks, threads, smem, s>>>(pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.fill.p, pl.n_leaf, pl.n_hang,
                                      pl.opA.p, pl.opB.p, pl.opAlpha.p, pl.opBeta.p, nullptr, pl.ip.p, x, y,
                                      pl.op.uses_scale ? scale : 1.0, ST_ARGS);
  }
  check_launch("matvec_leaf");
  pl.n_launch++;
  if (pl.timing) {
    DKT_CUDA(cudaEventRecord(e1, s));
    pl.ev.push_back(e0);
    pl.ev.push_back(e1);
    pl.timed_launches++;
  }
}

void q1fx_matvec(Plan &pl, const double *x, double *y, double scale, bool bc, cudaStream_t s);
void q2sf_matvec(Plan &pl, const double *x, double *y, double scale, cudaStream_t s);

// fem::matvec: y = 0, then the leaf kernel.
void matvec(Plan &pl, const double *x, double *y, double scale, cudaStream_t s)
{
  if (pl.fx_ready && pl.arith != 1) { q1fx_matvec(pl, x, y, scale, false, s); return; }
  DKT_CUDA(cudaMemsetAsync(y, 0, pl.n_nodes * sizeof(double), s));
  if (pl.n_leaf == 0) return;
  if (pl.sf_ready && pl.arith != 1) { q2sf_matvec(pl, x, y, scale, s); return; }
  stale_eval(pl, x, nullptr, s);
  switch (pl.dim * 10 + pl.order) {
    case 21: launch_leaf<2, 1>(pl, x, y, scale, s); break;
    case 22: launch_leaf<2, 2>(pl, x, y, scale, s); break;
    case 31: launch_leaf<3, 1>(pl, x, y, scale, s); break;
    case 32: launch_leaf<3, 2>(pl, x, y, scale, s); break;
    case 41: launch_leaf<4, 1>(pl, x, y, scale, s); break;
    case 42: launch_leaf<4, 2>(pl, x, y, scale, s); break;
    default: throw std::runtime_error("unsupported dim/order");
  }
}

// feMatrix::matVec: boundary-zeroed input copy, matvec, boundary-zeroed output
// (HeatMat::preMatVec/postMatVec) for the operators that have them.
void fematrix_matvec(Plan &pl, const double *x, double *y, double scale, cudaStream_t s)
{
  const bool bc = op_has_bc(pl.op.kind);
  if (pl.fx_ready && pl.arith != 1) { q1fx_matvec(pl, x, y, scale, bc, s); return; }
  if (!bc) { matvec(pl, x, y, scale, s); return; }
  if (pl.xin.n < (size_t) pl.n_nodes) pl.xin.alloc(pl.n_nodes);
  DKT_CUDA(cudaMemcpyAsync(pl.xin.p, x, pl.n_nodes * sizeof(double), cudaMemcpyDeviceToDevice, s));
  if (pl.n_bdry > 0) {
    k_zero_at<<<grid_for(pl.n_bdry), 256, 0, s>>>(pl.xin.p, pl.bdry.p, pl.n_bdry);
    check_launch("zero_bdry_in");
    pl.n_launch++;
  }
  matvec(pl, pl.xin.p, y, scale, s);
  if (pl.n_bdry > 0) {
    k_zero_at<<<grid_for(pl.n_bdry), 256, 0, s>>>(y, pl.bdry.p, pl.n_bdry);
    check_launch("zero_bdry_out");
    pl.n_launch++;
  }
}

// ---------------------------------------------------------------------------
// feMatrix::matVec without any device allocation.
//
// Some callers cannot let a matrix-vector product allocate device memory:
// a solver or serving loop that has reserved its whole device-memory budget
// up front (an allocation inside a request would break that accounting, or
// fail under memory pressure), and host code that must not stall the device
// (cudaMalloc and cudaFree can synchronise it).  For them this variant keeps
// its only scratch -- the boundary-zeroed copy of the input vector that the
// regular path allocates inside the plan -- in a fixed array in device global
// memory that every GPU loading this library holds until the process exits.
// ---------------------------------------------------------------------------
constexpr int64_t NOALLOC_MAX_NODES = int64_t(1) << 20;   // 1,048,576 doubles = 8 MiB per device
static __device__ __align__(256) double g_noalloc_xin[NOALLOC_MAX_NODES];

constexpr int NOALLOC_MAX_DEVICES = 64;
static double *g_noalloc_ptr[NOALLOC_MAX_DEVICES];   // device address of the array, per device
static cudaError_t g_noalloc_err[NOALLOC_MAX_DEVICES];
static std::once_flag g_noalloc_once[NOALLOC_MAX_DEVICES];

// The array's name is only a host-side handle; its device address is looked
// up once per device, with that device current.  Host threads that make
// their first call on a device at the same time wait for one lookup.
static cudaError_t noalloc_scratch(double **out)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
  std::call_once(g_noalloc_once[dev], [dev]() {
    void *p = nullptr;
    g_noalloc_err[dev] = cudaGetSymbolAddress(&p, g_noalloc_xin);
    g_noalloc_ptr[dev] = static_cast<double *>(p);
  });
  if (g_noalloc_err[dev] != cudaSuccess) return g_noalloc_err[dev];
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

template <int DIM, int P>
static void launch_leaf_noalloc(const Plan &pl, const double *x, double *y, double scale, cudaStream_t s)
{
  constexpr int M = P + 1, NPE = Pow<DIM, M>::v;
  const bool custom = pl.op.kind == OP_CUSTOM;
  const size_t smem = (size_t) (custom ? 0 : 2 * NPE * NPE) * sizeof(double) + 2 * M * M * sizeof(double) + 16;
  const unsigned threads = 128, blocks = grid_for(pl.n_leaf, threads);
  if (custom) {
    k_matvec_leaf<DIM, P, true><<<blocks, threads, smem, s>>>(pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.fill.p,
                                                              pl.n_leaf, pl.n_hang, nullptr, nullptr, nullptr, nullptr,
                                                              pl.opTable.p, pl.ip.p, x, y, scale, ST_ARGS);
  } else {
    auto kfn = k_matvec_leaf<DIM, P, false>;
    ensure_dyn_smem(kfn, smem);
    kfn<<<blocks, threads, smem, s>>>(pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.fill.p, pl.n_leaf, pl.n_hang,
                                      pl.opA.p, pl.opB.p, pl.opAlpha.p, pl.opBeta.p, nullptr, pl.ip.p, x, y,
                                      pl.op.uses_scale ? scale : 1.0, ST_ARGS);
  }
  check_launch("matvec_leaf_noalloc");
}

// Returns NOALLOC_OK, NOALLOC_TOO_LARGE (a plan beyond the fixed scratch, or
// an unsupported shape) or NOALLOC_CUDA, with the reason in err.
int fematrix_matvec_noalloc(const Plan &pl, const double *x, double *y, double scale, cudaStream_t s,
                            std::string &err)
{
  if (pl.n_nodes > NOALLOC_MAX_NODES) {
    err = "dkt_fematrix_matvec_noalloc: " + std::to_string(pl.n_nodes) + " nodes exceed its fixed scratch of " +
          std::to_string(NOALLOC_MAX_NODES) + " nodes";
    return NOALLOC_TOO_LARGE;
  }
  double *scratch = nullptr;
  cudaError_t e = noalloc_scratch(&scratch);
  if (e != cudaSuccess) {
    err = std::string("dkt_fematrix_matvec_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
    return NOALLOC_CUDA;
  }
  const bool bc = op_has_bc(pl.op.kind);
  const double *xin = x;
  if (bc) {
    // every entry that the kernel reads is overwritten here; nothing of the
    // previous call's contents survives into this one
    DKT_CUDA(cudaMemcpyAsync(scratch, x, pl.n_nodes * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (pl.n_bdry > 0) {
      k_zero_at<<<grid_for(pl.n_bdry), 256, 0, s>>>(scratch, pl.bdry.p, pl.n_bdry);
      check_launch("noalloc_zero_in");
    }
    xin = scratch;
  }
  DKT_CUDA(cudaMemsetAsync(y, 0, pl.n_nodes * sizeof(double), s));
  if (pl.n_leaf > 0) {
    stale_eval(const_cast<Plan &>(pl), xin, nullptr, s);
    switch (pl.dim * 10 + pl.order) {
      case 21: launch_leaf_noalloc<2, 1>(pl, xin, y, scale, s); break;
      case 22: launch_leaf_noalloc<2, 2>(pl, xin, y, scale, s); break;
      case 31: launch_leaf_noalloc<3, 1>(pl, xin, y, scale, s); break;
      case 32: launch_leaf_noalloc<3, 2>(pl, xin, y, scale, s); break;
      case 41: launch_leaf_noalloc<4, 1>(pl, xin, y, scale, s); break;
      case 42: launch_leaf_noalloc<4, 2>(pl, xin, y, scale, s); break;
      default: err = "dkt_fematrix_matvec_noalloc: unsupported dim/order"; return NOALLOC_TOO_LARGE;
    }
  }
  if (bc && pl.n_bdry > 0) {
    k_zero_at<<<grid_for(pl.n_bdry), 256, 0, s>>>(y, pl.bdry.p, pl.n_bdry);
    check_launch("noalloc_zero_out");
  }
  return NOALLOC_OK;
}

}  // namespace dkt
