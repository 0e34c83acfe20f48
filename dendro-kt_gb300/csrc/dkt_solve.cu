// Device-resident Jacobi-preconditioned CG and mixed-precision iterative
// refinement on the feMatrix operator of a plan -- one mesh, or a batch of
// independent meshes concatenated into one block-diagonal plan
// (dkt_batch.cu), each with its own scalars and its own convergence.
//
// The vectors are cut into chunks that never straddle two meshes; one CTA
// per chunk does the vector work and writes per-chunk partial sums, and a
// one-block-per-mesh kernel adds each mesh's partials in a fixed order (thread
// sums over a fixed stride, then a fixed reduction tree), so every dot product
// accumulates in FP64 across threads and is bitwise reproducible (a thread's
// eight terms of a binary32 vector are first added in binary32).  Chunks are
// small (2048 nodes, eight per thread) because FP64 additions are
// long-latency on this part: a thread's chain of dependent FP64
// accumulations must stay short.  All
// scalars (alpha, beta, r.z, r.r, a converged flag) stay on the device, so a
// block of iterations has no host synchronisation and is captured once into
// a CUDA graph that is relaunched until every mesh has converged.  A
// converged mesh is frozen (alpha = 0, p kept), so the iterations that run
// past its convergence change nothing.
//
// Mixed precision (reliable updates): one Jacobi-PCG sequence runs on
// binary32 vectors with the binary32 Q1 product, in units of the FP64
// residual norm at the last update.  Whenever a mesh's recursive residual has
// fallen 100x (or claims convergence), or 512 iterations passed without that,
// the accumulated correction is added to x in FP64, the residual is
// recomputed exactly (b - A x with the FP64 fixed-point product) and replaces
// the binary32 one, and the search direction is rescaled -- the Krylov space
// is kept, so the iteration count stays near that of FP64 PCG.  Only a mesh
// whose true residual is far above its recursive one (binary32 round-off has
// taken over) restarts its direction.  Convergence is only ever declared on
// the FP64 residual.  Each mesh of a batch is judged on its own: one whose
// true residual stopped falling while its recursion says it fell, or that 512
// iterations did not move, twice in a row (the system is beyond binary32,
// condition number near 1/eps32; the first time only restarts its
// direction), is frozen in the binary32 sequence and finished with FP64 PCG
// from its current x once the others are done.
#include <algorithm>
#include <cmath>
#include "dkt_internal.cuh"

namespace dkt {

void fematrix_matvec(Plan &pl, const double *x, double *y, double scale, cudaStream_t s);
void q1f32_apply(Plan &pl, const float *x, float *y, bool bc_in, bool bc_out, cudaStream_t s);
void diagonal(const Plan &pl, double *diag, cudaStream_t s);

namespace {

constexpr int ST = 256;                 // threads of the vector kernels
constexpr int64_t CHK = 2048;           // nodes per chunk
constexpr int CHUNK_IT = 16;            // CG iterations per captured graph

struct CgScal {
  double rz, pq, rr, alpha, beta, rr_stop;
  int done, it, conv_it, pad;
};

struct Chunks {
  int64_t n = 0;                        // chunks
  int P = 1;                            // meshes
  DBuf<int64_t> lo, hi;                 // node range of chunk c
  DBuf<int32_t> prob;                   // mesh of chunk c
  DBuf<int32_t> first;                  // chunks of mesh p: [first[p], first[p+1])
};

void make_chunks(const Plan &pl, Chunks &c, cudaStream_t s)
{
  std::vector<int64_t> seg = pl.seg;
  if (seg.size() < 2) seg = {0, pl.n_nodes};
  c.P = (int) seg.size() - 1;
  std::vector<int64_t> lo, hi;
  std::vector<int32_t> prob, first;
  for (int p = 0; p < c.P; p++) {
    first.push_back((int32_t) lo.size());
    for (int64_t a = seg[p]; a < seg[p + 1]; a += CHK) {
      lo.push_back(a);
      hi.push_back(std::min(a + CHK, seg[p + 1]));
      prob.push_back(p);
    }
  }
  first.push_back((int32_t) lo.size());
  c.n = (int64_t) lo.size();
  if (c.n == 0) { lo.push_back(0); hi.push_back(0); prob.push_back(0); }
  c.lo.upload(lo.data(), lo.size(), s);
  c.hi.upload(hi.data(), hi.size(), s);
  c.prob.upload(prob.data(), prob.size(), s);
  c.first.upload(first.data(), first.size(), s);
}

__device__ __forceinline__ double block_sum(double v, double *sh)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  v = (threadIdx.x < blockDim.x / 32) ? sh[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Widening of a binary32 value to FP64 with integer operations: a hardware
// conversion runs on the FP64 pipe, which on this part retires about one
// warp instruction per 64 cycles per sub-partition and would bound the
// binary32 vector kernels.  Exact for normal numbers, zeros, infinities and
// NaNs; binary32 subnormals (below 1.2e-38) become signed zeros, which
// changes a dot product by less than 1e-38 per term.
__device__ __forceinline__ double widen(float f)
{
  const uint32_t u = __float_as_uint(f), e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
  uint64_t r = e == 0u ? 0ull
                       : (e == 0xFFu ? (0x7FF0000000000000ull | ((uint64_t) m << 29))
                                     : (((uint64_t) (e + 896u) << 52) | ((uint64_t) m << 29)));
  r |= (uint64_t) (u & 0x80000000u) << 32;
  return __longlong_as_double((long long) r);
}
__device__ __forceinline__ double widen(double d) { return d; }

// part[c] = sum over chunk c of a*b (FP64 across threads)
template <typename T>
__global__ void __launch_bounds__(ST) k_dot(const T *__restrict__ a, const T *__restrict__ b,
                                           const int64_t *__restrict__ lo, const int64_t *__restrict__ hi,
                                           double *__restrict__ part, const int *__restrict__ skip = nullptr,
                                           const int32_t *__restrict__ prob = nullptr, int stride = 1)
{
  __shared__ double sh[ST / 32];
  // chunks of converged meshes contribute nothing (their sums are not used)
  if (skip && skip[(int64_t) prob[blockIdx.x] * stride]) {
    if (threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  // each thread's eight terms in T (binary32 vectors: binary32 partials, one
  // widening per thread, so the FP64 pipe adds 256 partials per chunk instead
  // of 2048 terms), then the fixed FP64 block tree
  T t = T(0);
  for (int64_t i = lo[blockIdx.x] + threadIdx.x; i < hi[blockIdx.x]; i += ST) t = fma(a[i], b[i], t);
  const double s = block_sum(widen(t), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Per mesh (one block of FIN threads): sum of its chunks' partials in a fixed
// order -- thread t adds chunks c0 + t, c0 + t + FIN, ... in turn, then the
// fixed shuffle and shared-memory tree of block_sum.  A block, not a warp:
// FP64 additions are long-latency on this part, and a warp would add about
// 80 partials in one dependent chain per lane on a 5 M-node mesh.  Thread 0
// returns the total.
constexpr int FIN = 256;
__device__ __forceinline__ double mesh_sum(const double *part, int stride, int off, int c0, int c1, double *sh)
{
  double s = 0.0;
#pragma unroll 4
  for (int c = c0 + (int) threadIdx.x; c < c1; c += FIN) s += part[(int64_t) c * stride + off];
  return block_sum(s, sh);
}
// one block per mesh in the finalisers
#define MESH_OF_BLOCK(P)                                                     \
  __shared__ double sh_fin[FIN / 32];                                        \
  const int p = (int) blockIdx.x;                                            \
  if (p >= (P)) return;

// alpha = r.z / p.q (0 once converged or on breakdown)
__global__ void k_fin_alpha(const double *__restrict__ part, const int32_t *__restrict__ first, int P,
                            CgScal *__restrict__ sc)
{
  MESH_OF_BLOCK(P)
  const double pq = mesh_sum(part, 1, 0, first[p], first[p + 1], sh_fin);
  if (threadIdx.x != 0) return;
  CgScal &q = sc[p];
  q.pq = pq;
  q.alpha = (q.done || !(pq != 0.0)) ? 0.0 : q.rz / pq;
}

// x += alpha p; r -= alpha q; z = dinv r; partial sums of r.z and r.r
template <typename T>
__global__ void __launch_bounds__(ST) k_update(T *__restrict__ x, T *__restrict__ r, T *__restrict__ z,
                                              const T *__restrict__ p, const T *__restrict__ q,
                                              const T *__restrict__ dinv, const int64_t *__restrict__ lo,
                                              const int64_t *__restrict__ hi, const int32_t *__restrict__ prob,
                                              const CgScal *__restrict__ sc, double *__restrict__ part)
{
  __shared__ double sh[ST / 32];
  if (sc[prob[blockIdx.x]].done) {   // a converged mesh: frozen, its sums unused
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = 0.0; part[2 * blockIdx.x + 1] = 0.0; }
    return;
  }
  const double a = sc[prob[blockIdx.x]].alpha;
  const T at = (T) a;
  T trz = T(0), trr = T(0);   // each thread's terms in T, as in k_dot
  for (int64_t i = lo[blockIdx.x] + threadIdx.x; i < hi[blockIdx.x]; i += ST) {
    T ri = r[i];
    if (a != 0.0) {
      x[i] += at * p[i];
      ri -= at * q[i];
      r[i] = ri;
    }
    const T zi = dinv ? ri * dinv[i] : ri;
    z[i] = zi;
    trz = fma(ri, zi, trz);
    trr = fma(ri, ri, trr);
  }
  const double srz = block_sum(widen(trz), sh);
  const double srr = block_sum(widen(trr), sh);
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = srz; part[2 * blockIdx.x + 1] = srr; }
}

// beta = rz_new / rz; convergence test on r.r
__global__ void k_fin_beta(const double *__restrict__ part, const int32_t *__restrict__ first, int P,
                           CgScal *__restrict__ sc, int count, int *__restrict__ n_done)
{
  MESH_OF_BLOCK(P)
  const double a = mesh_sum(part, 2, 0, first[p], first[p + 1], sh_fin);
  const double b = mesh_sum(part, 2, 1, first[p], first[p + 1], sh_fin);
  if (threadIdx.x != 0) return;
  CgScal &q = sc[p];
  if (!q.done) {
    if (count) q.it++;
    q.beta = (q.rz != 0.0) ? a / q.rz : 0.0;
    q.rz = a;
    q.rr = b;
    if (b <= q.rr_stop || !(b == b)) {
      q.done = 1;
      q.conv_it = q.it;
      atomicAdd(n_done, 1);
    }
  } else {
    q.beta = 0.0;
  }
}

template <typename T>
__global__ void k_pupd(T *__restrict__ p, const T *__restrict__ z, const int64_t *__restrict__ lo,
                       const int64_t *__restrict__ hi, const int32_t *__restrict__ prob, const CgScal *__restrict__ sc,
                       int first)
{
  const CgScal &q = sc[prob[blockIdx.x]];
  if (q.done && !first) return;
  const T b = (T) q.beta;
  for (int64_t i = lo[blockIdx.x] + threadIdx.x; i < hi[blockIdx.x]; i += ST) p[i] = first ? z[i] : z[i] + b * p[i];
}

__global__ void k_residual(const double *__restrict__ b, const double *__restrict__ ax, double *__restrict__ r,
                           int64_t n)
{
  for (int64_t i = (int64_t) blockIdx.x * ST + threadIdx.x; i < n; i += (int64_t) gridDim.x * ST) r[i] = b[i] - ax[i];
}

// per mesh: nrm[p] = sqrt(sum of its partials)
__global__ void k_norms(const double *__restrict__ part, const int32_t *__restrict__ first, int P,
                        double *__restrict__ nrm)
{
  MESH_OF_BLOCK(P)
  const double v = mesh_sum(part, 1, 0, first[p], first[p + 1], sh_fin);
  if (threadIdx.x == 0) nrm[p] = sqrt(v);
}

__global__ void k_invert(const double *__restrict__ d, double *__restrict__ o64, float *__restrict__ o32, int64_t n)
{
  for (int64_t i = (int64_t) blockIdx.x * ST + threadIdx.x; i < n; i += (int64_t) gridDim.x * ST) {
    const double v = (d[i] != 0.0) ? 1.0 / d[i] : 1.0;
    if (o64) o64[i] = v;
    if (o32) o32[i] = (float) v;
  }
}
__global__ void k_init_scal(CgScal *sc, int P, const double *__restrict__ rr_stop, double rr_stop_all,
                            int *__restrict__ n_done)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p == 0) *n_done = 0;
  if (p >= P) return;
  CgScal &q = sc[p];
  q.rz = q.pq = q.rr = q.alpha = q.beta = 0.0;
  q.rr_stop = rr_stop ? rr_stop[p] : rr_stop_all;
  q.done = 0;
  q.it = 0;
  q.conv_it = -1;
}

// The operator of one CG: FP64 feMatrix product or binary32 product.
template <typename T> struct CgOp;
template <> struct CgOp<double> {
  static void apply(Plan &pl, const double *x, double *y, cudaStream_t s) { fematrix_matvec(pl, x, y, 1.0, s); }
};
template <> struct CgOp<float> {
  // CG vectors keep zero boundary entries, so the input needs no clearing
  static void apply(Plan &pl, const float *x, float *y, cudaStream_t s) { q1f32_apply(pl, x, y, false, true, s); }
};

inline unsigned pgrid(int P) { return (unsigned) ((P + 127) / 128); }
inline unsigned wgrid(int P) { return (unsigned) std::max(P, 1); }   // finalisers: a block of FIN threads per mesh

// Jacobi-PCG on all meshes of the plan, in type T (FP64 dots).  r must hold
// b - A x on entry.
template <typename T>
struct Cg {
  Plan &pl;
  const Chunks &ch;
  int64_t n;
  DBuf<T> z, p, q;
  DBuf<double> part;
  DBuf<CgScal> sc;
  DBuf<int> n_done;
  std::vector<CgScal> hsc;
  int h_done_v = 0;
  int *h_done = &h_done_v;   // pageable: pinned memory would cost a device-wide sync to free
  cudaGraphExec_t exec = nullptr;
  T *gx = nullptr, *gr = nullptr;
  const T *gd = nullptr;
  int64_t graph_count = 0;   // kernels in one launch of the graph

  Cg(Plan &pl_, const Chunks &ch_)
      : pl(pl_), ch(ch_), n(pl_.n_nodes), z(n), p(n), q(n), part(2 * std::max<int64_t>(ch_.n, 1)), sc(ch_.P),
        n_done(1), hsc(ch_.P)
  {
  }
  ~Cg()
  {
    if (exec) cudaGraphExecDestroy(exec);
  }

  void iteration(T *x, T *r, const T *dinv, cudaStream_t s)
  {
    const unsigned nb = (unsigned) ch.n;
    CgOp<T>::apply(pl, p.p, q.p, s);
    k_dot<T><<<nb, ST, 0, s>>>(p.p, q.p, ch.lo.p, ch.hi.p, part.p, &sc.p[0].done, ch.prob.p,
                               (int) (sizeof(CgScal) / sizeof(int)));
    k_fin_alpha<<<wgrid(ch.P), FIN, 0, s>>>(part.p, ch.first.p, ch.P, sc.p);
    k_update<T><<<nb, ST, 0, s>>>(x, r, z.p, p.p, q.p, dinv, ch.lo.p, ch.hi.p, ch.prob.p, sc.p, part.p);
    k_fin_beta<<<wgrid(ch.P), FIN, 0, s>>>(part.p, ch.first.p, ch.P, sc.p, 1, n_done.p);
    k_pupd<T><<<nb, ST, 0, s>>>(p.p, z.p, ch.lo.p, ch.hi.p, ch.prob.p, sc.p, 0);
    check_launch("cg_iteration");
    pl.n_launch += 5;
  }

  // Runs until every mesh converged or max_iter iterations; per-mesh
  // results in hsc (conv_it = -1: not converged).
  void solve(T *x, T *r, const T *dinv, const double *rr_stop_dev, double rr_stop, int max_iter, cudaStream_t s)
  {
    if (ch.n == 0) return;
    const unsigned nb = (unsigned) ch.n;
    k_init_scal<<<pgrid(ch.P), 128, 0, s>>>(sc.p, ch.P, rr_stop_dev, rr_stop, n_done.p);
    // z = dinv r, r.z, r.r (alpha = 0 leaves x and r unchanged), p = z
    k_update<T><<<nb, ST, 0, s>>>(x, r, z.p, p.p, q.p, dinv, ch.lo.p, ch.hi.p, ch.prob.p, sc.p, part.p);
    k_fin_beta<<<wgrid(ch.P), FIN, 0, s>>>(part.p, ch.first.p, ch.P, sc.p, 0, n_done.p);
    k_pupd<T><<<nb, ST, 0, s>>>(p.p, z.p, ch.lo.p, ch.hi.p, ch.prob.p, sc.p, 1);
    check_launch("cg_start");
    pl.n_launch += 4;
    ensure_graph(x, r, dinv, s);
    int done_iters = 0;
    for (;;) {
      DKT_CUDA(cudaMemcpyAsync(h_done, n_done.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      DKT_CUDA(cudaStreamSynchronize(s));
      if (*h_done >= ch.P || done_iters >= max_iter) break;
      DKT_CUDA(cudaGraphLaunch(exec, s));
      pl.n_launch += graph_count;
      done_iters += CHUNK_IT;
    }
    DKT_CUDA(cudaMemcpyAsync(hsc.data(), sc.p, ch.P * sizeof(CgScal), cudaMemcpyDeviceToHost, s));
    DKT_CUDA(cudaStreamSynchronize(s));
  }

  // CHUNK_IT iterations captured once into a graph (re-captured when the
  // vectors change)
  void ensure_graph(T *x, T *r, const T *dinv, cudaStream_t s)
  {
    if (exec == nullptr || gx != x || gr != r || gd != dinv) {
      if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
      cudaGraph_t g = nullptr;
      const int64_t before = pl.n_launch;
      // products inside the iterations skip the tiles of converged meshes
      pl.skip_mesh = ch.P > 1 ? &sc.p[0].done : nullptr;
      pl.skip_stride = (int) (sizeof(CgScal) / sizeof(int));
      DKT_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      try {
        for (int k = 0; k < CHUNK_IT; k++) iteration(x, r, dinv, s);
      } catch (...) {
        cudaStreamEndCapture(s, &g);
        if (g) cudaGraphDestroy(g);
        pl.n_launch = before;
        pl.skip_mesh = nullptr;
        throw;
      }
      pl.skip_mesh = nullptr;
      DKT_CUDA(cudaStreamEndCapture(s, &g));
      graph_count = pl.n_launch - before;
      pl.n_launch = before;
      const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
      cudaGraphDestroy(g);
      DKT_CUDA(e);
      gx = x; gr = r; gd = dinv;
    }
  }
};

// Reliable-update kernels (per chunk, per mesh scalars).
// x += sig[p] * xc on the meshes whose binary32 recursion is finite; xc = 0
__global__ void k_fold(double *__restrict__ x, float *__restrict__ xc, const int64_t *__restrict__ lo,
                       const int64_t *__restrict__ hi, const int32_t *__restrict__ prob, const double *__restrict__ sig,
                       const int *__restrict__ use)
{
  const int q = prob[blockIdx.x];
  const double a = use[q] ? sig[q] : 0.0;
  for (int64_t i = lo[blockIdx.x] + threadIdx.x; i < hi[blockIdx.x]; i += ST) {
    if (a != 0.0) x[i] += a * (double) xc[i];
    xc[i] = 0.0f;
  }
}
// r32 = r / signew (0 on finished meshes); p *= sig / signew
__global__ void k_rescale(const double *__restrict__ r, float *__restrict__ r32, float *__restrict__ p,
                          const int64_t *__restrict__ lo, const int64_t *__restrict__ hi,
                          const int32_t *__restrict__ prob, const double *__restrict__ sig,
                          const double *__restrict__ signew, const int *__restrict__ active)
{
  const int q = prob[blockIdx.x];
  const bool on = active[q] && signew[q] > 0.0;
  const double inv = on ? 1.0 / signew[q] : 0.0;
  const float ps = on ? (float) (sig[q] / signew[q]) : 0.0f;
  for (int64_t i = lo[blockIdx.x] + threadIdx.x; i < hi[blockIdx.x]; i += ST) {
    r32[i] = (float) (r[i] * inv);
    p[i] *= ps;
  }
}
// p = z (a fresh search direction) on the meshes flagged
__global__ void k_restart(float *__restrict__ p, const float *__restrict__ z, const int64_t *__restrict__ lo,
                          const int64_t *__restrict__ hi, const int32_t *__restrict__ prob, const int *__restrict__ flag)
{
  if (!flag[prob[blockIdx.x]]) return;
  for (int64_t i = lo[blockIdx.x] + threadIdx.x; i < hi[blockIdx.x]; i += ST) p[i] = z[i];
}
// per mesh: finished meshes freeze (done), the others take alpha = 0 for the
// z / r.z refresh that follows
__global__ void k_mark(CgScal *__restrict__ sc, const int *__restrict__ active, int P)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  sc[q].alpha = 0.0;
  sc[q].done = active[q] ? 0 : 1;
  sc[q].rr_stop = -1.0;   // the binary32 recursion never declares convergence itself
}

}  // namespace

// FP64 Jacobi-PCG (precision 0) or mixed-precision refinement (precision 1)
// on every mesh of the plan.  Per mesh: iterations, refinements and the
// relative residual ||b - A x|| / ||b||.  Returns 0 when every mesh reached
// tol, -5 otherwise.
int pcg_solve(Plan &pl, const double *b, double *x, int precision, int max_iter, double tol, bool jacobi,
              int *iters, int *refinements, double *relres, cudaStream_t user)
{
  const int64_t n = pl.n_nodes;
  if (precision == 1 && !pl.f32_ready)
    throw std::runtime_error("mixed precision needs a Q1 or Q2 built-in operator without stale parent reads");
  const bool saved_timing = pl.timing;
  pl.timing = false;
  cudaStream_t s = nullptr;
  cudaEvent_t ev = nullptr;
  DKT_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  DKT_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  DKT_CUDA(cudaEventRecord(ev, user));
  DKT_CUDA(cudaStreamWaitEvent(s, ev, 0));
  int rc = -5;
  try {
    Chunks ch;
    make_chunks(pl, ch, s);
    const int P = ch.P;
    const unsigned nb = (unsigned) std::max<int64_t>(ch.n, 1);
    std::vector<int> tot(P, 0), outer(P, 0), h_active(P, 1);
    std::vector<double> rel(P, 0.0), hb(P), hr(P);
    DBuf<double> d(n), dinv(jacobi ? n : 0), ax(n), part(std::max<int64_t>(ch.n, 1)), bnrm(P), rnrm(P);
    DBuf<float> dinv32(jacobi && precision == 1 ? n : 0);
    DBuf<int> active(P);
    if (jacobi) {
      diagonal(pl, d.p, s);
      k_invert<<<608, ST, 0, s>>>(d.p, dinv.p, dinv32.p, n);
      pl.n_launch += 2;
    }
    // per-mesh ||b||
    k_dot<double><<<nb, ST, 0, s>>>(b, b, ch.lo.p, ch.hi.p, part.p);
    k_norms<<<wgrid(P), FIN, 0, s>>>(part.p, ch.first.p, P, bnrm.p);
    pl.n_launch += 2;
    DKT_CUDA(cudaMemcpyAsync(hb.data(), bnrm.p, P * sizeof(double), cudaMemcpyDeviceToHost, s));
    DKT_CUDA(cudaStreamSynchronize(s));
    for (int p = 0; p < P; p++) if (!(hb[p] > 0.0)) hb[p] = 1.0;
    // FP64 Jacobi-PCG from the current x on every mesh (meshes already at
    // tolerance stop at once); used by precision 0 and as the fallback of
    // the mixed solver
    int used = 0;
    // per-mesh ||b - A x|| / ||b|| with the FP64 product, into rel; returns
    // the number of meshes still above tol
    auto true_relres = [&](DBuf<double> &r) {
      fematrix_matvec(pl, x, ax.p, 1.0, s);
      k_residual<<<608, ST, 0, s>>>(b, ax.p, r.p, n);
      k_dot<double><<<nb, ST, 0, s>>>(r.p, r.p, ch.lo.p, ch.hi.p, part.p);
      k_norms<<<wgrid(P), FIN, 0, s>>>(part.p, ch.first.p, P, rnrm.p);
      pl.n_launch += 4;
      DKT_CUDA(cudaMemcpyAsync(hr.data(), rnrm.p, P * sizeof(double), cudaMemcpyDeviceToHost, s));
      DKT_CUDA(cudaStreamSynchronize(s));
      int above = 0;
      for (int p = 0; p < P; p++) {
        rel[p] = hr[p] == 0.0 ? 0.0 : hr[p] / hb[p];   // b = 0: x = 0 is exact
        above += rel[p] > tol ? 1 : 0;
      }
      return above;
    };
    // Convergence is declared on the true residual: the CG recursion stops
    // on its recursive residual, which drifts from b - A x by round-off, so
    // each stop is checked against b - A x and the iteration restarts from
    // x (keeping the iterations spent) while some mesh is still above tol.
    auto fp64_pcg = [&](int budget) {
      Cg<double> cg(pl, ch);
      DBuf<double> r(n), stop(P);
      std::vector<double> hs(P);
      for (int p = 0; p < P; p++) hs[p] = tol * tol * hb[p] * hb[p];
      stop.upload(hs.data(), P, s);
      rc = -5;
      for (int pass = 0; pass < 8 && budget > 0; pass++) {
        fematrix_matvec(pl, x, ax.p, 1.0, s);
        k_residual<<<608, ST, 0, s>>>(b, ax.p, r.p, n);
        pl.n_launch++;
        cg.solve(x, r.p, jacobi ? dinv.p : nullptr, stop.p, 0.0, budget, s);
        int spent = 0;
        for (int p = 0; p < P; p++) {
          const CgScal &q = cg.hsc[p];
          const int k = q.conv_it >= 0 ? q.conv_it : q.it;
          tot[p] += k;
          spent = std::max(spent, k);
        }
        budget -= std::max(spent, 1);
        if (true_relres(r) == 0) { rc = 0; break; }
      }
    };
    if (precision == 0) {
      fp64_pcg(max_iter);
    } else {
      // One binary32 Krylov sequence in units of sig (the FP64 residual norm
      // at the last reliable update); every few chunks of iterations the
      // correction is folded into x in FP64 and the true residual replaces
      // the recursive one (reliable updates), so the Krylov space is kept
      // across the precision boundary.
      Cg<float> cg(pl, ch);
      DBuf<float> xc(n), r32(n);
      DBuf<double> r(n), sig(P), signew(P);
      DBuf<int> act(P), fold_ok(P), rflag(P);
      std::vector<double> hsig(P, 0.0);
      // meshes whose true residual stopped following their binary32
      // recursion: frozen in the binary32 sequence, finished by FP64 PCG
      std::vector<int> beyond(P, 0);
      std::vector<int> stalls(P, 0);   // consecutive updates that found the mesh stalled
      const double delta = 1e-2;      // update once the recursive residual fell by this much
      int since = 0, updates = 0;
      DKT_CUDA(cudaMemsetAsync(xc.p, 0, n * sizeof(float), s));
      auto true_residual = [&]() {
        fematrix_matvec(pl, x, ax.p, 1.0, s);
        k_residual<<<608, ST, 0, s>>>(b, ax.p, r.p, n);
        k_dot<double><<<nb, ST, 0, s>>>(r.p, r.p, ch.lo.p, ch.hi.p, part.p);
        k_norms<<<wgrid(P), FIN, 0, s>>>(part.p, ch.first.p, P, signew.p);
        pl.n_launch += 3;
        DKT_CUDA(cudaMemcpyAsync(hr.data(), signew.p, P * sizeof(double), cudaMemcpyDeviceToHost, s));
        DKT_CUDA(cudaStreamSynchronize(s));
        int n_above = 0;
        for (int p = 0; p < P; p++) {
          rel[p] = hr[p] == 0.0 ? 0.0 : hr[p] / hb[p];   // b = 0: x = 0 is exact
          n_above += rel[p] > tol ? 1 : 0;
          h_active[p] = rel[p] > tol && !beyond[p] ? 1 : 0;
        }
        act.upload(h_active.data(), P, s);
        return n_above;
      };
      if (true_residual() == 0) {
        rc = 0;
      } else {
        // start: r32 = r / |r|, z, r.z, p = z
        k_rescale<<<nb, ST, 0, s>>>(r.p, r32.p, cg.p.p, ch.lo.p, ch.hi.p, ch.prob.p, signew.p, signew.p, act.p);
        DKT_CUDA(cudaMemcpyAsync(sig.p, signew.p, P * sizeof(double), cudaMemcpyDeviceToDevice, s));
        k_init_scal<<<pgrid(P), 128, 0, s>>>(cg.sc.p, P, nullptr, -1.0, cg.n_done.p);
        k_mark<<<pgrid(P), 128, 0, s>>>(cg.sc.p, act.p, P);
        k_update<float><<<nb, ST, 0, s>>>(xc.p, r32.p, cg.z.p, cg.p.p, cg.q.p, dinv32.p ? dinv32.p : nullptr,
                                          ch.lo.p, ch.hi.p, ch.prob.p, cg.sc.p, cg.part.p);
        k_fin_beta<<<wgrid(P), FIN, 0, s>>>(cg.part.p, ch.first.p, P, cg.sc.p, 0, cg.n_done.p);
        k_pupd<float><<<nb, ST, 0, s>>>(cg.p.p, cg.z.p, ch.lo.p, ch.hi.p, ch.prob.p, cg.sc.p, 1);
        pl.n_launch += 6;
        hsig = hr;
        cg.ensure_graph(xc.p, r32.p, jacobi ? dinv32.p : nullptr, s);
        while (used < max_iter) {
          DKT_CUDA(cudaGraphLaunch(cg.exec, s));
          pl.n_launch += cg.graph_count;
          used += CHUNK_IT;
          since += CHUNK_IT;
          for (int p = 0; p < P; p++) if (h_active[p]) tot[p] += CHUNK_IT;
          DKT_CUDA(cudaMemcpyAsync(cg.hsc.data(), cg.sc.p, P * sizeof(CgScal), cudaMemcpyDeviceToHost, s));
          DKT_CUDA(cudaStreamSynchronize(s));
          // update when some active mesh's recursive residual fell by delta or
          // claims convergence, or after 512 iterations without one
          const bool long_run = since >= 512;
          bool upd = long_run;
          for (int p = 0; p < P; p++) {
            if (!h_active[p]) continue;
            const double rr = cg.hsc[p].rr;   // |r32|^2, |r32| = 1 at the last update
            if (rr <= delta * delta || std::sqrt(rr) * hsig[p] <= tol * hb[p] || !(rr == rr)) upd = true;
          }
          if (!upd) continue;
          std::vector<double> rec(P);
          std::vector<int> finite(P);
          for (int p = 0; p < P; p++) {
            rec[p] = std::sqrt(cg.hsc[p].rr) * hsig[p];
            finite[p] = (rec[p] == rec[p]) ? 1 : 0;   // a NaN recursion's correction is dropped
          }
          fold_ok.upload(finite.data(), P, s);
          // reliable update: x += sig * xc, true residual, rescale r32 and p
          k_fold<<<nb, ST, 0, s>>>(x, xc.p, ch.lo.p, ch.hi.p, ch.prob.p, sig.p, fold_ok.p);
          pl.n_launch++;
          updates++;
          since = 0;
          for (int p = 0; p < P; p++) outer[p] += h_active[p];
          if (true_residual() == 0) { rc = 0; break; }
          // per mesh: a stall is a true residual that stopped falling while
          // the recursion says it fell, or one that 512 binary32 iterations did
          // not lower by a tenth.  A first stall restarts the mesh's direction
          // (binary32 rounding can throw one sequence off, and the product's
          // float atomics make runs differ); a second in a row, or a recursion
          // gone NaN, means the mesh is beyond binary32.  The other meshes of a
          // batch carry on, whatever stage of their convergence this update
          // finds them at.
          int n_mixed = 0;
          bool newly = false;
          for (int p = 0; p < P; p++) {
            if (!h_active[p]) continue;
            const bool stalled = (rec[p] <= 0.1 * hsig[p] && hr[p] > 0.5 * hsig[p]) ||
                                 (long_run && hr[p] > 0.9 * hsig[p]);
            stalls[p] = stalled ? stalls[p] + 1 : 0;
            if (!(rec[p] == rec[p]) || stalls[p] >= 2) {
              beyond[p] = 1;
              h_active[p] = 0;
              newly = true;
            }
            n_mixed += h_active[p];
          }
          if (newly) act.upload(h_active.data(), P, s);
          if (n_mixed == 0) break;
          k_rescale<<<nb, ST, 0, s>>>(r.p, r32.p, cg.p.p, ch.lo.p, ch.hi.p, ch.prob.p, sig.p, signew.p, act.p);
          DKT_CUDA(cudaMemcpyAsync(sig.p, signew.p, P * sizeof(double), cudaMemcpyDeviceToDevice, s));
          k_mark<<<pgrid(P), 128, 0, s>>>(cg.sc.p, act.p, P);
          k_update<float><<<nb, ST, 0, s>>>(xc.p, r32.p, cg.z.p, cg.p.p, cg.q.p, jacobi ? dinv32.p : nullptr,
                                            ch.lo.p, ch.hi.p, ch.prob.p, cg.sc.p, cg.part.p);
          k_fin_beta<<<wgrid(P), FIN, 0, s>>>(cg.part.p, ch.first.p, P, cg.sc.p, 0, cg.n_done.p);
          pl.n_launch += 4;
          // the kept direction only fits a residual that the recursion still
          // tracks; where the true residual is far above the recursive one
          // (binary32 round-off has taken over), that mesh restarts from p = z.
          // A mesh whose recursion still tracks keeps its direction however
          // long the run was: ill-conditioned meshes (2D at depth 14) need
          // thousands of iterations, and a restart every 512 would turn CG
          // into a much slower restarted method.
          std::vector<int> rs(P, 0);
          bool any = false;
          for (int p = 0; p < P; p++)
            if (h_active[p] && (stalls[p] > 0 || !(hr[p] <= 10.0 * rec[p]))) rs[p] = 1, any = true;
          if (any) {
            rflag.upload(rs.data(), P, s);
            k_restart<<<nb, ST, 0, s>>>(cg.p.p, cg.z.p, ch.lo.p, ch.hi.p, ch.prob.p, rflag.p);
            pl.n_launch++;
          }
          hsig = hr;
        }
      }
      if (rc != 0 && used < max_iter) {
        fp64_pcg(max_iter - used);
        pl.fallbacks++;
      }
    }
    check_launch("pcg");
    DKT_CUDA(cudaEventRecord(ev, s));
    DKT_CUDA(cudaStreamWaitEvent(user, ev, 0));
    DKT_CUDA(cudaStreamSynchronize(s));
    for (int p = 0; p < P; p++) {
      if (iters) iters[p] = tot[p];
      if (refinements) refinements[p] = outer[p];
      if (relres) relres[p] = rel[p];
    }
  } catch (...) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    cudaEventDestroy(ev);
    pl.timing = saved_timing;
    throw;
  }
  cudaStreamDestroy(s);
  cudaEventDestroy(ev);
  pl.timing = saved_timing;
  return rc;
}

}  // namespace dkt
