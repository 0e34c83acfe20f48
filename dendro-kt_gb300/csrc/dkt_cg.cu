// Conjugate gradients on feMatrix::matVec in the form of HeatMat::cgSolve
// (FEM/examples/src/heatMat.cpp:164-325), with an optional Jacobi
// preconditioner, stopping on the relative 2-norm residual -- or, in the
// reference mode, HeatMat::cgSolve itself: no preconditioner and the stop
// ||r||_inf / ||b||_inf <= tol (heatMat.cpp:207-227, 251-257).  All vectors
// stay on the device; reductions are two-stage with a fixed summation order,
// so a solve is bitwise reproducible.
#include <algorithm>
#include <cmath>
#include "dkt_internal.cuh"

namespace dkt {

void fematrix_matvec(Plan &pl, const double *x, double *y, double scale, cudaStream_t s);

constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 512;

__global__ void k_dot_partial(const double *__restrict__ a, const double *__restrict__ b, int64_t n,
                              double *__restrict__ part)
{
  __shared__ double sh[RED_THREADS];
  double s = 0.0;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x)
    s += a[i] * b[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = RED_THREADS / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_sum_partials(const double *__restrict__ part, int n, double *__restrict__ out)
{
  __shared__ double sh[RED_THREADS];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = RED_THREADS / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// max |a_i| per block, NaN if the block holds a NaN (normLInfty,
// include/mathUtils.tcc:69-80, returns NaN for any NaN entry)
__global__ void k_absmax_partial(const double *__restrict__ a, int64_t n, double *__restrict__ part)
{
  __shared__ double sh[RED_THREADS];
  double m = 0.0;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x) {
    const double v = fabs(a[i]);
    m = (v > m || v != v) ? v : m;   // a NaN sticks
  }
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int o = RED_THREADS / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      const double v = sh[threadIdx.x + o];
      if (v > sh[threadIdx.x] || v != v) sh[threadIdx.x] = v;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_max_partials(const double *__restrict__ part, int n, double *__restrict__ out)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double m = 0.0;
  for (int i = 0; i < n; i++) {
    const double v = part[i];
    if (v > m || v != v) m = v;
    if (m != m) break;
  }
  *out = m;
}

static double norm_inf(const double *a, int64_t n, double *part, double *res, cudaStream_t s)
{
  k_absmax_partial<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, n, part);
  k_max_partials<<<1, 32, 0, s>>>(part, RED_BLOCKS, res);
  check_launch("norm_inf");
  double h = 0.0;
  DKT_CUDA(cudaMemcpyAsync(&h, res, sizeof(double), cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaStreamSynchronize(s));
  return h;
}

static double dot(const double *a, const double *b, int64_t n, double *part, double *res, cudaStream_t s)
{
  k_dot_partial<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, b, n, part);
  k_sum_partials<<<1, RED_THREADS, 0, s>>>(part, RED_BLOCKS, res);
  check_launch("dot");
  double h = 0.0;
  DKT_CUDA(cudaMemcpyAsync(&h, res, sizeof(double), cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaStreamSynchronize(s));
  return h;
}

__global__ void k_axpy2(double *__restrict__ x, double *__restrict__ r, const double *__restrict__ p,
                        const double *__restrict__ Ap, double alpha, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
}
__global__ void k_sub(const double *__restrict__ b, const double *__restrict__ Ax, double *__restrict__ r, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) r[i] = b[i] - Ax[i];
}
__global__ void k_prec(const double *__restrict__ r, const double *__restrict__ dinv, double *__restrict__ z, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) z[i] = dinv ? r[i] * dinv[i] : r[i];
}
__global__ void k_pupdate(double *__restrict__ p, const double *__restrict__ z, double beta, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = z[i] + beta * p[i];
}

// Diagonal of the element operators assembled over the directly owned ranks
// of every leaf (interpolated hanging contributions are left out, which keeps
// it a valid Jacobi scaling).  Boundary rows, which feMatrix zeroes, get 1.
// Accumulated in int64 fixed point (scale 2^sc from the largest element
// diagonal) so that the sum, and every solve that uses it, is bitwise
// reproducible whatever the order of the atomics.
__global__ void k_diag(const int32_t *__restrict__ e2n, const uint32_t *__restrict__ info, int64_t n_leaf, int npe,
                       const double *__restrict__ A, const double *__restrict__ B, const double *__restrict__ alpha,
                       const double *__restrict__ beta, const double *__restrict__ table, int sc,
                       unsigned long long *__restrict__ dq)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_leaf) return;
  const int L = info[i] & 0xFFu;
  for (int r = 0; r < npe; r++) {
    const int32_t n = e2n[(int64_t) i * npe + r];
    if (n < 0) continue;
    const double v = table ? table[((int64_t) L * npe + r) * npe + r]
                           : alpha[L] * A[r * npe + r] + beta[L] * B[r * npe + r];
    atomicAdd(dq + n, (unsigned long long) __double2ll_rn(ldexp(v, sc)));
  }
}
__global__ void k_diag_out(const long long *__restrict__ dq, double *__restrict__ d, int64_t n, int sc)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = ldexp((double) dq[i], -sc);
}
__global__ void k_invert_diag(double *__restrict__ d, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = (d[i] != 0.0) ? 1.0 / d[i] : 1.0;
}
__global__ void k_set_at(double *__restrict__ v, const uint32_t *__restrict__ ids, int64_t nb, double val)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nb) v[ids[i]] = val;
}

void diagonal(const Plan &pl, double *diag, cudaStream_t s)
{
  const bool custom = pl.op.kind == OP_CUSTOM;
  // largest |element diagonal entry| over the levels, from the host copies
  double mx = 0.0;
  const int npe = pl.npe, nlev = pl.md + 1;
  for (int L = 0; L < nlev; L++)
    for (int r = 0; r < npe; r++) {
      const double v = custom ? pl.op.table[((size_t) L * npe + r) * npe + r]
                              : pl.op.alpha[L] * pl.op.A[(size_t) r * npe + r] + pl.op.beta[L] * pl.op.B[(size_t) r * npe + r];
      mx = std::max(mx, std::fabs(v));
    }
  int e = 0;
  if (mx > 0.0) std::frexp(mx, &e);          // mx < 2^e
  const int sc = 62 - 8 - e;                 // up to 256 contributions per node
  DBuf<unsigned long long> dq(pl.n_nodes);
  DKT_CUDA(cudaMemsetAsync(dq.p, 0, pl.n_nodes * sizeof(unsigned long long), s));
  k_diag<<<grid_for(pl.n_leaf), 256, 0, s>>>(pl.e2n.p, pl.info.p, pl.n_leaf, pl.npe, pl.opA.p, pl.opB.p,
                                             pl.opAlpha.p, pl.opBeta.p, custom ? pl.opTable.p : nullptr, sc, dq.p);
  check_launch("diag");
  k_diag_out<<<grid_for(pl.n_nodes), 256, 0, s>>>((const long long *) dq.p, diag, pl.n_nodes, sc);
  check_launch("diag_out");
  if (op_has_bc(pl.op.kind) && pl.n_bdry > 0) {
    k_set_at<<<grid_for(pl.n_bdry), 256, 0, s>>>(diag, pl.bdry.p, pl.n_bdry, 1.0);
    check_launch("diag_bdry");
  }
  DKT_CUDA(cudaStreamSynchronize(s));   // dq is freed on return
}

// linf: the reference's own stopping rule (no preconditioner, relative
// L-infinity residual); status -5 when max_iter iterations did not reach tol.
int cg_solve(Plan &pl, const double *b, double *x, int max_iter, double tol, bool jacobi, bool linf, int *iters,
             double *relres, cudaStream_t s)
{
  const int64_t n = pl.n_nodes;
  if (linf) jacobi = false;
  DBuf<double> r(n), z(n), p(n), Ap(n), dinv(jacobi ? n : 0), part(RED_BLOCKS), res(1);
  if (jacobi) {
    diagonal(pl, dinv.p, s);
    k_invert_diag<<<grid_for(n), 256, 0, s>>>(dinv.p, n);
  }
  auto norm = [&](const double *v) {
    return linf ? norm_inf(v, n, part.p, res.p, s) : std::sqrt(dot(v, v, n, part.p, res.p, s));
  };
  double nb = norm(b);
  if (nb == 0.0) nb = 1.0;
  double rz = 0.0, rr = 0.0;
  // r = b - A x, z, p = z, r.z and the relative residual
  auto start = [&]() {
    fematrix_matvec(pl, x, Ap.p, 1.0, s);
    k_sub<<<grid_for(n), 256, 0, s>>>(b, Ap.p, r.p, n);
    k_prec<<<grid_for(n), 256, 0, s>>>(r.p, jacobi ? dinv.p : nullptr, z.p, n);
    DKT_CUDA(cudaMemcpyAsync(p.p, z.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    rz = dot(r.p, z.p, n, part.p, res.p, s);
    rr = norm(r.p) / nb;
  };
  start();
  int it = 0;
  for (int confirm = 0;; confirm++) {
    while (rr > tol && it < max_iter) {
      fematrix_matvec(pl, p.p, Ap.p, 1.0, s);
      const double pAp = dot(p.p, Ap.p, n, part.p, res.p, s);
      if (pAp == 0.0) break;
      const double alpha = rz / pAp;
      k_axpy2<<<grid_for(n), 256, 0, s>>>(x, r.p, p.p, Ap.p, alpha, n);
      rr = norm(r.p) / nb;
      it++;
      if (rr <= tol) break;
      k_prec<<<grid_for(n), 256, 0, s>>>(r.p, jacobi ? dinv.p : nullptr, z.p, n);
      const double rz2 = dot(r.p, z.p, n, part.p, res.p, s);
      const double beta = rz2 / rz;
      rz = rz2;
      k_pupdate<<<grid_for(n), 256, 0, s>>>(p.p, z.p, beta, n);
    }
    // The reference mode stops on its recursive residual, as cgSolve does.
    // Otherwise convergence is confirmed on the true residual b - A x, and
    // the iteration restarts from x while that is still above tol (the
    // recursive residual drifts from it by round-off).
    if (linf || rr > tol || confirm >= 8) break;
    start();
    if (rr <= tol || it >= max_iter) break;
  }
  check_launch("cg");
  DKT_CUDA(cudaStreamSynchronize(s));
  if (iters) *iters = it;
  if (relres) *relres = rr;
  return rr <= tol ? 0 : -5;
}

}  // namespace dkt
