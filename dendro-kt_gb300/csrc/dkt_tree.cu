// Tree construction on the device: refinement by a predicate, level by level,
// and 2:1 balancing with the semantics of SFC_Tree::propagateNeighbours +
// reconstruction (src/tsort.cpp:777-854): the set S of cells closed under
// "parent and the parent's in-domain neighbours at the parent level"; the
// balanced leaves are the children of the parents of S-cells that are not
// parents of S-cells themselves.  Cells are 64-bit keys (level | anchors);
// every set operation is a radix sort + unique + binary search.
#include <cmath>
#include <vector>
#include "dkt_host.h"
#include "dkt_internal.cuh"

namespace dkt {

constexpr uint64_t TSENT = ~0ull;

__device__ inline void tdecode(uint64_t k, int dim, int md, uint32_t *a, int &lev)
{
  const uint64_t m = (1ull << md) - 1ull;
  for (int d = 0; d < dim; d++) { a[d] = (uint32_t) (k & m); k >>= md; }
  lev = (int) k;
}

__global__ void k_parents(const uint64_t *__restrict__ in, uint64_t *__restrict__ out, int64_t n, int dim, int md)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t a[MAX_DIM];
  int lev;
  tdecode(in[i], dim, md, a, lev);
  const uint32_t mask = ~((1u << (md - lev + 1)) - 1u);
  for (int d = 0; d < dim; d++) a[d] &= mask;
  out[i] = cell_key(a, lev - 1, dim, md);
}

// cell and its 3^dim - 1 in-domain same-level neighbours (appendAllNeighbours)
__global__ void k_neighbourhood(const uint64_t *__restrict__ in, uint64_t *__restrict__ out, int64_t n, int dim, int md,
                                int n3)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t a[MAX_DIM];
  int lev;
  tdecode(in[i], dim, md, a, lev);
  const uint64_t len = 1ull << (md - lev), top = 1ull << md;
  for (int idx = 0; idx < n3; idx++) {
    uint32_t b[MAX_DIM];
    bool ok = true;
    int r = idx;
    for (int d = 0; d < dim; d++) {
      const int delta = r % 3;
      r /= 3;
      b[d] = a[d];
      if (delta == 1) { if (a[d] + len >= top) ok = false; else b[d] = (uint32_t) (a[d] + len); }
      else if (delta == 2) { if (a[d] < len) ok = false; else b[d] = (uint32_t) (a[d] - len); }
    }
    out[i * n3 + idx] = ok ? cell_key(b, lev, dim, md) : TSENT;
  }
}

__global__ void k_tunique_flags(const uint64_t *__restrict__ k, uint32_t *__restrict__ f, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) f[i] = (k[i] != TSENT && (i == 0 || k[i] != k[i - 1])) ? 1u : 0u;
}

__global__ void k_children_not_in(const uint64_t *__restrict__ I, int64_t nI, uint64_t *__restrict__ out, int dim,
                                  int md)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nI) return;
  const int nc = 1 << dim;
  uint32_t a[MAX_DIM];
  int lev;
  tdecode(I[i], dim, md, a, lev);
  const uint32_t cl = 1u << (md - lev - 1);
  for (int c = 0; c < nc; c++) {
    uint32_t b[MAX_DIM];
    for (int d = 0; d < dim; d++) b[d] = a[d] | (((c >> d) & 1) ? cl : 0u);
    uint64_t k = cell_key(b, lev + 1, dim, md);
    const int64_t pos = lower_bound_u64(I, nI, k);
    if (pos < nI && I[pos] == k) k = TSENT;
    out[i * nc + c] = k;
  }
}

static void t_sort_unique(DBuf<uint64_t> &keys, int64_t &n, int bits, cudaStream_t s)
{
  if (n == 0) return;
  radix_sort_pairs<uint64_t, uint32_t>(keys.p, nullptr, n, bits, s);
  DBuf<uint32_t> f(n), pos(n);
  k_tunique_flags<<<grid_for(n), 256, 0, s>>>(keys.p, f.p, n);
  check_launch("t_unique");
  const int64_t m = (int64_t) exclusive_scan_total<uint32_t>(f.p, pos.p, n, s);
  DBuf<uint64_t> out(m > 0 ? m : 1);
  scatter_if_kernel<uint64_t><<<grid_for(n), 256, 0, s>>>(keys.p, f.p, pos.p, out.p, n);
  check_launch("t_unique_scatter");
  DKT_CUDA(cudaStreamSynchronize(s));
  keys = std::move(out);
  n = m;
}

static void t_concat(DBuf<uint64_t> &a, int64_t &na, const uint64_t *b, int64_t nb, cudaStream_t s)
{
  DBuf<uint64_t> c(na + nb > 0 ? na + nb : 1);
  if (na) DKT_CUDA(cudaMemcpyAsync(c.p, a.p, na * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
  if (nb) DKT_CUDA(cudaMemcpyAsync(c.p + na, b, nb * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
  DKT_CUDA(cudaStreamSynchronize(s));
  a = std::move(c);
  na += nb;
}

__global__ void k_level_of(const uint64_t *__restrict__ k, uint8_t *__restrict__ lev, int64_t n, int dim, int md)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) lev[i] = (uint8_t) (k[i] >> (dim * md));
}

// Balanced leaves (cell keys) of the complete tree given by `leaves` (keys).
void balance_device(DBuf<uint64_t> &leaves, int64_t &n, int dim, int md, cudaStream_t s)
{
  const int bits = dim * md + 6;
  int n3 = 1;
  for (int d = 0; d < dim; d++) n3 *= 3;
  t_sort_unique(leaves, n, bits, s);
  // split by level (level is the top field of the key, so sorted keys are grouped)
  std::vector<DBuf<uint64_t>> S(md + 1);
  std::vector<int64_t> nS(md + 1, 0);
  {
    std::vector<uint64_t> h(n);
    DKT_CUDA(cudaMemcpyAsync(h.data(), leaves.p, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    DKT_CUDA(cudaStreamSynchronize(s));
    int64_t b = 0;
    for (int l = 0; l <= md; l++) {
      int64_t e = b;
      while (e < n && (int) (h[e] >> (dim * md)) == l) e++;
      nS[l] = e - b;
      if (nS[l]) {
        S[l].alloc(nS[l]);
        DKT_CUDA(cudaMemcpyAsync(S[l].p, leaves.p + b, nS[l] * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
      }
      b = e;
    }
  }
  DBuf<uint64_t> I;
  int64_t nI = 0;
  for (int l = md; l >= 1; l--) {
    if (nS[l] == 0) continue;
    DBuf<uint64_t> P(nS[l]);
    int64_t nP = nS[l];
    k_parents<<<grid_for(nP), 256, 0, s>>>(S[l].p, P.p, nP, dim, md);
    check_launch("parents");
    t_sort_unique(P, nP, bits, s);
    t_concat(I, nI, P.p, nP, s);
    DBuf<uint64_t> N(nP * n3);
    int64_t nN = nP * n3;
    k_neighbourhood<<<grid_for(nP), 256, 0, s>>>(P.p, N.p, nP, dim, md, n3);
    check_launch("neighbourhood");
    t_concat(N, nN, S[l - 1].p, nS[l - 1], s);
    t_sort_unique(N, nN, bits, s);
    S[l - 1] = std::move(N);
    nS[l - 1] = nN;
  }
  t_sort_unique(I, nI, bits, s);
  DBuf<uint64_t> C(nI * (1 << dim));
  int64_t nC = nI * (1 << dim);
  k_children_not_in<<<grid_for(nI), 256, 0, s>>>(I.p, nI, C.p, dim, md);
  check_launch("children_not_in");
  t_sort_unique(C, nC, bits, s);
  leaves = std::move(C);
  n = nC;
}

// ---------------------------------------------------------------------------
// Moving ball (dim 4), refined level by level on the device.  Same test as
// the host generator: exact distance interval of the box to the moving
// centre (golden-section minimum over t, maximum at an end of the t-range).
// ---------------------------------------------------------------------------
__device__ double d_box_dist(const double *lo, const double *hi, const double *c)
{
  double s = 0.0;
  for (int d = 0; d < 3; d++) {
    const double g = c[d] < lo[d] ? __dsub_rn(lo[d], c[d]) : (c[d] > hi[d] ? __dsub_rn(c[d], hi[d]) : 0.0);
    s = __dadd_rn(s, __dmul_rn(g, g));
  }
  return sqrt(s);
}
__device__ double d_box_far(const double *lo, const double *hi, const double *c)
{
  double s = 0.0;
  for (int d = 0; d < 3; d++) {
    const double f = fmax(fabs(__dsub_rn(c[d], lo[d])), fabs(__dsub_rn(hi[d], c[d])));
    s = __dadd_rn(s, __dmul_rn(f, f));
  }
  return sqrt(s);
}
__device__ void d_centre(double t, const double *c0, const double *c1, double *out)
{
  for (int d = 0; d < 3; d++) out[d] = __dadd_rn(c0[d], __dmul_rn(__dsub_rn(c1[d], c0[d]), t));
}

struct BallParams {
  double R, w, c0[3], c1[3];
};

__global__ void k_ball_test(const uint64_t *__restrict__ cells, int64_t n, int md, int level, BallParams bp,
                            uint32_t *__restrict__ refine)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t a[4];
  int lev;
  tdecode(cells[i], 4, md, a, lev);
  const double sc = ldexp(1.0, -md), h = ldexp(1.0, -lev);
  double lo[3], hi[3];
  for (int d = 0; d < 3; d++) { lo[d] = __dmul_rn((double) a[d], sc); hi[d] = __dadd_rn(lo[d], h); }
  const double t0 = __dmul_rn((double) a[3], sc), t1 = __dadd_rn(t0, h);
  double ca[3], cb[3];
  d_centre(t0, bp.c0, bp.c1, ca);
  d_centre(t1, bp.c0, bp.c1, cb);
  const double dmax = fmax(d_box_far(lo, hi, ca), d_box_far(lo, hi, cb));
  double lo_t = t0, hi_t = t1;
  const double gr = 0.5 * (sqrt(5.0) - 1.0);
  for (int it = 0; it < 80; it++) {
    const double m1 = __dsub_rn(hi_t, __dmul_rn(gr, __dsub_rn(hi_t, lo_t)));
    const double m2 = __dadd_rn(lo_t, __dmul_rn(gr, __dsub_rn(hi_t, lo_t)));
    double p1[3], p2[3];
    d_centre(m1, bp.c0, bp.c1, p1);
    d_centre(m2, bp.c0, bp.c1, p2);
    if (d_box_dist(lo, hi, p1) <= d_box_dist(lo, hi, p2)) hi_t = m2; else lo_t = m1;
  }
  double pm[3];
  d_centre(__dmul_rn(0.5, __dadd_rn(lo_t, hi_t)), bp.c0, bp.c1, pm);
  const double dmin = fmin(d_box_dist(lo, hi, pm), fmin(d_box_dist(lo, hi, ca), d_box_dist(lo, hi, cb)));
  const bool meets = (dmin <= bp.R + bp.w) && (dmax >= bp.R - bp.w);
  refine[i] = (meets && lev < level) ? 1u : 0u;
}

__global__ void k_children(const uint64_t *__restrict__ cells, const uint32_t *__restrict__ flag,
                           const uint32_t *__restrict__ pos, uint64_t *__restrict__ out, int64_t n, int dim, int md)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !flag[i]) return;
  const int nc = 1 << dim;
  uint32_t a[MAX_DIM];
  int lev;
  tdecode(cells[i], dim, md, a, lev);
  const uint32_t cl = 1u << (md - lev - 1);
  for (int c = 0; c < nc; c++) {
    uint32_t b[MAX_DIM];
    for (int d = 0; d < dim; d++) b[d] = a[d] | (((c >> d) & 1) ? cl : 0u);
    out[(int64_t) pos[i] * nc + c] = cell_key(b, lev + 1, dim, md);
  }
}

__global__ void k_not_flag(const uint32_t *__restrict__ f, uint32_t *__restrict__ g, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) g[i] = f[i] ? 0u : 1u;
}

// Static sphere shell in dim 2..4: refine every cell of level < `level` whose
// box meets |‖x - c‖ - R| <= w (exact box distance interval).
struct ShellParams {
  double R, w, c[MAX_DIM];
};

__global__ void k_shell_test(const uint64_t *__restrict__ cells, int64_t n, int dim, int md, int level,
                             ShellParams sp, uint32_t *__restrict__ refine)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t a[MAX_DIM];
  int lev;
  tdecode(cells[i], dim, md, a, lev);
  const double sc = ldexp(1.0, -md), h = ldexp(1.0, -lev);
  double s_near = 0.0, s_far = 0.0;
  for (int d = 0; d < dim; d++) {
    const double lo = __dmul_rn((double) a[d], sc), hi = __dadd_rn(lo, h);
    const double g = sp.c[d] < lo ? __dsub_rn(lo, sp.c[d]) : (sp.c[d] > hi ? __dsub_rn(sp.c[d], hi) : 0.0);
    const double f = fmax(fabs(__dsub_rn(sp.c[d], lo)), fabs(__dsub_rn(hi, sp.c[d])));
    s_near = __dadd_rn(s_near, __dmul_rn(g, g));
    s_far = __dadd_rn(s_far, __dmul_rn(f, f));
  }
  const bool meets = (sqrt(s_near) <= sp.R + sp.w) && (sqrt(s_far) >= sp.R - sp.w);
  refine[i] = (meets && lev < level) ? 1u : 0u;
}

// Level-by-level refinement driven by a refine-flag kernel, then 2:1 balance.
template <typename TestFn>
static void refine_device(int dim, int md, TestFn test, DBuf<uint64_t> &out, int64_t &n_out, cudaStream_t s,
                          bool balance = true)
{
  DBuf<uint64_t> frontier(1);
  const uint32_t z[MAX_DIM] = {0, 0, 0, 0};
  const uint64_t root = cell_key(z, 0, dim, md);
  frontier.upload(&root, 1, s);
  int64_t nf = 1;
  DBuf<uint64_t> leaves;
  int64_t nl = 0;
  const int nc = 1 << dim;
  while (nf > 0) {
    DBuf<uint32_t> flag(nf), pos(nf), keep(nf), kpos(nf);
    test(frontier.p, nf, flag.p);
    check_launch("refine_test");
    const int64_t nr = (int64_t) exclusive_scan_total<uint32_t>(flag.p, pos.p, nf, s);
    k_not_flag<<<grid_for(nf), 256, 0, s>>>(flag.p, keep.p, nf);
    const int64_t nk = (int64_t) exclusive_scan_total<uint32_t>(keep.p, kpos.p, nf, s);
    if (nk) {
      DBuf<uint64_t> kept(nk);
      scatter_if_kernel<uint64_t><<<grid_for(nf), 256, 0, s>>>(frontier.p, keep.p, kpos.p, kept.p, nf);
      check_launch("refine_keep");
      t_concat(leaves, nl, kept.p, nk, s);
    }
    DBuf<uint64_t> next(nr * nc > 0 ? nr * nc : 1);
    if (nr) {
      k_children<<<grid_for(nf), 256, 0, s>>>(frontier.p, flag.p, pos.p, next.p, nf, dim, md);
      check_launch("refine_children");
    }
    DKT_CUDA(cudaStreamSynchronize(s));
    frontier = std::move(next);
    nf = nr * nc;
  }
  if (balance) balance_device(leaves, nl, dim, md, s);
  out = std::move(leaves);
  n_out = nl;
}

void sphere_shell_device(int dim, int md, int level, double R, double w, const double *c, DBuf<uint64_t> &out,
                         int64_t &n_out, cudaStream_t s)
{
  if (dim < 2 || dim > MAX_DIM) throw std::invalid_argument("sphere shell: dim must be 2..4");
  ShellParams sp;
  sp.R = R;
  sp.w = w;
  for (int d = 0; d < MAX_DIM; d++) sp.c[d] = d < dim ? c[d] : 0.0;
  refine_device(dim, md, [&](const uint64_t *cells, int64_t n, uint32_t *flag) {
    k_shell_test<<<grid_for(n), 256, 0, s>>>(cells, n, dim, md, level, sp, flag);
  }, out, n_out, s);
}

void moving_ball_device(int md, int level, double R, double w, const double *c0, const double *c1,
                        DBuf<uint64_t> &out, int64_t &n_out, cudaStream_t s)
{
  BallParams bp;
  bp.R = R;
  bp.w = w;
  for (int d = 0; d < 3; d++) { bp.c0[d] = c0[d]; bp.c1[d] = c1[d]; }
  refine_device(4, md, [&](const uint64_t *cells, int64_t n, uint32_t *flag) {
    k_ball_test<<<grid_for(n), 256, 0, s>>>(cells, n, md, level, bp, flag);
  }, out, n_out, s);
}

// Points -> complete tree with at most max_pts points per leaf (the root is
// always split), then 2:1 balanced: SFC_Tree::locTreeBalancing on one rank
// (src/tsort.cpp:826-854).  The points' full-resolution interleaved Morton
// keys are sorted once; a cell's points are the key range of its prefix, so
// each refinement test is two binary searches.
__device__ inline uint64_t morton_full_key(const uint32_t *a, int dim, int md)
{
  uint64_t k = 0;
  for (int bit = md - 1; bit >= 0; bit--)
    for (int d = dim - 1; d >= 0; d--) k = (k << 1) | ((a[d] >> bit) & 1u);
  return k;
}
__global__ void k_point_keys(const uint32_t *__restrict__ pts, int64_t n, int dim, int md, uint64_t *__restrict__ keys)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t a[MAX_DIM];
  for (int d = 0; d < dim; d++) a[d] = pts[i * dim + d];
  keys[i] = morton_full_key(a, dim, md);
}
__device__ inline int64_t first_not_below(const uint64_t *__restrict__ v, int64_t n, uint64_t key)
{
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (v[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}
__global__ void k_count_test(const uint64_t *__restrict__ cells, int64_t n, int dim, int md,
                             const uint64_t *__restrict__ pk, int64_t np, int64_t max_pts, uint32_t *__restrict__ refine)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t a[MAX_DIM];
  int lev;
  tdecode(cells[i], dim, md, a, lev);
  if (lev == 0) { refine[i] = 1u; return; }
  if (lev >= md) { refine[i] = 0u; return; }
  const uint64_t lo = morton_full_key(a, dim, md);
  const int shift = dim * (md - lev);   // < 64: lev >= 1 and dim * md <= 58
  const int64_t b = first_not_below(pk, np, lo);
  const int64_t e = first_not_below(pk, np, lo + (1ull << shift));
  refine[i] = (e - b > max_pts) ? 1u : 0u;
}

void tree_from_points_device(const uint32_t *pts_host, int64_t n, int dim, int md, int64_t max_pts,
                             DBuf<uint64_t> &out, int64_t &n_out, cudaStream_t s)
{
  if (dim < 2 || dim > MAX_DIM || n <= 0 || max_pts < 1) throw std::invalid_argument("tree from points: bad argument");
  DBuf<uint32_t> pts;
  pts.upload(pts_host, (size_t) n * dim, s);
  DBuf<uint64_t> pk(n);
  k_point_keys<<<grid_for(n), 256, 0, s>>>(pts.p, n, dim, md, pk.p);
  check_launch("point_keys");
  radix_sort_pairs<uint64_t, uint32_t>(pk.p, nullptr, (size_t) n, dim * md, s);
  refine_device(dim, md, [&](const uint64_t *cells, int64_t nc, uint32_t *flag) {
    k_count_test<<<grid_for(nc), 256, 0, s>>>(cells, nc, dim, md, pk.p, n, max_pts, flag);
  }, out, n_out, s);
}

// ot::function2Octree (include/octUtils.h:180-417) on the device.  From the
// root's children, level by level up to max_depth, a cell is split when
// interpolating any field from its element nodes (order p) to the element
// nodes of one of its children (IKD_Parent2Child) misses the field's values
// there by more than interp_tol (max norm).  The fields are evaluated by the
// caller on the host, on batches of points: per cell the parent's (p+1)^d
// element nodes, then each child's, in Morton child order, coordinates
// (anchor + len*i/p) / 2^max_depth as the reference forms them.  With
// balance the tree is then 2:1 balanced, as ot::DA<dim>::DA(func, ...)
// does (include/oda.tcc:67-88).
__global__ void k_fill_u32(uint32_t *__restrict__ f, int64_t n, uint32_t v)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) f[i] = v;
}
__global__ void k_f2o_points(const uint64_t *__restrict__ cells, int64_t nc, int dim, int md, int p, int npe,
                             double *__restrict__ pts)
{
  const int64_t idx = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const int per = ((1 << dim) + 1) * npe;
  if (idx >= nc * per) return;
  const int64_t cell = idx / per;
  const int rem = (int) (idx - cell * per), blk = rem / npe, node = rem - blk * npe;
  uint32_t a[MAX_DIM];
  int lev;
  tdecode(cells[cell], dim, md, a, lev);
  uint32_t len = 1u << (md - lev);
  if (blk > 0) {
    len >>= 1;
    for (int d = 0; d < dim; d++) a[d] += (((blk - 1) >> d) & 1) ? len : 0u;
  }
  const double scale = 1.0 / (double) (1u << md);
  int r = node;
  for (int d = 0; d < dim; d++) {
    const uint32_t i = (uint32_t) (r % (p + 1));
    r /= p + 1;
    const uint32_t c = (uint32_t) ((uint64_t) len * i / (uint32_t) p) + a[d];
    pts[idx * dim + d] = scale * (double) c;
  }
}
__global__ void k_f2o_test(int64_t nc, int dim, int p, int npe, const double *__restrict__ vals, int n_vars,
                           const double *__restrict__ ip, double tol, uint32_t *__restrict__ flag)
{
  const int64_t cell = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= nc) return;
  const int M = p + 1, nch = 1 << dim;
  const double *base = vals + cell * (int64_t) (nch + 1) * npe * n_vars;
  uint32_t split = 0u;
  double a[81], b[81];
  for (int c = 0; c < nch && !split; c++) {
    for (int var = 0; var < n_vars && !split; var++) {
      for (int k = 0; k < npe; k++) a[k] = base[(int64_t) k * n_vars + var];
      // parent -> child c along each axis, the last axis first
      for (int ax = dim - 1; ax >= 0; ax--) {
        const double *A = ip + ((c >> ax) & 1) * M * M;
        int stride = 1;
        for (int t = 0; t < ax; t++) stride *= M;
        for (int idx = 0; idx < npe; idx++) {
          const int j = (idx / stride) % M, b0 = idx - j * stride;
          double s = __dmul_rn(A[j], a[b0]);
          for (int k = 1; k < M; k++) s = __dadd_rn(s, __dmul_rn(A[k * M + j], a[b0 + k * stride]));
          b[idx] = s;
        }
        for (int idx = 0; idx < npe; idx++) a[idx] = b[idx];
      }
      const double *cv = base + (int64_t) (1 + c) * npe * n_vars;
      double err = 0.0;
      for (int k = 0; k < npe; k++) err = fmax(err, fabs(__dsub_rn(cv[(int64_t) k * n_vars + var], a[k])));
      if (err > tol) split = 1u;
    }
  }
  flag[cell] = split;
}

void function2octree_device(FieldFn fn, void *user, int n_vars, int dim, int md, int p, double tol, bool balance,
                            DBuf<uint64_t> &out, int64_t &n_out, cudaStream_t s)
{
  if (dim < 2 || dim > MAX_DIM || p < 1 || p > 2 || n_vars < 1 || !fn || md < 1 || dim * md + 6 > 64)
    throw std::invalid_argument("function2octree: bad argument");
  const RefEl1D re = refel_1d(p);
  std::vector<double> iph(re.ip0);
  iph.insert(iph.end(), re.ip1.begin(), re.ip1.end());
  DBuf<double> ip;
  ip.upload(iph.data(), iph.size(), s);
  int npe = 1;
  for (int d = 0; d < dim; d++) npe *= p + 1;
  const int per = ((1 << dim) + 1) * npe;
  const int64_t batch = std::max<int64_t>(1, (int64_t(1) << 22) / per);   // about 4 M points per callback
  refine_device(dim, md, [&](const uint64_t *cells, int64_t n, uint32_t *flag) {
    uint64_t k0 = 0;
    DKT_CUDA(cudaMemcpyAsync(&k0, cells, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    DKT_CUDA(cudaStreamSynchronize(s));
    const int lev = (int) (k0 >> (dim * md));   // a frontier holds one level
    if (lev == 0 || lev >= md) {
      k_fill_u32<<<grid_for(n), 256, 0, s>>>(flag, n, lev == 0 ? 1u : 0u);
      return;
    }
    const int64_t nb_max = std::min<int64_t>(batch, n);
    DBuf<double> pts((size_t) nb_max * per * dim), vals((size_t) nb_max * per * n_vars);
    std::vector<double> hp((size_t) nb_max * per * dim), hv((size_t) nb_max * per * n_vars);
    for (int64_t c0 = 0; c0 < n; c0 += nb_max) {
      const int64_t nb = std::min<int64_t>(nb_max, n - c0), np = nb * per;
      k_f2o_points<<<grid_for(np), 256, 0, s>>>(cells + c0, nb, dim, md, p, npe, pts.p);
      check_launch("f2o_points");
      DKT_CUDA(cudaMemcpyAsync(hp.data(), pts.p, np * dim * sizeof(double), cudaMemcpyDeviceToHost, s));
      DKT_CUDA(cudaStreamSynchronize(s));
      if (fn(hp.data(), np, dim, hv.data(), n_vars, user) != 0)
        throw std::runtime_error("function2octree: the field callback reported an error");
      DKT_CUDA(cudaMemcpyAsync(vals.p, hv.data(), np * n_vars * sizeof(double), cudaMemcpyHostToDevice, s));
      k_f2o_test<<<grid_for(nb, 128), 128, 0, s>>>(nb, dim, p, npe, vals.p, n_vars, ip.p, tol, flag + c0);
      check_launch("f2o_test");
      DKT_CUDA(cudaStreamSynchronize(s));
    }
  }, out, n_out, s, balance);
}

__global__ void k_unpack_cells(const uint64_t *__restrict__ k, uint32_t *__restrict__ x, uint8_t *__restrict__ lev,
                               int64_t n, int dim, int md)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t a[MAX_DIM];
  int l;
  tdecode(k[i], dim, md, a, l);
  for (int d = 0; d < dim; d++) x[i * dim + d] = a[d];
  lev[i] = (uint8_t) l;
}

// Keys -> host arrays (coords [n][dim], levels).
void unpack_cells_to_host(const DBuf<uint64_t> &keys, int64_t n, int dim, int md, uint32_t *coords, uint8_t *levels,
                          cudaStream_t s)
{
  DBuf<uint32_t> x(n * dim > 0 ? n * dim : 1);
  DBuf<uint8_t> l(n > 0 ? n : 1);
  k_unpack_cells<<<grid_for(n), 256, 0, s>>>(keys.p, x.p, l.p, n, dim, md);
  check_launch("unpack_cells");
  DKT_CUDA(cudaMemcpyAsync(coords, x.p, n * dim * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaMemcpyAsync(levels, l.p, n, cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaStreamSynchronize(s));
}

}  // namespace dkt
