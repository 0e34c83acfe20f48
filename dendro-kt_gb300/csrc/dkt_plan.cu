// Flattening of the mesh-free traversal fem::matvec (FEM/include/matvec.h:231-548)
// into a list of leaf visits, computed once per node list.
//
// The reference recurses from the root, duplicating every node into all
// children whose closed cell contains it (top_down, matvec.h:74-199), and
// treats a subtree S as a leaf when no node in its bucket is finer than S
// (matvec.h:101-107).  The bucket of S is therefore exactly the set of nodes in
// the closed cell of S, and S is visited as a leaf iff
//     closed(S) holds a node,  maxlevel(closed(S)) <= lev(S),
//     maxlevel(closed(parent(S))) >= lev(S).
// The non-leaf cells are the ancestors-or-self of the level-(l-1) cells that
// contain a level-l node; leaves are the children of non-leaf cells that are
// not non-leaf themselves and hold a node.  This includes the "virtual" leaves
// the reference creates where a domain-boundary node of a finer element lies on
// a coarser element (boundary sites are never hanging, nsort.tcc:911-926).
//
// Per leaf the plan stores the node of each lexicographic rank (or -1), and
// for leaves with missing ranks the parent's nodes of level L-1
// (matvec.h:411-431) and the leaf fill mask used by the transpose
// (matvec.h:497-521).
#include "dkt_internal.cuh"

namespace dkt {

constexpr uint64_t SENT = ~0ull;

__global__ void k_node_lookup_keys(const uint32_t *__restrict__ nx, uint64_t *__restrict__ key,
                                   uint32_t *__restrict__ idx, int64_t n, int dim, int md)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t x[MAX_DIM];
  for (int d = 0; d < dim; d++) x[d] = nx[i * dim + d];
  key[i] = coord_key(x, dim, md);
  idx[i] = (uint32_t) i;
}

__global__ void k_dup_check(const uint64_t *__restrict__ key, int64_t n, int *__restrict__ flag)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i > 0 && i < n && key[i] == key[i - 1]) atomicExch(flag, 1);
}

// Level-(l-1) cells whose closed cell contains node i (l = node level).
__global__ void k_deep_cells(const uint32_t *__restrict__ nx, const uint8_t *__restrict__ nl,
                             uint64_t *__restrict__ out, int64_t n, int dim, int md)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int nc = 1 << dim;
  const int lev = nl[i];
  for (int j = 0; j < nc; j++) out[i * nc + j] = SENT;
  if (lev < 1) return;
  const int l = lev - 1;
  const uint32_t len = 1u << (md - l), top = 1u << md;
  uint32_t opt[MAX_DIM][2];
  int nopt[MAX_DIM];
  for (int d = 0; d < dim; d++) {
    const uint32_t x = nx[i * dim + d];
    const uint32_t a0 = (x / len) * len;
    nopt[d] = 0;
    if (a0 < top) opt[d][nopt[d]++] = a0;
    if (a0 == x && x > 0) opt[d][nopt[d]++] = a0 - len;
  }
  int combos = 1;
  for (int d = 0; d < dim; d++) combos *= nopt[d];
  for (int c = 0; c < combos; c++) {
    int cc = c;
    uint32_t a[MAX_DIM];
    for (int d = 0; d < dim; d++) { a[d] = opt[d][cc % nopt[d]]; cc /= nopt[d]; }
    out[i * nc + c] = cell_key(a, l, dim, md);
  }
}

__device__ inline void decode_cell(uint64_t k, int dim, int md, uint32_t *a, int &lev)
{
  const uint64_t m = (1ull << md) - 1ull;
  for (int d = 0; d < dim; d++) { a[d] = (uint32_t) (k & m); k >>= md; }
  lev = (int) k;
}

__global__ void k_ancestors(const uint64_t *__restrict__ cells, uint64_t *__restrict__ out, int64_t n, int dim, int md)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t a[MAX_DIM];
  int lev;
  decode_cell(cells[i], dim, md, a, lev);
  for (int l = 0; l <= md; l++) {
    uint64_t k = SENT;
    if (l <= lev) {
      uint32_t b[MAX_DIM];
      const uint32_t mask = ~((1u << (md - l)) - 1u);
      for (int d = 0; d < dim; d++) b[d] = a[d] & mask;
      k = cell_key(b, l, dim, md);
    }
    out[i * (md + 1) + l] = k;
  }
}

__global__ void k_unique_flags(const uint64_t *__restrict__ k, uint32_t *__restrict__ f, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) f[i] = (k[i] != SENT && (i == 0 || k[i] != k[i - 1])) ? 1u : 0u;
}

// Children of non-leaf cells that are not non-leaf themselves.
__global__ void k_leaf_candidates(const uint64_t *__restrict__ nl, int64_t n_nl, uint64_t *__restrict__ out, int dim,
                                  int md)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nl) return;
  const int nc = 1 << dim;
  uint32_t a[MAX_DIM];
  int lev;
  decode_cell(nl[i], dim, md, a, lev);
  for (int c = 0; c < nc; c++) {
    uint64_t k = SENT;
    if (lev < md) {
      uint32_t b[MAX_DIM];
      const uint32_t cl = 1u << (md - lev - 1);
      for (int d = 0; d < dim; d++) b[d] = a[d] | (((c >> d) & 1) ? cl : 0u);
      k = cell_key(b, lev + 1, dim, md);
      const int64_t pos = lower_bound_u64(nl, n_nl, k);
      if (pos < n_nl && nl[pos] == k) k = SENT;
    }
    out[i * nc + c] = k;
  }
}

__device__ inline int32_t find_node(const uint64_t *__restrict__ lk, const uint32_t *__restrict__ li, int64_t n,
                                    const uint32_t *x, int dim, int md)
{
  const uint64_t k = coord_key(x, dim, md);
  const int64_t pos = lower_bound_u64(lk, n, k);
  return (pos < n && lk[pos] == k) ? (int32_t) li[pos] : -1;
}

// Build one leaf record: E2N, fill, parent nodes, stale-slot hazards.
__global__ void k_build_leaves(const uint64_t *__restrict__ cand, int64_t n_cand, const uint64_t *__restrict__ lk,
                               const uint32_t *__restrict__ li, const uint8_t *__restrict__ nlev, int64_t n_nodes,
                               int dim, int md, int p, int npe, const double *__restrict__ ip,
                               int32_t *__restrict__ e2n, int32_t *__restrict__ p2n, uint32_t *__restrict__ fill,
                               uint32_t *__restrict__ info, uint32_t *__restrict__ valid, uint32_t *__restrict__ hang,
                               unsigned long long *__restrict__ stale, int conforming)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_cand) return;
  uint32_t a[MAX_DIM];
  int L;
  decode_cell(cand[i], dim, md, a, L);
  const uint64_t len = 1ull << (md - L);
  uint32_t fm[3] = {0, 0, 0};
  int nfill = 0;
  for (int r = 0; r < npe; r++) {
    uint32_t x[MAX_DIM];
    int rr = r;
    for (int d = 0; d < dim; d++) { const int id = rr % (p + 1); rr /= (p + 1); x[d] = a[d] + (uint32_t) (len * id / p); }
    const int32_t nd = find_node(lk, li, n_nodes, x, dim, md);
    e2n[i * npe + r] = nd;
    if (nd >= 0) { fm[r >> 5] |= 1u << (r & 31); nfill++; }
  }
  const unsigned child = morton_at(a, dim, md, L);
  const bool hanging = nfill > 0 && nfill < npe;
  valid[i] = nfill > 0 ? 1u : 0u;
  hang[i] = hanging ? 1u : 0u;
  info[i] = (uint32_t) L | (child << 8) | ((hanging ? 1u : 0u) << 16);
  for (int w = 0; w < 3; w++) fill[i * 3 + w] = fm[w];
  if (!hanging) return;
  const uint64_t plen = len << 1;
  uint32_t pa[MAX_DIM];
  for (int d = 0; d < dim; d++) pa[d] = a[d] & ~((uint32_t) plen - 1u);
  const int M = p + 1;
  for (int q = 0; q < npe; q++) {
    uint32_t x[MAX_DIM];
    int qq = q;
    for (int d = 0; d < dim; d++) { const int id = qq % M; qq /= M; x[d] = pa[d] + (uint32_t) (plen * id / p); }
    int32_t nd = find_node(lk, li, n_nodes, x, dim, md);
    if (nd >= 0 && !conforming && (int) nlev[nd] != L - 1) nd = -1;
    p2n[i * npe + q] = nd;
    if (nd < 0) {
      // Weight of parent slot q on leaf rank r: prod_d ip_{bit_d}[q_d][r_d].
      bool hazard = false;
      for (int r = 0; r < npe && !hazard; r++) {
        if ((fm[r >> 5] >> (r & 31)) & 1u) continue;
        double w = 1.0;
        int rr = r, q2 = q;
        for (int d = 0; d < dim; d++) {
          const int rd = rr % M, qd = q2 % M;
          rr /= M; q2 /= M;
          w *= ip[((child >> d) & 1) * M * M + qd * M + rd];
        }
        hazard = (w != 0.0);
      }
      if (hazard) atomicAdd(stale, 1ull);
    }
  }
}

__global__ void k_leaf_sfc_keys(const uint64_t *__restrict__ cells, uint64_t *__restrict__ key, uint32_t *__restrict__ idx,
                                int64_t n, int dim, int md, CurveDev cv)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t a[MAX_DIM];
  int lev;
  decode_cell(cells[i], dim, md, a, lev);
  key[i] = tree_key(a, lev, dim, md, cv);
  idx[i] = (uint32_t) i;
}

// Final SoA layout in SFC leaf order.
__global__ void k_layout(const uint32_t *__restrict__ order, const uint32_t *__restrict__ vidx,
                         const int32_t *__restrict__ e2n_t, const int32_t *__restrict__ p2n_t,
                         const uint32_t *__restrict__ fill_t, const uint32_t *__restrict__ info_t,
                         const uint32_t *__restrict__ hpos, int64_t n_leaf, int64_t n_hang, int npe,
                         int32_t *__restrict__ e2n, uint32_t *__restrict__ info, int32_t *__restrict__ hidx,
                         int32_t *__restrict__ p2n, uint32_t *__restrict__ fill)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_leaf) return;
  const int64_t c = vidx[order[i]];   // candidate index
  const uint32_t inf = info_t[c];
  info[i] = inf;
  for (int r = 0; r < npe; r++) e2n[(int64_t) i * npe + r] = e2n_t[c * npe + r];
  if ((inf >> 16) & 1u) {
    const int64_t h = hpos[i];
    hidx[i] = (int32_t) h;
    for (int q = 0; q < npe; q++) p2n[(int64_t) h * npe + q] = p2n_t[c * npe + q];
    for (int w = 0; w < 3; w++) fill[(int64_t) h * 3 + w] = fill_t[c * 3 + w];
  } else {
    hidx[i] = -1;
  }
}

__global__ void k_hang_flags(const uint32_t *__restrict__ order, const uint32_t *__restrict__ vidx,
                             const uint32_t *__restrict__ info_t, uint32_t *__restrict__ f, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) f[i] = (info_t[vidx[order[i]]] >> 16) & 1u;
}

__global__ void k_iota_plan(uint32_t *__restrict__ v, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (uint32_t) i;
}

template <typename T>
static void sort_unique(DBuf<uint64_t> &keys, int64_t &n, int bits, cudaStream_t s)
{
  radix_sort_pairs<uint64_t, uint32_t>(keys.p, nullptr, n, bits, s);
  DBuf<uint32_t> f(n), pos(n);
  k_unique_flags<<<grid_for(n), 256, 0, s>>>(keys.p, f.p, n);
  check_launch("unique_flags");
  const int64_t m = (int64_t) exclusive_scan_total<uint32_t>(f.p, pos.p, n, s);
  DBuf<uint64_t> out(m > 0 ? m : 1);
  scatter_if_kernel<uint64_t><<<grid_for(n), 256, 0, s>>>(keys.p, f.p, pos.p, out.p, n);
  check_launch("unique_scatter");
  DKT_CUDA(cudaStreamSynchronize(s));
  keys = std::move(out);
  n = m;
}

void build_plan(Plan &pl, const uint32_t *node_x, const uint8_t *node_lev, int64_t n_nodes, const CurveHost &cv,
                const double *ip_host, cudaStream_t s)
{
  const int dim = pl.dim, md = pl.md, p = pl.order, nc = 1 << dim;
  int npe = 1;
  for (int d = 0; d < dim; d++) npe *= (p + 1);
  pl.npe = npe;
  pl.n_nodes = n_nodes;
  if (dim * md + 6 > 64) throw std::runtime_error("max_depth too large for dim (cell key > 64 bits)");
  if (n_nodes <= 0) throw std::runtime_error("empty node list");
  // Node lookup table.
  DBuf<uint64_t> lk(n_nodes);
  DBuf<uint32_t> li(n_nodes);
  k_node_lookup_keys<<<grid_for(n_nodes), 256, 0, s>>>(node_x, lk.p, li.p, n_nodes, dim, md);
  check_launch("lookup_keys");
  radix_sort_pairs<uint64_t, uint32_t>(lk.p, li.p, n_nodes, dim * (md + 1), s);
  {
    DBuf<int> flag(1);
    DKT_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), s));
    k_dup_check<<<grid_for(n_nodes), 256, 0, s>>>(lk.p, n_nodes, flag.p);
    int h = 0;
    DKT_CUDA(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    DKT_CUDA(cudaStreamSynchronize(s));
    if (h) throw std::runtime_error("node list has repeated coordinates");
  }
  // Non-leaf cells.
  int64_t n_deep = n_nodes * nc;
  DBuf<uint64_t> deep(n_deep);
  k_deep_cells<<<grid_for(n_nodes), 256, 0, s>>>(node_x, node_lev, deep.p, n_nodes, dim, md);
  check_launch("deep_cells");
  sort_unique<uint64_t>(deep, n_deep, dim * md + 6, s);
  DBuf<uint64_t> cand;
  int64_t n_cand = 0;
  if (n_deep == 0) {
    // Every node is at level 0: the root is the only leaf.
    uint32_t z[MAX_DIM] = {0, 0, 0, 0};
    const uint64_t rk = cell_key(z, 0, dim, md);
    cand.alloc(1);
    cand.upload(&rk, 1, s);
    n_cand = 1;
  } else {
    int64_t n_anc = n_deep * (md + 1);
    DBuf<uint64_t> anc(n_anc);
    k_ancestors<<<grid_for(n_deep), 256, 0, s>>>(deep.p, anc.p, n_deep, dim, md);
    check_launch("ancestors");
    deep.free();
    sort_unique<uint64_t>(anc, n_anc, dim * md + 6, s);
    int64_t n_c = n_anc * nc;
    DBuf<uint64_t> ck(n_c);
    k_leaf_candidates<<<grid_for(n_anc), 256, 0, s>>>(anc.p, n_anc, ck.p, dim, md);
    check_launch("leaf_candidates");
    anc.free();
    sort_unique<uint64_t>(ck, n_c, dim * md + 6, s);
    cand = std::move(ck);
    n_cand = n_c;
  }
  // Leaf records per candidate.
  const int M = p + 1;
  DBuf<double> ipd(2 * M * M);
  ipd.upload(ip_host, 2 * M * M, s);
  DBuf<int32_t> e2n_t(n_cand * npe), p2n_t(n_cand * npe);
  DBuf<uint32_t> fill_t(n_cand * 3), info_t(n_cand), valid(n_cand), hang(n_cand);
  DBuf<unsigned long long> stale(1);
  DKT_CUDA(cudaMemsetAsync(stale.p, 0, sizeof(unsigned long long), s));
  k_build_leaves<<<grid_for(n_cand, 128), 128, 0, s>>>(cand.p, n_cand, lk.p, li.p, node_lev, n_nodes, dim, md, p, npe,
                                                  ipd.p, e2n_t.p, p2n_t.p, fill_t.p, info_t.p, valid.p, hang.p,
                                                  stale.p, pl.conforming ? 1 : 0);
  check_launch("build_leaves");
  unsigned long long st = 0;
  DKT_CUDA(cudaMemcpyAsync(&st, stale.p, sizeof(st), cudaMemcpyDeviceToHost, s));
  // Compact valid leaves and order them along the SFC.
  DBuf<uint32_t> vpos(n_cand), vidx(n_cand), iota(n_cand);
  const int64_t n_leaf = (int64_t) exclusive_scan_total<uint32_t>(valid.p, vpos.p, n_cand, s);
  k_iota_plan<<<grid_for(n_cand), 256, 0, s>>>(iota.p, n_cand);
  scatter_if_kernel<uint32_t><<<grid_for(n_cand), 256, 0, s>>>(iota.p, valid.p, vpos.p, vidx.p, n_cand);
  DBuf<uint64_t> lcells(n_leaf);
  scatter_if_kernel<uint64_t><<<grid_for(n_cand), 256, 0, s>>>(cand.p, valid.p, vpos.p, lcells.p, n_cand);
  check_launch("leaf_compact");
  DBuf<uint64_t> skey(n_leaf);
  DBuf<uint32_t> order(n_leaf);
  k_leaf_sfc_keys<<<grid_for(n_leaf), 256, 0, s>>>(lcells.p, skey.p, order.p, n_leaf, dim, md, cv.dev());
  check_launch("leaf_keys");
  radix_sort_pairs<uint64_t, uint32_t>(skey.p, order.p, n_leaf, md * slot_bits(dim), s);
  DBuf<uint32_t> hf(n_leaf), hpos(n_leaf);
  k_hang_flags<<<grid_for(n_leaf), 256, 0, s>>>(order.p, vidx.p, info_t.p, hf.p, n_leaf);
  check_launch("hang_flags");
  const int64_t n_hang = (int64_t) exclusive_scan_total<uint32_t>(hf.p, hpos.p, n_leaf, s);
  pl.n_leaf = n_leaf;
  pl.n_hang = n_hang;
  pl.stale_slots = (int64_t) st;
  pl.e2n.alloc((size_t) npe * n_leaf);
  pl.info.alloc(n_leaf);
  pl.hidx.alloc(n_leaf);
  pl.p2n.alloc((size_t) npe * (n_hang > 0 ? n_hang : 1));
  pl.fill.alloc((size_t) 3 * (n_hang > 0 ? n_hang : 1));
  k_layout<<<grid_for(n_leaf), 256, 0, s>>>(order.p, vidx.p, e2n_t.p, p2n_t.p, fill_t.p, info_t.p, hpos.p, n_leaf,
                                            n_hang, npe, pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.fill.p);
  check_launch("layout");
  DKT_CUDA(cudaStreamSynchronize(s));
  pl.ip.alloc(2 * M * M);
  pl.ip.upload(ip_host, 2 * M * M, s);
}

}  // namespace dkt
