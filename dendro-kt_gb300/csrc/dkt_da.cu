// DA construction on the GPU: SFC sort of the tree, CG node generation,
// deduplication / hanging-node resolution, and the reference's DA node order.
//
// Replaces ot::DA<dim>::construct (src/oda.cpp:52-151) on one rank, which
// calls Element::appendExteriorNodes (include/nsort.tcc:360-389),
// SFC_NodeSort::countCGNodes (include/nsort.tcc:878-944, low-order resolver
// :1266-1313) and appendInteriorNodes (:336-358).  The reference's recursive
// bucketing is replaced by keys + radix sorts:
//   * sites: all generated points sorted by (coordinates, level); each run of
//     equal coordinates is one site, resolved exactly as scanForDuplicates +
//     resolveInterface_lowOrder do (boundary sites always kept, mixed levels
//     keep the coarsest, same-level sites kept iff 2^(dim-cdim) instances);
//   * order: selected sites sorted by a 128-bit key equal to the order
//     countCGNodes produces (post-order of the finest open container, then
//     hyperplane, then SFC point digits; domain-boundary sites last, keyed by
//     the root bucket and point digits).
#include "dkt_internal.cuh"

namespace dkt {

__global__ void k_tree_keys(const uint32_t *__restrict__ ex, const uint8_t *__restrict__ el, uint64_t *__restrict__ key,
                            uint32_t *__restrict__ idx, int64_t n, int dim, int md, CurveDev cv)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t x[MAX_DIM];
  for (int d = 0; d < dim; d++) x[d] = ex[i * dim + d];
  key[i] = tree_key(x, el[i], dim, md, cv);
  idx[i] = (uint32_t) i;
}

template <typename T>
__global__ void k_gather_rows(const T *__restrict__ in, T *__restrict__ out, const uint32_t *__restrict__ perm,
                              int64_t n, int w)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t s = perm[i];
  for (int c = 0; c < w; c++) out[i * w + c] = in[s * w + c];
}

// Exterior nodes of each element (Element::appendExteriorNodes), as site keys:
// coord_key << 5 | level.
__global__ void k_exterior_sites(const uint32_t *__restrict__ ex, const uint8_t *__restrict__ el,
                                 uint64_t *__restrict__ site, int64_t n_elem, int dim, int md, int p, int n_ext)
{
  const int64_t t = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_elem * n_ext) return;
  const int64_t e = t / n_ext;
  const int j = (int) (t - e * n_ext);
  const int lev = el[e];
  const uint64_t len = 1ull << (md - lev);
  // j-th exterior lattice index in lexicographic order (x fastest)
  int cnt = -1;
  int idx[MAX_DIM] = {0, 0, 0, 0};
  int npe = 1;
  for (int d = 0; d < dim; d++) npe *= (p + 1);
  for (int r = 0; r < npe; r++) {
    int rr = r, ext = 0;
    int tmp[MAX_DIM];
    for (int d = 0; d < dim; d++) { tmp[d] = rr % (p + 1); rr /= (p + 1); ext |= (tmp[d] == 0 || tmp[d] == p); }
    if (ext && ++cnt == j) { for (int d = 0; d < dim; d++) idx[d] = tmp[d]; break; }
  }
  uint32_t x[MAX_DIM];
  for (int d = 0; d < dim; d++) x[d] = (uint32_t) (len * (uint64_t) idx[d] / (uint64_t) p) + ex[e * dim + d];
  site[t] = (coord_key(x, dim, md) << 5) | (uint64_t) lev;
}

__global__ void k_site_heads(const uint64_t *__restrict__ site, uint32_t *__restrict__ head, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) head[i] = (i == 0 || (site[i] >> 5) != (site[i - 1] >> 5)) ? 1u : 0u;
}

__global__ void k_run_starts(const uint32_t *__restrict__ head, const uint32_t *__restrict__ runid,
                             uint32_t *__restrict__ start, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && head[i]) start[runid[i]] = (uint32_t) i;
}

__device__ inline void decode_coords(uint64_t ck, int dim, int md, uint32_t *x)
{
  const uint64_t mask = (1ull << (md + 1)) - 1ull;
  for (int d = 0; d < dim; d++) { x[d] = (uint32_t) (ck & mask); ck >>= (md + 1); }
}

// Resolve each site and build its DA-order key.
__global__ void k_resolve_sites(const uint64_t *__restrict__ site, const uint32_t *__restrict__ start,
                                int64_t n_runs, int64_t n_pts, int dim, int md, CurveDev cv, int W,
                                uint32_t *__restrict__ sel, Key128 *__restrict__ dakey,
                                uint64_t *__restrict__ node_out)
{
  const int64_t r = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_runs) return;
  const int64_t s = start[r];
  const int64_t e = (r + 1 < n_runs) ? (int64_t) start[r + 1] : n_pts;
  const uint64_t k0 = site[s];
  const int minLev = (int) (k0 & 31u), maxLev = (int) (site[e - 1] & 31u);
  uint32_t x[MAX_DIM];
  decode_coords(k0 >> 5, dim, md, x);
  const uint32_t top = 1u << md;
  bool bdry = false;
  for (int d = 0; d < dim; d++) bdry |= (x[d] == 0u || x[d] == top);
  bool keep;
  if (bdry || minLev != maxLev) keep = true;
  else {
    const uint32_t m = (1u << (md - minLev)) - 1u;
    int cdim = 0;
    for (int d = 0; d < dim; d++) cdim += (x[d] & m) != 0u;
    keep = (e - s) == (int64_t) (1u << (dim - cdim));
  }
  sel[r] = keep ? 1u : 0u;
  node_out[r] = (k0 >> 5 << 5) | (uint64_t) minLev;
  if (!keep) { dakey[r] = Key128{0, 0}; return; }
  const int nc = 1 << dim, B = slot_bits(dim);
  KeyBuilder kb;
  if (!bdry) {
    // finest open container level (TNPoint::getFinestOpenContainer, nsort.tcc:203-230)
    int hmax = 0;
    for (int d = 0; d < dim; d++) { const int lo = __ffs(x[d]) - 1; if (lo > hmax) hmax = lo; }
    const int Lc = md - hmax - 1;
    // hyperplane (get_firstIncidentHyperplane(Lc+1), nsort.tcc:137-151)
    const uint32_t hm = (1u << (md - Lc - 1)) - 1u;
    int h = dim;
    for (int d = dim - 1; d >= 0; d--) if ((x[d] & hm) == 0u) h = d;
    unsigned dig[32];
    int rr = 0;
    for (int l = 1; l <= md; l++) {
      const unsigned m = morton_at(x, dim, md, l);
      dig[l] = (unsigned) cv.rot[rr * 2 * nc + nc + m];
      rr = cv.ht[rr * nc + m];
    }
    kb.push(0, 1);
    for (int l = 1; l <= md; l++) kb.push(l <= Lc ? dig[l] : (l == Lc + 1 ? (unsigned) nc : 0u), B);
    kb.push((uint64_t) h, 2);
    for (int l = 1; l <= md; l++) kb.push(dig[l], dim);
  } else {
    const unsigned m0 = morton_at(x, dim, md, 0);
    kb.push(1, 1);
    kb.push((uint64_t) cv.rot[nc + m0], dim);
    int rr = 0;
    for (int l = 1; l <= md; l++) {
      const unsigned m = morton_at(x, dim, md, l);
      kb.push((uint64_t) cv.rot[rr * 2 * nc + nc + m], dim);
      rr = cv.ht[rr * nc + m];
    }
  }
  dakey[r] = kb.finish(W);
}

__global__ void k_emit_nodes(const uint64_t *__restrict__ node_code, const uint32_t *__restrict__ order,
                             uint32_t *__restrict__ nx, uint8_t *__restrict__ nl, int64_t n, int dim, int md)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t c = node_code[order[i]];
  uint32_t x[MAX_DIM];
  decode_coords(c >> 5, dim, md, x);
  for (int d = 0; d < dim; d++) nx[i * dim + d] = x[d];
  nl[i] = (uint8_t) (c & 31u);
}

// Element-interior nodes (order >= 2), appended in tree order.
__global__ void k_interior_nodes(const uint32_t *__restrict__ ex, const uint8_t *__restrict__ el,
                                 uint32_t *__restrict__ nx, uint8_t *__restrict__ nl, int64_t n_elem, int dim,
                                 int md, int p, int n_int)
{
  const int64_t t = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_elem * n_int) return;
  const int64_t e = t / n_int;
  int j = (int) (t - e * n_int);
  const int lev = el[e];
  const uint64_t len = 1ull << (md - lev);
  for (int d = 0; d < dim; d++) {
    const int id = j % (p - 1);
    j /= (p - 1);
    nx[t * dim + d] = (uint32_t) (len * (uint64_t) (id + 1) / (uint64_t) p) + ex[e * dim + d];
  }
  nl[t] = (uint8_t) lev;
}

__global__ void k_bdry_flags(const uint32_t *__restrict__ nx, uint32_t *__restrict__ flag, int64_t n, int dim, int md)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t mask = (1u << md) - 1u;
  bool b = false;
  for (int d = 0; d < dim; d++) b |= (nx[i * dim + d] & mask) == 0u;
  flag[i] = b ? 1u : 0u;
}

__global__ void k_iota(uint32_t *__restrict__ v, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (uint32_t) i;
}

// Boundary node ids of a node list (oda.cpp:145-150).
void boundary_ids(const uint32_t *nx, int64_t n, int dim, int md, DBuf<uint32_t> &out, int64_t &nb, cudaStream_t s)
{
  DBuf<uint32_t> flag(n), pos(n), ids(n);
  k_bdry_flags<<<grid_for(n), 256, 0, s>>>(nx, flag.p, n, dim, md);
  check_launch("bdry_flags");
  k_iota<<<grid_for(n), 256, 0, s>>>(ids.p, n);
  nb = (int64_t) exclusive_scan_total<uint32_t>(flag.p, pos.p, n, s);
  out.alloc(nb > 0 ? nb : 1);
  scatter_if_kernel<uint32_t><<<grid_for(n), 256, 0, s>>>(ids.p, flag.p, pos.p, out.p, n);
  check_launch("bdry_scatter");
  DKT_CUDA(cudaStreamSynchronize(s));
}

int key_width_interior(int dim, int md) { return 1 + md * slot_bits(dim) + 2 + md * dim; }

// Sort a tree (element anchors + levels) into SFC order on the device.
void sort_tree(DA &da, cudaStream_t s)
{
  const int64_t n = da.n_elem;
  const int dim = da.dim;
  DBuf<uint64_t> key(n);
  DBuf<uint32_t> idx(n);
  k_tree_keys<<<grid_for(n), 256, 0, s>>>(da.elem_x.p, da.elem_lev.p, key.p, idx.p, n, dim, da.md, da.cv.dev());
  check_launch("tree_keys");
  radix_sort_pairs<uint64_t, uint32_t>(key.p, idx.p, n, da.md * slot_bits(dim), s);
  DBuf<uint32_t> x2(n * dim);
  DBuf<uint8_t> l2(n);
  k_gather_rows<uint32_t><<<grid_for(n), 256, 0, s>>>(da.elem_x.p, x2.p, idx.p, n, dim);
  k_gather_rows<uint8_t><<<grid_for(n), 256, 0, s>>>(da.elem_lev.p, l2.p, idx.p, n, 1);
  check_launch("tree_gather");
  DKT_CUDA(cudaStreamSynchronize(s));
  da.elem_x = std::move(x2);
  da.elem_lev = std::move(l2);
}

void build_da_nodes(DA &da, cudaStream_t s)
{
  const int dim = da.dim, md = da.md, p = da.order;
  if (dim * (md + 1) + 5 > 64) throw std::runtime_error("max_depth too large for dim (site key > 64 bits)");
  if (key_width_interior(dim, md) > 128) throw std::runtime_error("max_depth too large for dim (DA key > 128 bits)");
  int npe = 1, nin = 1;
  for (int d = 0; d < dim; d++) { npe *= (p + 1); nin *= (p - 1); }
  const int n_ext = npe - (p >= 2 ? nin : 0);
  const int64_t n_pts = da.n_elem * n_ext;
  DBuf<uint64_t> site(n_pts);
  k_exterior_sites<<<grid_for(n_pts), 256, 0, s>>>(da.elem_x.p, da.elem_lev.p, site.p, da.n_elem, dim, md, p, n_ext);
  check_launch("exterior_sites");
  radix_sort_pairs<uint64_t, uint32_t>(site.p, nullptr, n_pts, dim * (md + 1) + 5, s);
  DBuf<uint32_t> head(n_pts), runid(n_pts);
  k_site_heads<<<grid_for(n_pts), 256, 0, s>>>(site.p, head.p, n_pts);
  check_launch("site_heads");
  const int64_t n_runs = (int64_t) exclusive_scan_total<uint32_t>(head.p, runid.p, n_pts, s);
  DBuf<uint32_t> start(n_runs);
  k_run_starts<<<grid_for(n_pts), 256, 0, s>>>(head.p, runid.p, start.p, n_pts);
  check_launch("run_starts");
  head.free();
  runid.free();
  DBuf<uint32_t> sel(n_runs), pos(n_runs);
  DBuf<Key128> dakey(n_runs);
  DBuf<uint64_t> code(n_runs);
  const int W = key_width_interior(dim, md);
  k_resolve_sites<<<grid_for(n_runs), 256, 0, s>>>(site.p, start.p, n_runs, n_pts, dim, md, da.cv.dev(), W, sel.p,
                                                    dakey.p, code.p);
  check_launch("resolve_sites");
  site.free();
  const int64_t n_sel = (int64_t) exclusive_scan_total<uint32_t>(sel.p, pos.p, n_runs, s);
  DBuf<Key128> skey(n_sel);
  DBuf<uint32_t> sidx(n_sel), ridx(n_runs);
  k_iota<<<grid_for(n_runs), 256, 0, s>>>(ridx.p, n_runs);
  scatter_if_kernel<Key128><<<grid_for(n_runs), 256, 0, s>>>(dakey.p, sel.p, pos.p, skey.p, n_runs);
  scatter_if_kernel<uint32_t><<<grid_for(n_runs), 256, 0, s>>>(ridx.p, sel.p, pos.p, sidx.p, n_runs);
  check_launch("select");
  radix_sort_pairs<Key128, uint32_t>(skey.p, sidx.p, n_sel, W, s);
  const int64_t n_int = (p >= 2) ? da.n_elem * nin : 0;
  da.n_nodes = n_sel + n_int;
  da.node_x.alloc(da.n_nodes * dim);
  da.node_lev.alloc(da.n_nodes);
  k_emit_nodes<<<grid_for(n_sel), 256, 0, s>>>(code.p, sidx.p, da.node_x.p, da.node_lev.p, n_sel, dim, md);
  check_launch("emit_nodes");
  if (n_int > 0) {
    k_interior_nodes<<<grid_for(n_int), 256, 0, s>>>(da.elem_x.p, da.elem_lev.p, da.node_x.p + n_sel * dim,
                                                      da.node_lev.p + n_sel, da.n_elem, dim, md, p, nin);
    check_launch("interior_nodes");
  }
  boundary_ids(da.node_x.p, da.n_nodes, dim, md, da.bdry, da.n_bdry, s);
  DKT_CUDA(cudaStreamSynchronize(s));
}

}  // namespace dkt
