// Tiled Q1 leaf kernel.
//
// The flattened traversal is cut into tiles of T consecutive leaves (SFC
// order).  Once per plan, every tile gets the sorted list of the distinct
// nodes its leaves touch (own nodes and, for hanging leaves, parent nodes)
// and 16-bit tile-local copies of the element-to-node and parent-to-node
// maps.  Per product, one CTA per tile
//   1. gathers the tile's node values into shared memory (one global read per
//      distinct node instead of one per leaf slot),
//   2. runs one thread per leaf entirely in registers: parent interpolation,
//      Walsh-Hadamard transform along every axis, per-mode scaling, inverse
//      transform, transpose of the interpolation -- no warp shuffles,
//   3. accumulates into a shared-memory copy of the tile's output and
//   4. flushes it with one global atomic per distinct node, or a plain store
//      for nodes that no other tile touches.
// SFC locality makes a tile's node set small (about two nodes per 4D leaf),
// so global gathers and atomics drop from ~2*2^dim per leaf to ~2, and the
// 16-bit maps halve the map bytes.
//
// Hanging leaves are stored reflected to child 0: the maps of a leaf with
// Morton child number c list rank k ^ c at position k (and its fill mask is
// permuted the same way).  The element matrix of a cube is invariant under
// reflections, so the product is unchanged, while the parent interpolation
// and its transpose always take the child-0 form -- no per-axis selects.
// Fixed point stays deterministic; in reflected coordinates some Hadamard
// modes change sign, so individual roundings of the mode scaling may differ
// by one unit (2^-50 of max|x|) from the per-leaf kernel.
#include <algorithm>
#include <type_traits>
#include "dkt_internal.cuh"
#include "dkt_q1.cuh"

namespace dkt {

constexpr uint16_t TL_NONE = 0xFFFFu;
// A tile's node entry: node id (bits 0-26), the node's fixed-point unit level
// (bits 27-30, see Plan::fx_lam) and the exclusive flag (bit 31: no other
// tile touches the node).
constexpr uint32_t TL_EXCL = 0x80000000u;
constexpr uint32_t TL_ID = 0x07FFFFFFu;
constexpr int TL_LAM = 27;
constexpr int TL_SINKS = 32;   // sink entries past a tile's nodes, one per lane

// ---------------------------------------------------------------------------
// Plan-time tile build: one CTA per tile sorts the tile's (node, slot) pairs
// in shared memory (bitonic), marks the distinct nodes and ranks them.
//   mode 0: count the distinct nodes per tile and, per node, the tiles that
//           touch it;
//   mode 1: write the node list (with the exclusive flag) and the local maps.
// Slot s < T*npe is rank s%npe of local leaf s/npe; slot T*npe + j*npe + q is
// parent slot q of local leaf j (hanging leaves only).
// ---------------------------------------------------------------------------
constexpr int TB_THREADS = 512;

__global__ void __launch_bounds__(TB_THREADS) k_tile_build(
    int mode, const int32_t *__restrict__ e2n, const uint32_t *__restrict__ info, const int32_t *__restrict__ hidx,
    const int32_t *__restrict__ p2n, int64_t n_leaf, int npe, int T, int cap, uint32_t *__restrict__ node_tiles,
    uint32_t *__restrict__ tile_cnt, const int64_t *__restrict__ tile_off, uint32_t *__restrict__ tile_nodes,
    uint16_t *__restrict__ e2l, uint16_t *__restrict__ p2l, const uint8_t *__restrict__ lam)
// (mode 1 writes the maps of hanging leaves reflected: rank r at position r ^ c)
{
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t *key = reinterpret_cast<uint64_t *>(smem);            // [cap]
  __shared__ uint32_t part[TB_THREADS];
  const int64_t tile = blockIdx.x;
  const int64_t l0 = tile * T;
  const int nl = (int) (n_leaf - l0 < T ? n_leaf - l0 : T);
  for (int s = threadIdx.x; s < cap; s += TB_THREADS) {
    int32_t node = -1;
    const int half = T * npe;
    if (s < half) {
      const int j = s / npe;
      if (j < nl) node = e2n[(l0 + j) * npe + s % npe];
    } else {
      const int j = (s - half) / npe;
      if (j < nl && ((info[l0 + j] >> 16) & 1u)) node = p2n[(int64_t) hidx[l0 + j] * npe + (s - half) % npe];
    }
    key[s] = node >= 0 ? (((uint64_t) (uint32_t) node << 32) | (uint32_t) s) : ~0ull;
  }
  __syncthreads();
  // bitonic sort, ascending
  for (int k = 2; k <= cap; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < cap; i += TB_THREADS) {
        const int p = i ^ j;
        if (p > i) {
          const uint64_t a = key[i], b = key[p];
          const bool up = (i & k) == 0;
          if ((a > b) == up) { key[i] = b; key[p] = a; }
        }
      }
      __syncthreads();
    }
  }
  // distinct-node ranks: each thread owns a contiguous run of cap/TB_THREADS keys
  const int per = cap / TB_THREADS;   // cap is a multiple of TB_THREADS
  const int b0 = threadIdx.x * per;
  uint32_t cnt = 0;
  for (int k = b0; k < b0 + per; k++) {
    const uint64_t a = key[k];
    if (a != ~0ull && (k == 0 || (key[k - 1] >> 32) != (a >> 32))) cnt++;
  }
  part[threadIdx.x] = cnt;
  __syncthreads();
  // inclusive scan of part (Hillis-Steele)
  for (int o = 1; o < TB_THREADS; o <<= 1) {
    const uint32_t v = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  const uint32_t total = part[TB_THREADS - 1];
  uint32_t rank = part[threadIdx.x] - cnt;   // heads before this run
  if (mode == 0 && threadIdx.x == 0) tile_cnt[tile] = total;
  const int64_t base = mode == 1 ? tile_off[tile] : 0;
  for (int k = b0; k < b0 + per; k++) {
    const uint64_t a = key[k];
    if (a == ~0ull) break;
    const uint32_t node = (uint32_t) (a >> 32);
    const bool head = (k == 0 || (key[k - 1] >> 32) != (a >> 32));
    if (head) {
      rank++;
      if (mode == 0) atomicAdd(node_tiles + node, 1u);
      else
        tile_nodes[base + rank - 1] = node | (node_tiles[node] == 1u ? TL_EXCL : 0u) |
                                      (lam ? ((uint32_t) lam[node] & 15u) << TL_LAM : 0u);
    }
    if (mode == 1) {
      const int s = (int) (uint32_t) a;
      const int half = T * npe;
      const uint16_t lr = (uint16_t) (rank - 1);
      if (s < half) {
        const int j = s / npe;
        const uint32_t inf = info[l0 + j];
        const int c = ((inf >> 16) & 1u) ? (int) ((inf >> 8) & 0xFFu) : 0;
        e2l[(l0 + j) * npe + ((s % npe) ^ c)] = lr;
      } else {
        const int j = (s - half) / npe;
        const int c = (int) ((info[l0 + j] >> 8) & 0xFFu);
        p2l[(int64_t) hidx[l0 + j] * npe + (((s - half) % npe) ^ c)] = lr;
      }
    }
  }
}

// Within every tile, hanging leaves first (stable): the warps of a tile then
// run mostly one code path (a hanging leaf does the interpolation and its
// transpose, about half again the work).  Leaf order does not matter to the
// product (integer sums); the hanging records stay indexed by h.
__global__ void k_tile_partition(const int32_t *__restrict__ e2n, const uint32_t *__restrict__ info,
                                 const int32_t *__restrict__ hidx, int32_t *__restrict__ e2n_o,
                                 uint32_t *__restrict__ info_o, int32_t *__restrict__ hidx_o, int64_t n_leaf, int T,
                                 int npe, int32_t *__restrict__ sfc_o)
{
  __shared__ uint32_t wc[32];
  const int64_t l0 = (int64_t) blockIdx.x * T;
  const int64_t i = l0 + threadIdx.x;
  const bool valid = i < n_leaf;
  const int nl = (int) (n_leaf - l0 < T ? n_leaf - l0 : T);
  const bool hang = valid && ((info[i] >> 16) & 1u);
  const unsigned m = __ballot_sync(0xffffffffu, hang);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) wc[w] = __popc(m);
  __syncthreads();
  uint32_t before = __popc(m & ((1u << lane) - 1u)), total = 0;
  for (int k = 0; k < (int) (blockDim.x >> 5); k++) {
    if (k < w) before += wc[k];
    total += wc[k];
  }
  if (!valid) return;
  const int64_t j = l0 + (hang ? (int64_t) before : (int64_t) total + (threadIdx.x - before));
  (void) nl;
  for (int k = 0; k < npe; k++) e2n_o[j * npe + k] = e2n[i * npe + k];
  info_o[j] = info[i];
  hidx_o[j] = hidx[i];
  sfc_o[j] = (int32_t) i;   // the input is in traversal order
}
// Leaf records back to the traversal order (record i to position sfc[i]),
// so that a plan tiled again is partitioned from that order: tiles then hold
// consecutive leaves whatever tile sizes were tried before.
__global__ void k_leaf_restore(const int32_t *__restrict__ e2n, const uint32_t *__restrict__ info,
                               const int32_t *__restrict__ hidx, const int32_t *__restrict__ sfc,
                               int32_t *__restrict__ e2n_o, uint32_t *__restrict__ info_o,
                               int32_t *__restrict__ hidx_o, int64_t n_leaf, int npe)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_leaf) return;
  const int64_t j = sfc[i];
  for (int k = 0; k < npe; k++) e2n_o[j * npe + k] = e2n[i * npe + k];
  info_o[j] = info[i];
  hidx_o[j] = hidx[i];
}
__global__ void k_flag27(const uint32_t *__restrict__ info, uint32_t *__restrict__ f, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) f[i] = (info[i] >> 27) & 1u;
}
__global__ void k_iota_i32(int32_t *__restrict__ v, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (int32_t) i;
}

// Reflected fill masks: bit k = fill bit (k ^ c) of hanging leaf h (Q1: nPe <= 16).
__global__ void k_tile_fmask(const uint32_t *__restrict__ info, const int32_t *__restrict__ hidx,
                             const uint32_t *__restrict__ fill, int64_t n_leaf, int npe, uint32_t *__restrict__ fm)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_leaf) return;
  const uint32_t inf = info[i];
  if (!((inf >> 16) & 1u)) return;
  const int c = (int) ((inf >> 8) & 0xFFu);
  const int64_t h = hidx[i];
  const uint32_t f = fill[h * 3];
  uint32_t m = 0;
  for (int k = 0; k < npe; k++) m |= ((f >> (k ^ c)) & 1u) << k;
  fm[h] = m;
}
// Per tile: the hanging index of its first hanging leaf (hb), and in bits
// 17..26 of every hanging leaf's info word its rank among the tile's hanging
// leaves, so the kernel finds a leaf's hanging records without reading hidx.
// One CTA of `T` threads per tile.
__global__ void k_tile_ranks(uint32_t *__restrict__ info, const int32_t *__restrict__ hidx,
                             const int64_t *__restrict__ ls, int64_t *__restrict__ hb)
{
  __shared__ uint32_t wc[32];
  const int64_t t = blockIdx.x;
  const int64_t i = ls[t] + threadIdx.x;
  const bool valid = i < ls[t + 1];
  uint32_t inf = valid ? info[i] : 0u;
  const bool hang = valid && ((inf >> 16) & 1u);
  const unsigned m = __ballot_sync(0xffffffffu, hang);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) wc[w] = __popc(m);
  __syncthreads();
  uint32_t r = __popc(m & ((1u << lane) - 1u));
  for (int k = 0; k < w; k++) r += wc[k];
  if (threadIdx.x == 0) hb[t] = 0;
  __syncthreads();
  constexpr uint32_t RANK = 0x3FFu << 17;
  if (hang) {
    info[i] = (inf & ~RANK) | (r << 17);
    if (r == 0) hb[t] = hidx[i];
  } else if (valid) {
    info[i] = inf & ~RANK;
  }
}

// tau[t] = the coarsest leaf level of tile t (its fixed-point unit)
__global__ void k_tile_tau(const uint32_t *__restrict__ info, const int64_t *__restrict__ ls,
                           uint8_t *__restrict__ tau)
{
  __shared__ uint32_t m;
  if (threadIdx.x == 0) m = 255u;
  __syncthreads();
  const int64_t i = ls[blockIdx.x] + threadIdx.x;
  if (i < ls[blockIdx.x + 1]) atomicMin(&m, info[i] & 0xFFu);
  __syncthreads();
  if (threadIdx.x == 0) tau[blockIdx.x] = (uint8_t) (m == 255u ? 0u : m);
}

__global__ void k_tile_lstart(int64_t *__restrict__ ls, int64_t n_tile, int64_t T, int64_t n_leaf)
{
  const int64_t t = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t <= n_tile) ls[t] = t < n_tile ? t * T : n_leaf;
}

// Slots with no node (TL_NONE) are pointed at one of TL_SINKS per-lane sink
// entries past the tile's U nodes (U + lane): the leaf kernel reads 0 there
// and adds into a sink that is never written out, with no test per slot.
// Lanes of one warp have distinct sinks.  One CTA of `T` threads per tile.
__global__ void k_tile_sinks(uint16_t *__restrict__ e2l, uint16_t *__restrict__ p2l,
                             const uint32_t *__restrict__ info, const int32_t *__restrict__ hidx,
                             const int64_t *__restrict__ ls, const int64_t *__restrict__ off, int npe)
{
  const int64_t t = blockIdx.x;
  const int64_t i = ls[t] + threadIdx.x;
  if (i >= ls[t + 1]) return;
  const uint16_t sink = (uint16_t) (off[t + 1] - off[t] + (threadIdx.x & (TL_SINKS - 1)));
  for (int k = 0; k < npe; k++)
    if (e2l[i * npe + k] == TL_NONE) e2l[i * npe + k] = sink;
  if ((info[i] >> 16) & 1u) {
    const int64_t h = hidx[i];
    for (int k = 0; k < npe; k++)
      if (p2l[h * npe + k] == TL_NONE) p2l[h * npe + k] = sink;
  }
}

// Tile t's node entries at t * cap (then node 0 up to cap) and its count.
// One CTA per tile.
__global__ void k_tile_pad(const int64_t *__restrict__ off, const uint32_t *__restrict__ nodes,
                           uint32_t *__restrict__ pad, int32_t *__restrict__ ucnt, int cap)
{
  const int64_t t = blockIdx.x;
  const int U = (int) (off[t + 1] - off[t]);
  if (threadIdx.x == 0) ucnt[t] = U;
  for (int u = threadIdx.x; u < cap; u += blockDim.x) pad[t * cap + u] = u < U ? nodes[off[t] + u] : 0u;
}

void tile_pad(Plan &pl, cudaStream_t s)
{
  const int cap = ((int) pl.tl_umax + 3) & ~3;
  pl.tl_cap = cap;
  pl.tl_pad.alloc((size_t) std::max<int64_t>(pl.tl_n, 1) * cap);
  pl.tl_ucnt.alloc(std::max<int64_t>(pl.tl_n, 1));
  if (pl.tl_n) k_tile_pad<<<(unsigned) pl.tl_n, 256, 0, s>>>(pl.tl_off.p, pl.tl_nodes.p, pl.tl_pad.p, pl.tl_ucnt.p, cap);
  check_launch("tile_pad");
}

void tile_setup(Plan &pl, int T, cudaStream_t s)
{
  pl.tl_ready = false;
  pl.tl_T = 0;
  if (pl.order != 1 || pl.n_leaf == 0 || T <= 0) return;
  if (T < 32 || T > 1024 || (T & (T - 1))) throw std::invalid_argument("tile size must be a power of two in [32, 1024]");
  const int npe = pl.npe;
  int cap = 1;
  while (cap < 2 * T * npe) cap <<= 1;
  cap = std::max(cap, TB_THREADS);
  if (cap > 65536) throw std::invalid_argument("tile too large");   // 16-bit local indices
  if (pl.n_nodes > (int64_t) TL_ID + 1) throw std::invalid_argument("too many nodes for tiles");
  const int64_t n_tile = (pl.n_leaf + T - 1) / T;
  if (pl.seg.empty()) {
    // hanging leaves first within each tile (a single mesh: a batch keeps the
    // concatenated order of its meshes)
    DBuf<int32_t> e2n_o((size_t) pl.n_leaf * npe), hidx_o(pl.n_leaf), sfc_o(pl.n_leaf);
    DBuf<uint32_t> info_o(pl.n_leaf);
    if (pl.leaf_sfc.n == (size_t) pl.n_leaf) {
      // tiled before: back to the traversal order first
      k_leaf_restore<<<grid_for(pl.n_leaf), 256, 0, s>>>(pl.e2n.p, pl.info.p, pl.hidx.p, pl.leaf_sfc.p, e2n_o.p,
                                                         info_o.p, hidx_o.p, pl.n_leaf, npe);
      check_launch("leaf_restore");
      DKT_CUDA(cudaStreamSynchronize(s));
      std::swap(pl.e2n, e2n_o);
      std::swap(pl.info, info_o);
      std::swap(pl.hidx, hidx_o);
    }
    k_tile_partition<<<(unsigned) n_tile, T, 0, s>>>(pl.e2n.p, pl.info.p, pl.hidx.p, e2n_o.p, info_o.p, hidx_o.p,
                                                     pl.n_leaf, T, npe, sfc_o.p);
    check_launch("tile_partition");
    DKT_CUDA(cudaStreamSynchronize(s));
    pl.e2n = std::move(e2n_o);
    pl.info = std::move(info_o);
    pl.hidx = std::move(hidx_o);
    pl.leaf_sfc = std::move(sfc_o);
    if (pl.st_n_hleaf > 0) {
      // the leaves that read stale slots, renumbered
      DBuf<uint32_t> f(pl.n_leaf), pos(pl.n_leaf);
      DBuf<int32_t> iota(pl.n_leaf);
      k_flag27<<<grid_for(pl.n_leaf), 256, 0, s>>>(pl.info.p, f.p, pl.n_leaf);
      k_iota_i32<<<grid_for(pl.n_leaf), 256, 0, s>>>(iota.p, pl.n_leaf);
      const int64_t nh = (int64_t) exclusive_scan_total<uint32_t>(f.p, pos.p, pl.n_leaf, s);
      scatter_if_kernel<int32_t><<<grid_for(pl.n_leaf), 256, 0, s>>>(iota.p, f.p, pos.p, pl.st_hleaves.p, pl.n_leaf);
      check_launch("stale_leaves");
      DKT_CUDA(cudaStreamSynchronize(s));
      if (nh != pl.st_n_hleaf) throw std::runtime_error("stale leaf list changed size");
    }
  }
  DBuf<uint32_t> node_tiles(pl.n_nodes), cnt(n_tile);
  DKT_CUDA(cudaMemsetAsync(node_tiles.p, 0, pl.n_nodes * sizeof(uint32_t), s));
  const size_t smem = (size_t) cap * sizeof(uint64_t);
  ensure_dyn_smem(k_tile_build, smem);
  k_tile_build<<<(unsigned) n_tile, TB_THREADS, smem, s>>>(0, pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.n_leaf,
                                                          npe, T, cap, node_tiles.p, cnt.p, nullptr, nullptr,
                                                          nullptr, nullptr, nullptr);
  check_launch("tile_count");
  // offsets (host scan: one value per tile) and the largest tile
  std::vector<uint32_t> hc(n_tile);
  DKT_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, n_tile * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaStreamSynchronize(s));
  std::vector<int64_t> ho(n_tile + 1, 0);
  uint32_t umax = 0;
  for (int64_t t = 0; t < n_tile; t++) {
    ho[t + 1] = ho[t] + hc[t];
    umax = std::max(umax, hc[t]);
  }
  pl.tl_off.upload(ho.data(), ho.size(), s);
  pl.tl_nodes.alloc(std::max<int64_t>(ho[n_tile], 1));
  pl.tl_e2l.alloc((size_t) pl.n_leaf * npe);
  pl.tl_p2l.alloc((size_t) std::max<int64_t>(pl.n_hang, 1) * npe);
  DKT_CUDA(cudaMemsetAsync(pl.tl_e2l.p, 0xFF, (size_t) pl.n_leaf * npe * sizeof(uint16_t), s));
  DKT_CUDA(cudaMemsetAsync(pl.tl_p2l.p, 0xFF, (size_t) std::max<int64_t>(pl.n_hang, 1) * npe * sizeof(uint16_t), s));
  k_tile_build<<<(unsigned) n_tile, TB_THREADS, smem, s>>>(1, pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.n_leaf,
                                                          npe, T, cap, node_tiles.p, cnt.p, pl.tl_off.p,
                                                          pl.tl_nodes.p, pl.tl_e2l.p, pl.tl_p2l.p,
                                                          pl.fx_kappa > 0 ? pl.fx_lam.p : nullptr);
  check_launch("tile_fill");
  pl.tl_fm.alloc(std::max<int64_t>(pl.n_hang, 1));
  k_tile_fmask<<<grid_for(pl.n_leaf), 256, 0, s>>>(pl.info.p, pl.hidx.p, pl.fill.p, pl.n_leaf, npe, pl.tl_fm.p);
  pl.tl_lstart.alloc(n_tile + 1);
  k_tile_lstart<<<grid_for(n_tile + 1), 256, 0, s>>>(pl.tl_lstart.p, n_tile, T, pl.n_leaf);
  pl.tl_hb.alloc(n_tile + 1);
  k_tile_ranks<<<(unsigned) n_tile, T, 0, s>>>(pl.info.p, pl.hidx.p, pl.tl_lstart.p, pl.tl_hb.p);
  // U <= 2 T npe <= 32768 (T <= 1024, npe <= 16), so U + TL_SINKS stays clear of TL_NONE
  k_tile_sinks<<<(unsigned) n_tile, T, 0, s>>>(pl.tl_e2l.p, pl.tl_p2l.p, pl.info.p, pl.hidx.p, pl.tl_lstart.p,
                                               pl.tl_off.p, npe);
  pl.tl_tau.alloc(n_tile);
  k_tile_tau<<<(unsigned) n_tile, T, 0, s>>>(pl.info.p, pl.tl_lstart.p, pl.tl_tau.p);
  check_launch("tile_masks");
  DKT_CUDA(cudaStreamSynchronize(s));
  if (pl.lseg.size() >= 2) {
    // a re-tiled batch: the meshes each tile covers
    std::vector<int32_t> lo(n_tile), hi(n_tile);
    for (int64_t t = 0; t < n_tile; t++) {
      const int64_t a = t * T, b = std::min<int64_t>((t + 1) * T, pl.n_leaf) - 1;
      lo[t] = (int32_t) (std::upper_bound(pl.lseg.begin(), pl.lseg.end(), a) - pl.lseg.begin() - 1);
      hi[t] = (int32_t) (std::upper_bound(pl.lseg.begin(), pl.lseg.end(), b) - pl.lseg.begin() - 1);
    }
    pl.tl_mlo.upload(lo.data(), lo.size(), s);
    pl.tl_mhi.upload(hi.data(), hi.size(), s);
  }
  pl.tl_T = T;
  pl.tl_n = n_tile;
  pl.tl_umax = umax;
  pl.tl_ls_direct = true;
  tile_pad(pl, s);
  DKT_CUDA(cudaStreamSynchronize(s));
  pl.tl_sum_u = ho[n_tile];
  pl.tl_ready = true;
}

// ---------------------------------------------------------------------------
// The tiled leaf kernel.  One thread per leaf; blockDim.x == T.
// ---------------------------------------------------------------------------
// Walsh-Hadamard transform over the DIM axes.  Integers: two axes per pass,
// each output a sum of four inputs, which integer hardware adds three at a
// time (fewer instructions than two passes of pairwise butterflies; integer
// sums are exact, so the result is the same as axis by axis).  Binary32: axis
// by axis.
template <int DIM, typename T>
__device__ __forceinline__ void wht(T (&v)[1 << DIM])
{
  constexpr int D4 = std::is_integral<T>::value ? DIM / 2 * 2 : 0;   // axes done two at a time
#pragma unroll
  for (int d = 0; d < D4; d += 2)
#pragma unroll
    for (int k = 0; k < (1 << DIM); k++)
      if (!(k & (3 << d))) {
        const int i1 = 1 << d, i2 = 2 << d;
        const T a = v[k], b = v[k | i1], c = v[k | i2], e = v[k | i1 | i2];
        const T s = a + b, t = a - b;
        v[k] = s + c + e;
        v[k | i1] = t + c - e;
        v[k | i2] = s - c - e;
        v[k | i1 | i2] = t - c + e;
      }
#pragma unroll
  for (int d = D4; d < DIM; d++)
#pragma unroll
    for (int k = 0; k < (1 << DIM); k++)
      if (!(k & (1 << d))) {
        const T a = v[k], b = v[k | (1 << d)];
        v[k] = a + b;
        v[k | (1 << d)] = a - b;
      }
}

// Shared-memory accumulation of a tile's outputs.  Fixed point: a 64-bit sum
// kept as two 32-bit words (low word unsigned, high word signed) updated
// with native 32-bit shared atomics -- the carry out of the low word is
// detected from the value the atomic returns and added to the high word --
// which is exact for any number of contributions and cheaper than 64-bit
// shared atomics.  Binary32: one float atomic.
template <typename AR> struct TileAcc;
template <> struct TileAcc<FixedArith> {
  static constexpr int WORDS = 2;
  __device__ static __forceinline__ void zero(uint32_t *a, int U, int u) { a[u] = 0u; a[U + u] = 0u; }
  __device__ static __forceinline__ void add(uint32_t *a, int U, uint32_t u, long long v)
  {
    const uint32_t lo = (uint32_t) (unsigned long long) v;
    const int hi = (int) (v >> 32);
    const uint32_t old = atomicAdd(a + u, lo);
    // hi plus the carry out of old + lo, taken from the add's carry flag (two
    // instructions; the compare-and-select form measured 1% slower at level 8)
    uint32_t hc;
    asm("{\n\t.reg .u32 t;\n\tadd.cc.u32 t, %1, %2;\n\taddc.u32 %0, %3, 0;\n\t}"
        : "=r"(hc)
        : "r"(old), "r"(lo), "r"((uint32_t) hi));
    atomicAdd(reinterpret_cast<int *>(a + U) + u, (int) hc);
  }
  __device__ static __forceinline__ long long get(const uint32_t *a, int U, int u)
  {
    return (long long) (((unsigned long long) (uint32_t) a[U + u] << 32) | (unsigned long long) a[u]);
  }
};
template <> struct TileAcc<F32Arith> {
  static constexpr int WORDS = 1;
  __device__ static __forceinline__ void zero(uint32_t *a, int, int u) { a[u] = 0u; }
  __device__ static __forceinline__ void add(uint32_t *a, int, uint32_t u, float v)
  {
    atomicAdd(reinterpret_cast<float *>(a) + u, v);
  }
  __device__ static __forceinline__ float get(const uint32_t *a, int, int u) { return __uint_as_float(a[u]); }
};

// One row of NPE 16-bit local indices as NPE/2 packed words (16-byte loads).
template <int NPE>
__device__ __forceinline__ void load_row16(const uint16_t *__restrict__ row, uint32_t (&w)[NPE / 2])
{
  if constexpr (NPE == 16) {
    const uint4 a = __ldg(reinterpret_cast<const uint4 *>(row));
    const uint4 b = __ldg(reinterpret_cast<const uint4 *>(row) + 1);
    w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w; w[4] = b.x; w[5] = b.y; w[6] = b.z; w[7] = b.w;
  } else if constexpr (NPE == 8) {
    const uint4 a = __ldg(reinterpret_cast<const uint4 *>(row));
    w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w;
  } else {
    const uint2 a = __ldg(reinterpret_cast<const uint2 *>(row));
    w[0] = a.x; w[1] = a.y;
  }
}
template <int NPE>
__device__ __forceinline__ uint32_t idx16(const uint32_t (&w)[NPE / 2], int k)
{
  return (w[k >> 1] >> ((k & 1) * 16)) & 0xFFFFu;
}

// The integer multiples of the dyadic scaling (6^dim D_L = C1(k) alpha_L +
// C2(k) beta_L, k the popcount of the mode), passed as a kernel parameter:
// their loads are constant-bank operands of the multiply-adds.
struct DyConst {
  uint32_t c1[5], c2[5];
};
static int pow3_i(int e) { return e <= 0 ? 1 : 3 * pow3_i(e - 1); }
static int dy_c1(int dim, int k) { return k == 0 ? 0 : k * pow3_i(dim - k + 1); }
static int dy_c2(int dim, int k) { return pow3_i(dim - k); }

// c * v (0 <= c < 2^31, the product within 63 bits): one 32 x 32 -> 64
// multiply of the low word and one multiply-add of the high word.
__device__ __forceinline__ long long mul_small(long long v, uint32_t c)
{
  const uint32_t lo = (uint32_t) (unsigned long long) v, hi = (uint32_t) ((unsigned long long) v >> 32);
  unsigned long long p;
  asm("mul.wide.u32 %0, %1, %2;" : "=l"(p) : "r"(lo), "r"(c));
  uint32_t phi = (uint32_t) (p >> 32);
  asm("mad.lo.u32 %0, %1, %2, %0;" : "+r"(phi) : "r"(hi), "r"(c));
  return (long long) (((unsigned long long) phi << 32) | (uint32_t) p);
}
// v >> s (arithmetic) for 0 <= s <= 31: a funnel shift of the low word and a
// shift of the high word.
__device__ __forceinline__ long long sar_lt32(long long v, uint32_t s)
{
  const uint32_t lo = (uint32_t) (unsigned long long) v, hi = (uint32_t) ((unsigned long long) v >> 32);
  uint32_t rlo, rhi;
  asm("shf.r.clamp.b32 %0, %1, %2, %3;" : "=r"(rlo) : "r"(lo), "r"(hi), "r"(s));
  asm("shr.s32 %0, %1, %2;" : "=r"(rhi) : "r"(hi), "r"(s));
  return (long long) (((unsigned long long) rhi << 32) | rlo);
}

// v[k] <- sum over the subsets j of k of v[j] (integers; two axes per pass,
// each output of a pass at most one three-input sum)
template <int DIM, typename T>
__device__ __forceinline__ void subset_sums(T (&v)[1 << DIM])
{
  constexpr int D2 = DIM / 2 * 2;
#pragma unroll
  for (int d = 0; d < D2; d += 2)
#pragma unroll
    for (int k = 0; k < (1 << DIM); k++)
      if (!(k & (3 << d))) {
        const int i1 = 1 << d, i2 = 2 << d;
        const T a = v[k], b = v[k | i1], c = v[k | i2], e = v[k | i1 | i2];
        const T t = a + b;
        v[k | i1] = t;
        v[k | i2] = a + c;
        v[k | i1 | i2] = t + c + e;
      }
#pragma unroll
  for (int d = D2; d < DIM; d++)
#pragma unroll
    for (int k = 0; k < (1 << DIM); k++)
      if (!(k & (1 << d))) v[k | (1 << d)] += v[k];
}
// v[j] <- sum over the supersets k of j of v[k]
template <int DIM, typename T>
__device__ __forceinline__ void superset_sums(T (&v)[1 << DIM])
{
  constexpr int D2 = DIM / 2 * 2;
#pragma unroll
  for (int d = 0; d < D2; d += 2)
#pragma unroll
    for (int k = 0; k < (1 << DIM); k++)
      if (!(k & (3 << d))) {
        const int i1 = 1 << d, i2 = 2 << d;
        const T a = v[k], b = v[k | i1], c = v[k | i2], e = v[k | i1 | i2];
        const T t = b + e;
        v[k | i1] = t;
        v[k | i2] = c + e;
        v[k] = t + a + c;
      }
#pragma unroll
  for (int d = D2; d < DIM; d++)
#pragma unroll
    for (int k = 0; k < (1 << DIM); k++)
      if (!(k & (1 << d))) v[k] += v[k | (1 << d)];
}

// A thread's node slots of the tile are visited in groups of four, the four
// id loads issued before anything that depends on them: one global round trip
// per group for the ids and one for the values, instead of two per slot.
constexpr int TILE_G = 4;

// The tile's node values into shared memory, and its node entries into sid
// for the flush; sums zeroed.
template <int T_LEAVES, typename V, typename ACC>
__device__ __forceinline__ void tile_gather(const uint32_t *__restrict__ tile_nodes, int64_t u0, int U, int Us,
                                            const V *__restrict__ xq, V *xs, uint32_t *ys, uint32_t *sid, int cap)
{
  if (threadIdx.x < TL_SINKS) {
    xs[U + threadIdx.x] = V(0);
    ACC::zero(ys, Us, U + threadIdx.x);
  }
  // the first round's entry loads stay within the tile's padded block
  // (cap entries) and need not wait for U
  for (int b = threadIdx.x; b < U || b == (int) threadIdx.x; b += TILE_G * T_LEAVES) {
    uint32_t id[TILE_G];
    V xv[TILE_G];
#pragma unroll
    for (int j = 0; j < TILE_G; j++) {
      const int u = b + j * T_LEAVES;
      id[j] = u < cap ? __ldg(tile_nodes + u0 + u) : 0u;
    }
#pragma unroll
    for (int j = 0; j < TILE_G; j++) xv[j] = b + j * T_LEAVES < U ? __ldg(xq + (id[j] & TL_ID)) : V(0);
#pragma unroll
    for (int j = 0; j < TILE_G; j++) {
      const int u = b + j * T_LEAVES;
      if (u < U) {
        xs[u] = xv[j];
        sid[u] = id[j];
        ACC::zero(ys, Us, u);
      }
    }
  }
}

// The tile's sums out: stored where the tile is the node's only toucher,
// added atomically elsewhere.  put(id, u) writes slot u to node id (the node
// entries staged in sid by the gather).
template <int T_LEAVES, typename PUT>
__device__ __forceinline__ void tile_scatter(const uint32_t *sid, int U, PUT put)
{
  for (int u = threadIdx.x; u < U; u += T_LEAVES) put(sid[u], u);
}

// SC (fixed point only): 0 = per-(level, mode) multiply-high factors of the
// tile's unit (fm: the per-unit factor table); 1, 2, 3 = dyadic scaling with
// the Laplacian term (bit 0) and / or the mass term (bit 1), fm then pointing
// at the per-level shift words.
// One tile (one CTA's work); uniform exits only.
template <int DIM, int T_LEAVES, typename AR, int SC>
__device__ __forceinline__ void q1t_tile(
    const int64_t tile,
    const uint16_t *__restrict__ e2l, const uint16_t *__restrict__ p2l, const uint32_t *__restrict__ info,
    const int64_t *__restrict__ tile_hb, const uint32_t *__restrict__ fmask_r, const int64_t *__restrict__ tile_off,
    const int64_t *__restrict__ tile_ls, const uint32_t *__restrict__ tile_nodes, const void *__restrict__ fm,
    int n_fac, const typename AR::T *__restrict__ xq, typename AR::T *__restrict__ yq,
    const int32_t *__restrict__ hzoff, const int32_t *__restrict__ hztab, const typename AR::T *__restrict__ stvq,
    int conforming, int skip_stale, const int32_t *__restrict__ tile_mlo, const int32_t *__restrict__ tile_mhi,
    const int *__restrict__ skip_mesh, int skip_stride, const DyConst &dyc,
    const uint8_t *__restrict__ tile_tau, int kappa, int smax, const uint32_t *__restrict__ pad,
    const int32_t *__restrict__ ucnt, int cap, int64_t n_leaf, int ls_direct)
{
  using V = typename AR::T;
  using F = typename AR::Factor;
  constexpr int NPE = 1 << DIM;
  extern __shared__ __align__(16) unsigned char smem[];
  // a batched solve: tiles whose meshes have all converged are not needed (a
  // tile of small meshes covers several; every one of them is checked)
  if (skip_mesh) {
    bool all_done = true;
    for (int32_t m = tile_mlo[tile], me = tile_mhi[tile]; m <= me && all_done; m++)
      all_done = skip_mesh[(int64_t) m * skip_stride] != 0;
    if (all_done) return;
  }
  // the tile's node entries at tile * cap, its count beside them; its leaves
  // at tile * T unless the plan is a batch (concatenated tiles)
  (void) tile_off;
  const int64_t u0 = tile * (int64_t) cap;
  const int U = ucnt[tile];
  const int64_t i = (ls_direct ? tile * (int64_t) T_LEAVES : tile_ls[tile]) + threadIdx.x;
  bool valid = ls_direct ? i < n_leaf : i < tile_ls[tile + 1];
  // the leaf's records first, so their latency overlaps the node gather
  uint32_t inf = 0, fmask = 0xFFFFFFFFu;
  uint32_t w[NPE / 2], pw[NPE / 2];
  int64_t h = -1;
  if (valid) {
    inf = __ldg(info + i);
    if (skip_stale && ((inf >> 27) & 1u)) valid = false;   // done after the stale chain
  }
  if (valid) {
    load_row16<NPE>(e2l + i * NPE, w);
    if ((inf >> 16) & 1u) {
      h = tile_hb[tile] + ((inf >> 17) & 0x3FFu);
      fmask = __ldg(fmask_r + h);
      load_row16<NPE>(p2l + h * NPE, pw);
    }
  }
  using ACC = TileAcc<AR>;
  constexpr bool FX = std::is_same<AR, FixedArith>::value;
  static_assert(FX || SC == 0, "dyadic scaling is a fixed-point form");
  F *fac = reinterpret_cast<F *>(smem);
  uint32_t *fsh = reinterpret_cast<uint32_t *>(smem);     // SC != 0: per-level shift words
  const int Us = U + TL_SINKS;                            // the tile's nodes, then the sinks
  const int fac_bytes = SC ? ((n_fac * 4 + 15) & ~15) : n_fac * (int) sizeof(F);
  V *xs = reinterpret_cast<V *>(smem + fac_bytes);
  uint32_t *ys = reinterpret_cast<uint32_t *>(xs + Us);  // ACC::WORDS words per entry
  // the tile's node entries, past the largest tile's values and sums
  uint32_t *sid = reinterpret_cast<uint32_t *>(smem + fac_bytes + (size_t) 2 * smax * sizeof(V));
  // the tile's fixed-point unit: its coarsest leaf level (factor table row)
  const int tau = FX ? (int) tile_tau[tile] : 0;
  for (int k = threadIdx.x; k < n_fac; k += T_LEAVES) {
    if constexpr (SC != 0) fsh[k] = static_cast<const uint32_t *>(fm)[k];
    else fac[k] = AR::load_factor(fm, tau * n_fac + k);
  }
  tile_gather<T_LEAVES, V, ACC>(pad, u0, U, Us, xq, xs, ys, sid, cap);
  __shared__ uint32_t s_max;
  if (threadIdx.x == 0) s_max = 0u;
  __syncthreads();
  V v[NPE], zt[std::is_same<AR, FixedArith>::value ? 1 : NPE];
  if (valid) {
    const int L = inf & 0xFFu;
    const bool hang = h >= 0;
    auto lidx = [&](int k) -> uint32_t { return idx16<NPE>(w, k); };
    if (hang) {
      const int c = (int) ((inf >> 8) & 0xFFu);
      const int32_t hz = hzoff ? __ldg(hzoff + h) : -1;
#pragma unroll
      for (int k = 0; k < NPE; k++) v[k] = xs[idx16<NPE>(pw, k)];   // a sink reads 0
      if (hz >= 0) {
        // the parent slots with no node read the emulated static buffer
#pragma unroll
        for (int k = 0; k < NPE; k++)
          if (idx16<NPE>(pw, k) >= (uint32_t) U) {
            const int32_t id = __ldg(hztab + (int64_t) hz * NPE + (k ^ c));
            if (id >= 0) v[k] = __ldg(stvq + id);
          }
      }
      // parent -> child-0 interpolation: rank k takes the mean of the parent
      // values on the subsets of k (the sum, then one shift or scaling)
      subset_sums<DIM, V>(v);
#pragma unroll
      for (int k = 1; k < NPE; k++) {
        if constexpr (FX) v[k] >>= __popc(k);
        else v[k] *= 1.0f / (float) (1 << __popc(k));
      }
#pragma unroll
      for (int k = 0; k < NPE; k++)
        if ((fmask >> k) & 1u) v[k] = xs[lidx(k)];
    } else {
#pragma unroll
      for (int k = 0; k < NPE; k++) v[k] = xs[lidx(k)];
    }
    wht<DIM, V>(v);
    if constexpr (SC == 0) {
#pragma unroll
      for (int k = 0; k < NPE; k++) v[k] = AR::apply(v[k], fac[L * NPE + k]);
    } else {
      // k = popcount of the mode; in the tile's unit (level tau):
      //   both terms  (C1(k) w + (C2(k) w >> d_L)) >> (s_L - kappa tau)
      //   one term    (C(k) w) >> (s_L - kappa tau)
      // every shift below 32 (checked when the plan was set up)
      const uint32_t sh = fsh[L];
      const uint32_t sl = (sh & 0xFFu) - (uint32_t) (kappa * tau), dl = (sh >> 8) & 0xFFu;
#pragma unroll
      for (int k = 0; k < NPE; k++) {
        long long t;
        if constexpr (SC == 3) {
          const long long m2 = sar_lt32(mul_small(v[k], dyc.c2[__popc(k)]), dl);
          t = __popc(k) != 0 ? mul_small(v[k], dyc.c1[__popc(k)]) + m2 : m2;
        } else if constexpr (SC == 1) {
          t = __popc(k) != 0 ? mul_small(v[k], dyc.c1[__popc(k)]) : 0;
        } else {
          t = mul_small(v[k], dyc.c2[__popc(k)]);
        }
        v[k] = sar_lt32(t, sl);
      }
    }
    wht<DIM, V>(v);
    if constexpr (std::is_same<AR, FixedArith>::value) {
#pragma unroll
      for (int k = 0; k < NPE; k++) ACC::add(ys, Us, lidx(k), v[k]);
      if (hang) {
        // transpose of the child-0 interpolation on the unfilled ranks, into
        // the parent nodes: parent rank j takes the sum over the supersets k
        // of j of v[k] / 2^popcount(k)
#pragma unroll
        for (int k = 0; k < NPE; k++) v[k] = ((fmask >> k) & 1u) ? V(0) : (v[k] >> __popc(k));
        superset_sums<DIM, V>(v);
#pragma unroll
        for (int k = 0; k < NPE; k++) {
          const uint32_t p = idx16<NPE>(pw, k);
          if (conforming || !((fmask >> k) & 1u)) ACC::add(ys, Us, p, v[k]);
        }
      }
    } else if (hang) {
#pragma unroll
      for (int k = 0; k < NPE; k++) zt[k] = ((fmask >> k) & 1u) ? V(0) : v[k] * (1.0f / (float) (1 << __popc(k)));
      superset_sums<DIM, V>(zt);
    }
  }
  if constexpr (!std::is_same<AR, FixedArith>::value) {
    // binary32: the tile's contributions are quantised against the tile's
    // largest one (22 bits) and summed with native integer shared atomics;
    // each node's sum goes out with one float atomic.  The rounding to an
    // integer is one fused multiply-add: v * up + 1.5 * 2^23 lands in
    // [2^23, 2^24), where binary32 spacing is 1, for |v * up| < 2^22, and its
    // bits less those of 1.5 * 2^23 are the rounded integer.
    // The largest contribution bounds the scale.  The outputs of unfilled
    // ranks, which go to sinks, count too: they are element outputs like the
    // others, and leaving them out would cost a test per rank.
    float m = 0.0f;
    if (valid) {
#pragma unroll
      for (int k = 0; k < NPE; k++) m = fmaxf(m, fabsf(v[k]));
      if (h >= 0) {
#pragma unroll
        for (int k = 0; k < NPE; k++) m = fmaxf(m, fabsf(zt[k]));
      }
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&s_max, __float_as_uint(m));
    __syncthreads();
    int e = 0;
    frexpf(__uint_as_float(s_max), &e);              // max < 2^e
    const float up = ldexpf(1.0f, 22 - e);
    auto quant = [up](float v) { return __float_as_int(fmaf(v, up, 12582912.0f)) - 0x4B400000; };
    if (valid) {
#pragma unroll
      for (int k = 0; k < NPE; k++) {
        atomicAdd(reinterpret_cast<int *>(ys) + idx16<NPE>(w, k), quant(v[k]));
      }
      if (h >= 0) {
#pragma unroll
        for (int k = 0; k < NPE; k++) {
          const uint32_t p = idx16<NPE>(pw, k);
          if (conforming || !((fmask >> k) & 1u))
            atomicAdd(reinterpret_cast<int *>(ys) + p, quant(zt[k]));
        }
      }
    }
    __syncthreads();
    const float down = ldexpf(1.0f, e - 22);
    tile_scatter<T_LEAVES>(sid, U, [&](uint32_t id, int u) {
      const int a = reinterpret_cast<const int *>(ys)[u];
      if (id & TL_EXCL) yq[id & TL_ID] = (V) a * down;
      else if (a != 0) atomicAdd(yq + (id & TL_ID), (V) a * down);
    });
    return;
  }
  __syncthreads();
  // the tile's sums from its unit (level tau) to each node's (level lam):
  // a factor 2^(kappa (lam - tau)), lam >= tau for a node only this tile's
  // finer leaves touch, lam < tau for one that coarser leaves elsewhere touch
  const int ktau = kappa * tau;
  tile_scatter<T_LEAVES>(sid, U, [&](uint32_t id, int u) {
    V a = ACC::get(ys, Us, u);
    if constexpr (FX) {
      if (kappa > 0) {
        const int d = kappa * (int) ((id >> TL_LAM) & 15u) - ktau;
        a = d >= 0 ? (V) ((unsigned long long) a << d) : (a >> -d);
      }
    }
    if (id & TL_EXCL) yq[id & TL_ID] = a;
    else if (a != V(0)) AR::add(yq + (id & TL_ID), a);
  });
}

// The tiled kernel.  PERSIST false: one CTA per tile (a plain grid of n_tile
// CTAs).  PERSIST true: a persistent launch, a grid of as many CTAs as fit on
// the device at once, each pulling the next tile from *counter (zero at
// launch) until all n_tile are taken; in a batched solve the tiles whose
// meshes have converged are passed over as they are pulled.
template <int DIM, int T_LEAVES, typename AR, int SC, bool PERSIST>
__global__ void __launch_bounds__(T_LEAVES, 1024 / T_LEAVES) k_matvec_q1t(
    const uint16_t *__restrict__ e2l, const uint16_t *__restrict__ p2l, const uint32_t *__restrict__ info,
    const int64_t *__restrict__ tile_hb, const uint32_t *__restrict__ fmask_r, const int64_t *__restrict__ tile_off,
    const int64_t *__restrict__ tile_ls, const uint32_t *__restrict__ tile_nodes, const void *__restrict__ fm,
    int n_fac, const typename AR::T *__restrict__ xq, typename AR::T *__restrict__ yq,
    const int32_t *__restrict__ hzoff, const int32_t *__restrict__ hztab, const typename AR::T *__restrict__ stvq,
    int conforming, int skip_stale, const int32_t *__restrict__ tile_mlo, const int32_t *__restrict__ tile_mhi,
    const int *__restrict__ skip_mesh, int skip_stride, const __grid_constant__ DyConst dyc,
    const uint8_t *__restrict__ tile_tau, int kappa, unsigned long long *__restrict__ counter, int64_t n_tile,
    int smax, const uint32_t *__restrict__ pad, const int32_t *__restrict__ ucnt, int cap, int64_t n_leaf,
    int ls_direct)
{
  if constexpr (!PERSIST) {
    q1t_tile<DIM, T_LEAVES, AR, SC>(blockIdx.x, e2l, p2l, info, tile_hb, fmask_r, tile_off, tile_ls, tile_nodes, fm,
                                    n_fac, xq, yq, hzoff, hztab, stvq, conforming, skip_stale, tile_mlo, tile_mhi,
                                    skip_mesh, skip_stride, dyc, tile_tau, kappa, smax, pad, ucnt, cap, n_leaf,
                                    ls_direct);
    return;
  } else {
  __shared__ long long s_tile;
  for (;;) {
    if (threadIdx.x == 0) s_tile = (long long) atomicAdd(counter, 1ull);
    __syncthreads();
    const int64_t t = s_tile;
    __syncthreads();                 // every thread has read s_tile
    if (t >= n_tile) return;
    q1t_tile<DIM, T_LEAVES, AR, SC>(t, e2l, p2l, info, tile_hb, fmask_r, tile_off, tile_ls, tile_nodes, fm, n_fac,
                                    xq, yq, hzoff, hztab, stvq, conforming, skip_stale, tile_mlo, tile_mhi, skip_mesh,
                                    skip_stride, dyc, tile_tau, kappa, smax, pad, ucnt, cap, n_leaf, ls_direct);
    __syncthreads();                 // the tile's shared memory is free again
  }
  }
}

template <int DIM, int TL, typename AR, int SC>
static void launch_tiled(Plan &pl, const void *fm, const typename AR::T *x, typename AR::T *y,
                         const int32_t *hzoff, const int32_t *hztab, const typename AR::T *stv, bool skip_stale,
                         cudaStream_t s)
{
  // the persistent form is compiled for dims 2 and 3 (the batched meshes);
  // a 4D plan asking for it runs the plain grid
  constexpr bool CAN_PERSIST = DIM <= 3;
  const bool persist = CAN_PERSIST && pl.tl_persist;
  auto kfn = persist ? k_matvec_q1t<DIM, TL, AR, SC, CAN_PERSIST> : k_matvec_q1t<DIM, TL, AR, SC, false>;
  DyConst dyc{};
  for (int k = 0; k <= DIM; k++) {
    dyc.c1[k] = (uint32_t) dy_c1(DIM, k);
    dyc.c2[k] = (uint32_t) dy_c2(DIM, k);
  }
  // one row of the per-unit factor table, or the per-level shift words
  const int n_fac = SC ? pl.md + 1 : (pl.md + 1) * (1 << DIM);
  const size_t fac_bytes = SC ? (size_t) ((n_fac * 4 + 15) & ~15) : (size_t) n_fac * sizeof(typename AR::Factor);
  // values and sums of the largest tile (plus sinks), then its node entries
  const int smax = (int) pl.tl_umax + TL_SINKS;
  const size_t smem = fac_bytes + (size_t) 2 * smax * sizeof(typename AR::T) + (size_t) smax * sizeof(uint32_t);
  ensure_dyn_smem(kfn, smem);
  unsigned grid = (unsigned) pl.tl_n;
  unsigned long long *counter = nullptr;
  if (persist) {
    int dev = 0, sms = 0, per_sm = 0;
    DKT_CUDA(cudaGetDevice(&dev));
    DKT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DKT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, TL, smem));
    grid = (unsigned) std::max<int64_t>(1, std::min<int64_t>(pl.tl_n, (int64_t) sms * std::max(per_sm, 1)));
    if (pl.tl_counter.n < 1) pl.tl_counter.alloc(1);
    counter = pl.tl_counter.p;
    DKT_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s));
  }
  kfn<<<grid, TL, smem, s>>>(pl.tl_e2l.p, pl.tl_p2l.p, pl.info.p, pl.tl_hb.p, pl.tl_fm.p, pl.tl_off.p,
                                           pl.tl_lstart.p, pl.tl_nodes.p, fm, n_fac, x, y, hzoff, hztab, stv,
                                           pl.conforming ? 1 : 0, skip_stale ? 1 : 0, pl.tl_mlo.p, pl.tl_mhi.p,
                                           pl.tl_mlo.p ? pl.skip_mesh : nullptr, pl.skip_stride, dyc, pl.tl_tau.p,
                                           std::is_same<AR, FixedArith>::value ? pl.fx_kappa : 0, counter,
                                           pl.tl_n, smax, pl.tl_pad.p, pl.tl_ucnt.p, pl.tl_cap, pl.n_leaf,
                                           pl.tl_ls_direct ? 1 : 0);
}

template <typename AR, int SC>
static void launch_tiled_dim(Plan &pl, const void *fm, const typename AR::T *x, typename AR::T *y,
                             const int32_t *hzoff, const int32_t *hztab, const typename AR::T *stv, bool skip_stale,
                             cudaStream_t s)
{
#define DKT_TL_CASE(D, TL) \
  case (D) * 10000 + (TL): launch_tiled<D, TL, AR, SC>(pl, fm, x, y, hzoff, hztab, stv, skip_stale, s); break;
  switch (pl.dim * 10000 + pl.tl_T) {
    DKT_TL_CASE(2, 128) DKT_TL_CASE(2, 256) DKT_TL_CASE(2, 512)
    DKT_TL_CASE(3, 128) DKT_TL_CASE(3, 256) DKT_TL_CASE(3, 512)
    DKT_TL_CASE(4, 64) DKT_TL_CASE(4, 128) DKT_TL_CASE(4, 256)
    default: throw std::runtime_error("unsupported dim / tile size for the tiled kernel");
  }
#undef DKT_TL_CASE
  check_launch("matvec_q1t");
  pl.n_launch++;
}

// skip_stale: leave the leaves that read stale slots to a later launch.  The
// leaves that remain read no stale slot, so they need no look-up of one.
void tiled_fixed(Plan &pl, bool skip_stale, cudaStream_t s)
{
  const int32_t *hz = (pl.st_ready && !skip_stale) ? pl.st_hzoff.p : nullptr;
  switch (pl.fx_scale) {
#define DKT_SC_CASE(SC, FM) \
  case SC: launch_tiled_dim<FixedArith, SC>(pl, FM, pl.xq.p, pl.yq.p, hz, pl.st_hztab.p, pl.st_vq.p, skip_stale, s); break;
    DKT_SC_CASE(0, pl.fx_fm.p) DKT_SC_CASE(1, pl.fx_shift.p) DKT_SC_CASE(2, pl.fx_shift.p) DKT_SC_CASE(3, pl.fx_shift.p)
#undef DKT_SC_CASE
    default: throw std::runtime_error("bad fixed-point scaling mode");
  }
}

void tiled_f32(Plan &pl, const float *x, float *y, cudaStream_t s)
{
  launch_tiled_dim<F32Arith, 0>(pl, pl.f32_f.p, x, y, nullptr, nullptr, nullptr, false, s);
}

bool tile_size_supported(int dim, int T)
{
  if (dim == 4) return T == 64 || T == 128 || T == 256;
  return T == 128 || T == 256 || T == 512;
}

}  // namespace dkt
