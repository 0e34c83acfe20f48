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
// info bit 28: a hanging leaf whose unfilled ranks read hanging-node slots
constexpr uint32_t INFO_HNS = 1u << 28;

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
    // hanging leaves that read no hanging-node slots are the per-leaf
    // kernel's: nothing of theirs goes into the tile
    if (s < half) {
      const int j = s / npe;
      if (j < nl && !(((info[l0 + j] >> 16) & 1u) && !(info[l0 + j] & INFO_HNS)))
        node = e2n[(l0 + j) * npe + s % npe];
    } else {
      const int j = (s - half) / npe;
      if (j < nl && (info[l0 + j] & INFO_HNS)) node = p2n[(int64_t) hidx[l0 + j] * npe + (s - half) % npe];
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

// Which hanging leaves read hanging-node slots (info bit 28; the others go
// to the per-leaf kernel).  In the reflected frame (rank k of the leaf, parent
// rank k, at position k ^ c of the maps), with U the unfilled ranks:
//   * the leaf reads no stale parent slot (info bit 27);
//   * rank 0 is filled, and no unfilled rank spans every axis (a face of at
//     most 2^(dim-1) corners);
//   * every unfilled rank's face has two opposite corners that are nodes
//     (they name the face; a corner with no node reads 0 in both forms);
//   * reference traversal only: U is closed under removing an axis (down to
//     rank 0), and rank 0 is the parent's rank-0 node.  Then the parent ranks
//     the reference transpose reaches (unfilled ones) are exactly the corners
//     of the unfilled ranks' faces other than rank 0, and the slot form sends
//     to every corner and takes rank 0's share back.
__global__ void k_hns_flag(const int32_t *__restrict__ e2n, uint32_t *__restrict__ info,
                           const int32_t *__restrict__ hidx, const int32_t *__restrict__ p2n,
                           const uint32_t *__restrict__ fill, int64_t n_leaf, int npe, int dim, int conforming,
                           int enable)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_leaf) return;
  uint32_t inf = info[i] & ~INFO_HNS;
  if (enable && ((inf >> 16) & 1u) && !((inf >> 27) & 1u)) {
    const int c = (int) ((inf >> 8) & 0xFFu);
    const int64_t h = hidx[i];
    const uint32_t f = fill[h * 3];
    const int32_t *pr = p2n + h * npe, *er = e2n + i * npe;
    uint32_t um = 0;
    for (int k = 0; k < npe; k++) um |= (((f >> (k ^ c)) & 1u) ^ 1u) << k;
    bool ok = !(um & 1u) && (conforming || (er[c] >= 0 && er[c] == pr[c]));
    for (int k = 1; k < npe && ok; k++) {
      if (!((um >> k) & 1u)) continue;
      if (__popc(k) >= dim) ok = false;
      if (!conforming)
        for (int d = 0; d < dim; d++)
          if (((k >> d) & 1) && k != (1 << d) && !((um >> (k ^ (1 << d))) & 1u)) ok = false;
      bool pair = false;
      for (int q = 0; q < npe; q++)
        if (!(q & ~k) && pr[q ^ c] >= 0 && pr[(q ^ k) ^ c] >= 0) pair = true;
      ok = ok && pair;
    }
    if (ok) inf |= INFO_HNS;
  }
  info[i] = inf;
}

// Within every tile (stable): slot-reading hanging leaves, then non-hanging
// leaves, then the hanging leaves left to the per-leaf kernel (idle here).
// The warps of a tile then mostly run one code path.  Leaf order does not
// matter to the product (integer sums); the hanging records stay indexed by
// hidx.
__global__ void k_tile_partition(const int32_t *__restrict__ e2n, const uint32_t *__restrict__ info,
                                 const int32_t *__restrict__ hidx, int32_t *__restrict__ e2n_o,
                                 uint32_t *__restrict__ info_o, int32_t *__restrict__ hidx_o, int64_t n_leaf, int T,
                                 int npe)
{
  __shared__ uint32_t wc[3][32];
  const int64_t l0 = (int64_t) blockIdx.x * T;
  const int64_t i = l0 + threadIdx.x;
  const bool valid = i < n_leaf;
  const uint32_t inf = valid ? info[i] : 0u;
  const int cls = !valid ? 3 : ((inf >> 16) & 1u) ? ((inf & INFO_HNS) ? 0 : 2) : 1;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (int) (blockDim.x >> 5);
  unsigned m[3];
  for (int q = 0; q < 3; q++) {
    m[q] = __ballot_sync(0xffffffffu, cls == q);
    if (lane == 0) wc[q][w] = __popc(m[q]);
  }
  __syncthreads();
  if (!valid) return;
  uint32_t pos = __popc(m[cls] & ((1u << lane) - 1u));
  for (int q = 0; q < 3; q++)
    for (int k = 0; k < nw; k++)
      if (q < cls || (q == cls && k < w)) pos += wc[q][k];
  const int64_t j = l0 + pos;
  for (int k = 0; k < npe; k++) e2n_o[j * npe + k] = e2n[i * npe + k];
  info_o[j] = inf;
  hidx_o[j] = hidx[i];
}
__global__ void k_flag27(const uint32_t *__restrict__ info, uint32_t *__restrict__ f, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) f[i] = (info[i] >> 27) & 1u;
}
// hanging leaves that read no hanging-node slots
__global__ void k_flag_rest(const uint32_t *__restrict__ info, uint32_t *__restrict__ f, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) f[i] = ((info[i] >> 16) & 1u) && !(info[i] & INFO_HNS) ? 1u : 0u;
}
__global__ void k_iota_i32(int32_t *__restrict__ v, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (int32_t) i;
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
// entries past the tile's U nodes and H hanging-node slots (U + H + lane):
// the leaf kernel reads 0 there and adds into a sink that is never written
// out, with no test per slot.  Lanes of one warp have distinct sinks.  One
// CTA of `T` threads per tile.
__global__ void k_tile_sinks(uint16_t *__restrict__ e2l, const int64_t *__restrict__ ls,
                             const int64_t *__restrict__ off, const int64_t *__restrict__ hs_off, int npe)
{
  const int64_t t = blockIdx.x;
  const int64_t i = ls[t] + threadIdx.x;
  if (i >= ls[t + 1]) return;
  const uint16_t sink = (uint16_t) (off[t + 1] - off[t] + (hs_off[t + 1] - hs_off[t]) + (threadIdx.x & (TL_SINKS - 1)));
  for (int k = 0; k < npe; k++)
    if (e2l[i * npe + k] == TL_NONE) e2l[i * npe + k] = sink;
}

// ---------------------------------------------------------------------------
// Hanging-node slots.  In the reflected (child-0) frame an unfilled rank k of
// a hanging leaf is the centre of the parent face spanned by the axes of k,
// and its interpolated value is the mean of the parent nodes on the subsets
// of k -- the face's 2^popcount(k) corners.  The value depends on the point
// only, so the leaves of a tile that meet at one hanging point share one
// slot: its value is computed once per tile from the face's corners, and the
// leaves read and add into it like a node.  The transpose then sends each
// slot's sum to every corner of its face once per tile; in the reference
// traversal a leaf's transpose leaves out the parent corner it shares (rank
// 0), so the leaf takes its own share back at its rank-0 node (k_hns_flag
// has the conditions).  Integer sums: the fixed-point product is the same as
// interpolating and transposing per leaf in the same tile.
//
// A face is named by the corner with the smallest local index among those
// whose opposite corner is also a node, and that opposite corner (two
// opposite corners fix an axis-aligned box).  One CTA of HB_THREADS per tile
// sorts the (face, leaf, rank) keys of its slot-reading leaves in shared
// memory:
//   mode 0: count the faces;
//   mode 1: write the slots (corners, p) and point the leaves' unfilled
//           ranks at them (U + slot).
// Key: p (bits 62-63), first corner (46-61), opposite corner (30-45), leaf
// within the tile (4-13), rank (0-3); a tile's slots come sorted by p.
// A corner with no node is written as the tile's first sink (U + H), which
// reads 0 and is never written out.
// ---------------------------------------------------------------------------
constexpr int HB_THREADS = 256;

template <int NPE>
__global__ void __launch_bounds__(HB_THREADS) k_hns_build(
    int mode, const uint32_t *__restrict__ info, const int32_t *__restrict__ hidx, const int64_t *__restrict__ ls,
    const int64_t *__restrict__ off, uint16_t *__restrict__ e2l, const uint16_t *__restrict__ p2l, int cap,
    uint32_t *__restrict__ cnt, const int64_t *__restrict__ hs_off, uint16_t *__restrict__ hs_def,
    uint8_t *__restrict__ hs_p, int *__restrict__ err)
{
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t *key = reinterpret_cast<uint64_t *>(smem);            // [cap]
  __shared__ uint32_t part[HB_THREADS];
  const int64_t t = blockIdx.x;
  const int64_t l0 = ls[t];
  const int nl = (int) (ls[t + 1] - l0);
  const uint32_t U = (uint32_t) (off[t + 1] - off[t]);
  for (int s = threadIdx.x; s < cap; s += HB_THREADS) key[s] = ~0ull;
  __syncthreads();
  for (int j = threadIdx.x; j < nl; j += HB_THREADS) {
    const int64_t i = l0 + j;
    if (!(info[i] & INFO_HNS)) continue;
    const uint16_t *er = e2l + i * NPE, *pr = p2l + (int64_t) hidx[i] * NPE;
    for (int k = 1; k < NPE; k++) {
      if (er[k] != TL_NONE) continue;                    // filled
      uint32_t a = 0xFFFFu;
      int qa = -1;
      for (int q = 0; q < NPE; q++)
        if (!(q & ~k) && pr[q] < U && pr[q ^ k] < U && pr[q] < a) { a = pr[q]; qa = q; }
      if (qa < 0) { atomicOr(err, 1); continue; }       // excluded by k_hns_flag
      const uint32_t b = pr[qa ^ k];
      key[j * (NPE - 1) + (k - 1)] = ((uint64_t) __popc(k) << 62) | ((uint64_t) a << 46) | ((uint64_t) b << 30) |
                                     (uint64_t) ((j << 4) | k);
    }
  }
  __syncthreads();
  // bitonic sort, ascending
  for (int k = 2; k <= cap; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < cap; i += HB_THREADS) {
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
  // distinct faces (key >> 30): each thread owns a contiguous run of keys
  const int per = cap / HB_THREADS;   // cap is a multiple of HB_THREADS
  const int b0 = threadIdx.x * per;
  uint32_t c = 0;
  for (int k = b0; k < b0 + per; k++) {
    const uint64_t a = key[k];
    if (a != ~0ull && (k == 0 || (key[k - 1] >> 30) != (a >> 30))) c++;
  }
  part[threadIdx.x] = c;
  __syncthreads();
  for (int o = 1; o < HB_THREADS; o <<= 1) {
    const uint32_t v = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  if (mode == 0) {
    if (threadIdx.x == 0) cnt[t] = part[HB_THREADS - 1];
    return;
  }
  uint32_t rank = part[threadIdx.x] - c;
  const int64_t base = hs_off[t];
  const uint16_t sink = (uint16_t) (U + (hs_off[t + 1] - base));
  for (int k = b0; k < b0 + per; k++) {
    const uint64_t a = key[k];
    if (a == ~0ull) break;
    const bool head = (k == 0 || (key[k - 1] >> 30) != (a >> 30));
    if (head) rank++;
    const int j = (int) ((a >> 4) & 0x3FFu), r = (int) (a & 15u);
    const int64_t i = l0 + j;
    e2l[i * NPE + r] = (uint16_t) (U + rank - 1);
    if (head) {
      const uint16_t *pr = p2l + (int64_t) hidx[i] * NPE;
      uint16_t *row = hs_def + (base + rank - 1) * 8;
      int n = 0;
      for (int q = 0; q < NPE; q++)
        if (!(q & ~r)) row[n++] = pr[q] < U ? pr[q] : sink;
      for (; n < 8; n++) row[n] = sink;
      hs_p[base + rank - 1] = (uint8_t) __popc(r);
    }
  }
}

void tile_setup(Plan &pl, int T, cudaStream_t s)
{
  pl.tl_ready = false;
  pl.tl_T = 0;
  if (pl.order != 1 || pl.n_leaf == 0 || T <= 0) return;
  if (T < 32 || T > 1024 || (T & (T - 1))) throw std::invalid_argument("tile size must be a power of two in [32, 1024]");
  const int npe = pl.npe;
  if (npe != 4 && npe != 8 && npe != 16) throw std::invalid_argument("tiles need a Q1 plan");
  int cap = 1;
  while (cap < 2 * T * npe) cap <<= 1;
  cap = std::max(cap, TB_THREADS);
  if (cap > 65536) throw std::invalid_argument("tile too large");   // 16-bit local indices
  if (pl.n_nodes > (int64_t) TL_ID + 1) throw std::invalid_argument("too many nodes for tiles");
  const int64_t n_tile = (pl.n_leaf + T - 1) / T;
  // slot keys per tile: T (npe - 1) (leaf, rank) pairs
  int hcap = HB_THREADS;
  while (hcap < T * (npe - 1)) hcap <<= 1;
  const bool hns = pl.tl_hns_enable && (size_t) hcap * sizeof(uint64_t) <= 128 * 1024;
  k_hns_flag<<<grid_for(pl.n_leaf), 256, 0, s>>>(pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.fill.p, pl.n_leaf, npe,
                                                 pl.dim, pl.conforming ? 1 : 0, hns ? 1 : 0);
  check_launch("hns_flag");
  if (pl.seg.empty()) {
    // a single mesh: every tile's leaves in three runs (a batch keeps the
    // concatenated order of its meshes)
    DBuf<int32_t> e2n_o((size_t) pl.n_leaf * npe), hidx_o(pl.n_leaf);
    DBuf<uint32_t> info_o(pl.n_leaf);
    k_tile_partition<<<(unsigned) n_tile, T, 0, s>>>(pl.e2n.p, pl.info.p, pl.hidx.p, e2n_o.p, info_o.p, hidx_o.p,
                                                     pl.n_leaf, T, npe);
    check_launch("tile_partition");
    DKT_CUDA(cudaStreamSynchronize(s));
    pl.e2n = std::move(e2n_o);
    pl.info = std::move(info_o);
    pl.hidx = std::move(hidx_o);
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
  {
    // the hanging leaves left to the per-leaf kernel
    DBuf<uint32_t> f(pl.n_leaf), pos(pl.n_leaf);
    DBuf<int32_t> iota(pl.n_leaf);
    k_flag_rest<<<grid_for(pl.n_leaf), 256, 0, s>>>(pl.info.p, f.p, pl.n_leaf);
    k_iota_i32<<<grid_for(pl.n_leaf), 256, 0, s>>>(iota.p, pl.n_leaf);
    pl.tl_n_rest = (int64_t) exclusive_scan_total<uint32_t>(f.p, pos.p, pl.n_leaf, s);
    pl.tl_rest.alloc(std::max<int64_t>(pl.tl_n_rest, 1));
    scatter_if_kernel<int32_t><<<grid_for(pl.n_leaf), 256, 0, s>>>(iota.p, f.p, pos.p, pl.tl_rest.p, pl.n_leaf);
    check_launch("rest_leaves");
    DKT_CUDA(cudaStreamSynchronize(s));
    pl.tl_n_hleaf = pl.n_hang - pl.tl_n_rest;
  }
  DBuf<uint32_t> node_tiles(pl.n_nodes), cnt(n_tile);
  DKT_CUDA(cudaMemsetAsync(node_tiles.p, 0, pl.n_nodes * sizeof(uint32_t), s));
  const size_t smem = (size_t) cap * sizeof(uint64_t);
  ensure_dyn_smem(k_tile_build, smem);
  k_tile_build<<<(unsigned) n_tile, TB_THREADS, smem, s>>>(0, pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.n_leaf,
                                                          npe, T, cap, node_tiles.p, cnt.p, nullptr, nullptr,
                                                          nullptr, nullptr, nullptr);
  check_launch("tile_count");
  // offsets (host scan: one value per tile)
  std::vector<uint32_t> hc(n_tile);
  DKT_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, n_tile * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaStreamSynchronize(s));
  std::vector<int64_t> ho(n_tile + 1, 0);
  for (int64_t t = 0; t < n_tile; t++) ho[t + 1] = ho[t] + hc[t];
  pl.tl_off.upload(ho.data(), ho.size(), s);
  pl.tl_nodes.alloc(std::max<int64_t>(ho[n_tile], 1));
  pl.tl_e2l.alloc((size_t) pl.n_leaf * npe);
  // tile-local parent maps: only for building the slots
  DBuf<uint16_t> p2l((size_t) std::max<int64_t>(pl.n_hang, 1) * npe);
  DKT_CUDA(cudaMemsetAsync(pl.tl_e2l.p, 0xFF, (size_t) pl.n_leaf * npe * sizeof(uint16_t), s));
  DKT_CUDA(cudaMemsetAsync(p2l.p, 0xFF, (size_t) std::max<int64_t>(pl.n_hang, 1) * npe * sizeof(uint16_t), s));
  k_tile_build<<<(unsigned) n_tile, TB_THREADS, smem, s>>>(1, pl.e2n.p, pl.info.p, pl.hidx.p, pl.p2n.p, pl.n_leaf,
                                                          npe, T, cap, node_tiles.p, cnt.p, pl.tl_off.p,
                                                          pl.tl_nodes.p, pl.tl_e2l.p, p2l.p,
                                                          pl.fx_kappa > 0 ? pl.fx_lam.p : nullptr);
  check_launch("tile_fill");
  pl.tl_lstart.alloc(n_tile + 1);
  k_tile_lstart<<<grid_for(n_tile + 1), 256, 0, s>>>(pl.tl_lstart.p, n_tile, T, pl.n_leaf);
  // hanging-node slots
  std::vector<int64_t> hso(n_tile + 1, 0);
  DBuf<int> err(1);
  DKT_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  auto kb = npe == 16 ? k_hns_build<16> : npe == 8 ? k_hns_build<8> : k_hns_build<4>;
  const size_t hsm = (size_t) hcap * sizeof(uint64_t);
  if (hns && pl.tl_n_hleaf > 0) {
    ensure_dyn_smem(kb, hsm);
    kb<<<(unsigned) n_tile, HB_THREADS, hsm, s>>>(0, pl.info.p, pl.hidx.p, pl.tl_lstart.p, pl.tl_off.p, pl.tl_e2l.p,
                                                   p2l.p, hcap, cnt.p, nullptr, nullptr, nullptr, err.p);
    check_launch("hns_count");
    DKT_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, n_tile * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    DKT_CUDA(cudaStreamSynchronize(s));
    for (int64_t t = 0; t < n_tile; t++) hso[t + 1] = hso[t] + hc[t];
  }
  uint32_t umax = 0, hmax = 0;
  for (int64_t t = 0; t < n_tile; t++) {
    umax = std::max<uint32_t>(umax, (uint32_t) (ho[t + 1] - ho[t] + hso[t + 1] - hso[t]));
    hmax = std::max<uint32_t>(hmax, (uint32_t) (hso[t + 1] - hso[t]));
  }
  // U + H + TL_SINKS below TL_NONE keeps every local index clear of it
  if ((int64_t) umax + TL_SINKS >= (int64_t) TL_NONE) throw std::invalid_argument("tile too large");
  pl.tl_hs_off.upload(hso.data(), hso.size(), s);
  pl.tl_n_hs = hso[n_tile];
  pl.tl_hs_def.alloc((size_t) std::max<int64_t>(pl.tl_n_hs, 1) * 8);
  pl.tl_hs_p.alloc((size_t) std::max<int64_t>(pl.tl_n_hs, 1));
  if (pl.tl_n_hs > 0) {
    kb<<<(unsigned) n_tile, HB_THREADS, hsm, s>>>(1, pl.info.p, pl.hidx.p, pl.tl_lstart.p, pl.tl_off.p, pl.tl_e2l.p,
                                                   p2l.p, hcap, cnt.p, pl.tl_hs_off.p, pl.tl_hs_def.p, pl.tl_hs_p.p,
                                                   err.p);
    check_launch("hns_fill");
  }
  int herr = 0;
  DKT_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaStreamSynchronize(s));
  if (herr) throw std::runtime_error("hanging-node slot build: a face without two opposite nodes");
  k_tile_sinks<<<(unsigned) n_tile, T, 0, s>>>(pl.tl_e2l.p, pl.tl_lstart.p, pl.tl_off.p, pl.tl_hs_off.p, npe);
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
  pl.tl_hmax = hmax;
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
    atomicAdd(reinterpret_cast<int *>(a + U) + u, hi + ((uint32_t) (old + lo) < old ? 1 : 0));
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

// A thread's node slots of the tile are visited in groups of four, the four
// id loads issued before anything that depends on them: one global round trip
// per group for the ids and one for the values, instead of two per slot.
constexpr int TILE_G = 4;

// The tile's node values into shared memory (and its node entries into sid
// for the flush), its slot definitions into srow / sp (loads issued first,
// independent of the node loads), sums zeroed.
template <int T_LEAVES, typename V, typename ACC>
__device__ __forceinline__ void tile_gather(const uint32_t *__restrict__ tile_nodes, int64_t u0, int U, int H,
                                            int Us, const V *__restrict__ xq, V *xs, uint32_t *ys, uint32_t *sid,
                                            int64_t hs0, const uint16_t *__restrict__ hs_def,
                                            const uint8_t *__restrict__ hs_p, uint4 *srow, uint8_t *sp)
{
  for (int q = threadIdx.x; q < H; q += T_LEAVES) {
    srow[q] = __ldg(reinterpret_cast<const uint4 *>(hs_def) + hs0 + q);
    sp[q] = hs_p[hs0 + q];
  }
  // the hanging-node slots and the sinks: sums zeroed, sinks read 0
  for (int u = U + threadIdx.x; u < Us; u += T_LEAVES) {
    if (u >= U + H) xs[u] = V(0);
    ACC::zero(ys, Us, u);
  }
  for (int b = threadIdx.x; b < U; b += TILE_G * T_LEAVES) {
    uint32_t id[TILE_G];
    V xv[TILE_G];
#pragma unroll
    for (int j = 0; j < TILE_G; j++) {
      const int u = b + j * T_LEAVES;
      id[j] = u < U ? __ldg(tile_nodes + u0 + u) : 0u;
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
// added atomically elsewhere.  put(id, u) writes slot u to node id (the
// node entries staged in sid by the gather).
template <int T_LEAVES, typename PUT>
__device__ __forceinline__ void tile_scatter(const uint32_t *sid, int U, PUT put)
{
  for (int u = threadIdx.x; u < U; u += T_LEAVES) put(sid[u], u);
}

// The 2^p corners of a slot (local indices packed two to a word), one
// unrolled body per p: a tile's slots come sorted by p, so the warps of a
// slot phase mostly take one branch.
template <int P, typename F>
__device__ __forceinline__ void for_corners(const uint32_t (&cw)[4], F f)
{
#pragma unroll
  for (int c = 0; c < (1 << P); c++) f((cw[c >> 1] >> ((c & 1) * 16)) & 0xFFFFu);
}
template <int DIM, typename F>
__device__ __forceinline__ void corners_of(int p, const uint32_t (&cw)[4], F f)
{
  if (p == 1) for_corners<1>(cw, f);
  if constexpr (DIM >= 3) if (p == 2) for_corners<2>(cw, f);
  if constexpr (DIM >= 4) if (p == 3) for_corners<3>(cw, f);
}

// Hanging-node slot values: the mean of each slot's face corners (2^p of
// them, 1 <= p < DIM; a corner with no node is a sink and reads 0).  The
// slot definitions are staged in shared memory (srow, sp) by the gather.
template <int DIM, int T_LEAVES, bool FX, typename V>
__device__ __forceinline__ void slot_means(V *xs, int U, int H, const uint4 *srow, const uint8_t *sp)
{
  for (int q = threadIdx.x; q < H; q += T_LEAVES) {
    const int p = sp[q];
    const uint4 rw = srow[q];
    const uint32_t cw[4] = {rw.x, rw.y, rw.z, rw.w};
    V acc = V(0);
    corners_of<DIM>(p, cw, [&](uint32_t c) { acc += xs[c]; });
    if constexpr (FX) xs[U + q] = acc >> p;
    else xs[U + q] = acc * (1.0f / (float) (1 << p));
  }
}

// Each slot's sum to every corner of its face (the transposed interpolation).
template <int DIM, int T_LEAVES, typename ADD>
__device__ __forceinline__ void slot_sums_out(int U, int H, const uint4 *srow, const uint8_t *sp, ADD add)
{
  for (int q = threadIdx.x; q < H; q += T_LEAVES) {
    const int p = sp[q];
    const uint4 rw = srow[q];
    const uint32_t cw[4] = {rw.x, rw.y, rw.z, rw.w};
    add(U + q, [&](auto put) { corners_of<DIM>(p, cw, put); });
  }
}

// SC (fixed point only): 0 = per-(level, mode) multiply-high factors of the
// tile's unit (fm: the per-unit factor table); 1, 2, 3 = dyadic scaling with
// the Laplacian term (bit 0) and / or the mass term (bit 1), fm then pointing
// at the per-level shift words.
// One tile (one CTA's work); uniform exits only.  Every hanging leaf handled
// here reads hanging-node slots; the other hanging leaves (info bit 28 clear)
// are the per-leaf kernel's, and their threads idle.
template <int DIM, int T_LEAVES, typename AR, int SC>
__device__ __forceinline__ void q1t_tile(
    const int64_t tile, const uint16_t *__restrict__ e2l, const uint32_t *__restrict__ info,
    const int64_t *__restrict__ tile_off, const int64_t *__restrict__ tile_ls,
    const uint32_t *__restrict__ tile_nodes, const void *__restrict__ fm, int n_fac,
    const typename AR::T *__restrict__ xq, typename AR::T *__restrict__ yq, int conforming,
    const int32_t *__restrict__ tile_mlo, const int32_t *__restrict__ tile_mhi, const int *__restrict__ skip_mesh,
    int skip_stride, const DyConst &dyc, const uint8_t *__restrict__ tile_tau, int kappa,
    const int64_t *__restrict__ hs_off, const uint16_t *__restrict__ hs_def, const uint8_t *__restrict__ hs_p,
    int smax, int hmax)
{
  using V = typename AR::T;
  using F = typename AR::Factor;
  constexpr int NPE = 1 << DIM;
  constexpr bool FX = std::is_same<AR, FixedArith>::value;
  static_assert(FX || SC == 0, "dyadic scaling is a fixed-point form");
  using ACC = TileAcc<AR>;
  extern __shared__ __align__(16) unsigned char smem[];
  // a batched solve: tiles whose meshes have all converged are not needed
  if (skip_mesh && skip_mesh[(int64_t) tile_mlo[tile] * skip_stride] &&
      skip_mesh[(int64_t) tile_mhi[tile] * skip_stride])
    return;
  const int64_t u0 = tile_off[tile];
  const int U = (int) (tile_off[tile + 1] - u0);
  const int64_t hs0 = hs_off[tile];
  const int H = (int) (hs_off[tile + 1] - hs0);
  const int64_t i = tile_ls[tile] + threadIdx.x;
  bool valid = i < tile_ls[tile + 1];
  // the leaf's records first, so their latency overlaps the node gather
  uint32_t inf = 0;
  uint32_t w[NPE / 2];
  if (valid) {
    inf = __ldg(info + i);
    if (((inf >> 16) & 1u) && !(inf & INFO_HNS)) valid = false;
  }
  if (valid) load_row16<NPE>(e2l + i * NPE, w);
  const bool hang = valid && ((inf >> 16) & 1u);
  F *fac = reinterpret_cast<F *>(smem);
  uint32_t *fsh = reinterpret_cast<uint32_t *>(smem);     // SC != 0: per-level shift words
  const int Us = U + H + TL_SINKS;                        // the tile's nodes, its slots, the sinks
  const int fac_bytes = SC ? ((n_fac * 4 + 15) & ~15) : n_fac * (int) sizeof(F);
  V *xs = reinterpret_cast<V *>(smem + fac_bytes);
  uint32_t *ys = reinterpret_cast<uint32_t *>(xs + Us);  // ACC::WORDS words per entry
  // staged slot definitions, past the largest tile's node and slot sums
  uint4 *srow = reinterpret_cast<uint4 *>(smem + ((fac_bytes + (size_t) 2 * smax * sizeof(V) + 15) & ~(size_t) 15));
  uint32_t *sid = reinterpret_cast<uint32_t *>(srow + hmax);   // the tile's node entries
  uint8_t *sp = reinterpret_cast<uint8_t *>(sid + smax);
  // the tile's fixed-point unit: its coarsest leaf level (factor table row)
  const int tau = FX ? (int) tile_tau[tile] : 0;
  for (int k = threadIdx.x; k < n_fac; k += T_LEAVES) {
    if constexpr (SC != 0) fsh[k] = static_cast<const uint32_t *>(fm)[k];
    else fac[k] = AR::load_factor(fm, tau * n_fac + k);
  }
  tile_gather<T_LEAVES, V, ACC>(tile_nodes, u0, U, H, Us, xq, xs, ys, sid, hs0, hs_def, hs_p, srow, sp);
  __shared__ uint32_t s_max;
  if (threadIdx.x == 0) s_max = 0u;
  __syncthreads();
  if (H > 0) {
    slot_means<DIM, T_LEAVES, FX, V>(xs, U, H, srow, sp);
    __syncthreads();
  }
  auto lidx = [&](int k) -> uint32_t { return idx16<NPE>(w, k); };
  V v[NPE];
  if (valid) {
    const int L = inf & 0xFFu;
    // a hanging leaf's unfilled ranks read their slots (the parent-face means)
#pragma unroll
    for (int k = 0; k < NPE; k++) v[k] = xs[lidx(k)];
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
    // a hanging leaf's unfilled ranks (their local index is a slot's): the
    // transposed interpolation weight 2^-popcount, into the slot
    if constexpr (FX) {
      // the reference transpose leaves out the shared parent corner (rank 0
      // is always filled), which the slots' sums reach: the leaf's share is
      // taken back at its rank-0 node, the same corner, added last
      const bool back_out = hang && !conforming;
      V back = V(0);
#pragma unroll
      for (int k = 1; k < NPE; k++) {
        if (hang && lidx(k) >= (uint32_t) U) {
          v[k] >>= __popc(k);
          if (back_out) back += v[k];
        }
        ACC::add(ys, Us, lidx(k), v[k]);
      }
      ACC::add(ys, Us, lidx(0), v[0] - back);
    } else if (hang) {
#pragma unroll
      for (int k = 1; k < NPE; k++)
        if (lidx(k) >= (uint32_t) U) v[k] *= 1.0f / (float) (1 << __popc(k));
    }
  }
  if constexpr (!FX) {
    // binary32: the tile's contributions are quantised against the tile's
    // largest one (22 bits) and summed with native integer shared atomics;
    // each node's sum goes out with one float atomic.  The rounding to an
    // integer is one fused multiply-add: v * up + 1.5 * 2^23 lands in
    // [2^23, 2^24), where binary32 spacing is 1, for |v * up| < 2^22, and its
    // bits less those of 1.5 * 2^23 are the rounded integer.
    float m = 0.0f;
    if (valid) {
#pragma unroll
      for (int k = 0; k < NPE; k++)
        if (lidx(k) < (uint32_t) (U + H)) m = fmaxf(m, fabsf(v[k]));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&s_max, __float_as_uint(m));
    __syncthreads();
    int e = 0;
    frexpf(__uint_as_float(s_max), &e);              // max < 2^e
    const float up = ldexpf(1.0f, 22 - e);
    auto quant = [up](float v) { return __float_as_int(fmaf(v, up, 12582912.0f)) - 0x4B400000; };
    if (valid) {
      // the shared parent corner's share taken back at rank 0 (reference
      // traversal), in integers
      const bool back_out = hang && !conforming;
      int back = 0, q0 = 0;
#pragma unroll
      for (int k = 0; k < NPE; k++) {
        const int qv = quant(v[k]);
        if (k == 0) {
          q0 = qv;
        } else {
          if (back_out && lidx(k) >= (uint32_t) U) back += qv;
          atomicAdd(reinterpret_cast<int *>(ys) + lidx(k), qv);
        }
      }
      atomicAdd(reinterpret_cast<int *>(ys) + lidx(0), q0 - back);
    }
    __syncthreads();
    if (H > 0) {
      slot_sums_out<DIM, T_LEAVES>(U, H, srow, sp, [&](int u, auto each) {
        const int a = reinterpret_cast<const int *>(ys)[u];
        if (a != 0) each([&](uint32_t c) { atomicAdd(reinterpret_cast<int *>(ys) + c, a); });
      });
      __syncthreads();
    }
    const float down = ldexpf(1.0f, e - 22);
    tile_scatter<T_LEAVES>(sid, U, [&](uint32_t id, int u) {
      const int a = reinterpret_cast<const int *>(ys)[u];
      if (id & TL_EXCL) yq[id & TL_ID] = (V) a * down;
      else if (a != 0) atomicAdd(yq + (id & TL_ID), (V) a * down);
    });
    return;
  }
  __syncthreads();
  if (H > 0) {
    slot_sums_out<DIM, T_LEAVES>(U, H, srow, sp, [&](int u, auto each) {
      const V a = ACC::get(ys, Us, u);
      if (a != V(0)) each([&](uint32_t c) { ACC::add(ys, Us, c, a); });
    });
    __syncthreads();
  }
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
    const uint16_t *__restrict__ e2l, const uint32_t *__restrict__ info, const int64_t *__restrict__ tile_off,
    const int64_t *__restrict__ tile_ls, const uint32_t *__restrict__ tile_nodes, const void *__restrict__ fm,
    int n_fac, const typename AR::T *__restrict__ xq, typename AR::T *__restrict__ yq, int conforming,
    const int32_t *__restrict__ tile_mlo, const int32_t *__restrict__ tile_mhi, const int *__restrict__ skip_mesh,
    int skip_stride, const __grid_constant__ DyConst dyc, const uint8_t *__restrict__ tile_tau, int kappa,
    unsigned long long *__restrict__ counter, int64_t n_tile, const int64_t *__restrict__ hs_off,
    const uint16_t *__restrict__ hs_def, const uint8_t *__restrict__ hs_p, int smax, int hmax)
{
  if constexpr (!PERSIST) {
    q1t_tile<DIM, T_LEAVES, AR, SC>(blockIdx.x, e2l, info, tile_off, tile_ls, tile_nodes, fm, n_fac, xq, yq,
                                    conforming, tile_mlo, tile_mhi, skip_mesh, skip_stride, dyc, tile_tau, kappa,
                                    hs_off, hs_def, hs_p, smax, hmax);
    return;
  } else {
  __shared__ long long s_tile;
  for (;;) {
    if (threadIdx.x == 0) s_tile = (long long) atomicAdd(counter, 1ull);
    __syncthreads();
    const int64_t t = s_tile;
    __syncthreads();                 // every thread has read s_tile
    if (t >= n_tile) return;
    q1t_tile<DIM, T_LEAVES, AR, SC>(t, e2l, info, tile_off, tile_ls, tile_nodes, fm, n_fac, xq, yq, conforming,
                                    tile_mlo, tile_mhi, skip_mesh, skip_stride, dyc, tile_tau, kappa, hs_off,
                                    hs_def, hs_p, smax, hmax);
    __syncthreads();                 // the tile's shared memory is free again
  }
  }
}

template <int DIM, int TL, typename AR, int SC>
static void launch_tiled(Plan &pl, const void *fm, const typename AR::T *x, typename AR::T *y, cudaStream_t s)
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
  // tl_umax: the largest U + H of a tile; then the staged slot definitions
  // (16 + 1 bytes per slot of the tile with most) and node entries (4 bytes)
  const int smax = (int) pl.tl_umax + TL_SINKS, hmax = (int) pl.tl_hmax;
  const size_t smem = ((fac_bytes + (size_t) 2 * smax * sizeof(typename AR::T) + 15) & ~(size_t) 15) +
                      (size_t) hmax * 17 + (size_t) smax * 4;
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
  kfn<<<grid, TL, smem, s>>>(pl.tl_e2l.p, pl.info.p, pl.tl_off.p, pl.tl_lstart.p, pl.tl_nodes.p, fm, n_fac, x, y,
                             pl.conforming ? 1 : 0, pl.tl_mlo.p, pl.tl_mhi.p, pl.tl_mlo.p ? pl.skip_mesh : nullptr,
                             pl.skip_stride, dyc, pl.tl_tau.p,
                             std::is_same<AR, FixedArith>::value ? pl.fx_kappa : 0, counter, pl.tl_n,
                             pl.tl_hs_off.p, pl.tl_hs_def.p, pl.tl_hs_p.p, smax, hmax);
}

template <typename AR, int SC>
static void launch_tiled_dim(Plan &pl, const void *fm, const typename AR::T *x, typename AR::T *y, cudaStream_t s)
{
#define DKT_TL_CASE(D, TL) \
  case (D) * 10000 + (TL): launch_tiled<D, TL, AR, SC>(pl, fm, x, y, s); break;
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

// Every leaf but the hanging leaves that read no hanging-node slots (the
// per-leaf kernel's, over pl.tl_rest).
void tiled_fixed(Plan &pl, cudaStream_t s)
{
  switch (pl.fx_scale) {
#define DKT_SC_CASE(SC, FM) case SC: launch_tiled_dim<FixedArith, SC>(pl, FM, pl.xq.p, pl.yq.p, s); break;
    DKT_SC_CASE(0, pl.fx_fm.p) DKT_SC_CASE(1, pl.fx_shift.p) DKT_SC_CASE(2, pl.fx_shift.p) DKT_SC_CASE(3, pl.fx_shift.p)
#undef DKT_SC_CASE
    default: throw std::runtime_error("bad fixed-point scaling mode");
  }
}

void tiled_f32(Plan &pl, const float *x, float *y, cudaStream_t s)
{
  launch_tiled_dim<F32Arith, 0>(pl, pl.f32_f.p, x, y, s);
}

bool tile_size_supported(int dim, int T)
{
  if (dim == 4) return T == 64 || T == 128 || T == 256;
  return T == 128 || T == 256 || T == 512;
}

}  // namespace dkt
