// Shared definitions of the GB300 implementation of the k-tree matvec path:
// SFC digit arithmetic, device-resident DA and matvec-plan structures.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>
#include "dkt_prims.cuh"

namespace dkt {

constexpr int MAX_DIM = 4;
constexpr int MAX_NPE = 81;   // (p+1)^dim for p <= 2, dim <= 4

// Curve tables in the reference's layout (src/KDhcurvedata.cpp, hcurvedata.h):
//   rot[r*2*nc + sfc]      = Morton child visited at SFC position sfc
//   rot[r*2*nc + nc + m]   = SFC position of Morton child m
//   ht[r*nc + m]           = orientation of Morton child m
struct CurveDev {
  const int8_t *rot = nullptr;
  const int32_t *ht = nullptr;
  int nrot = 1;
};

struct CurveHost {
  std::vector<int8_t> rot;
  std::vector<int32_t> ht;
  int nrot = 1;
  DBuf<int8_t> drot;
  DBuf<int32_t> dht;
  void morton(int dim)
  {
    const int nc = 1 << dim;
    rot.assign(2 * nc, 0);
    ht.assign(nc, 0);
    for (int c = 0; c < nc; c++) { rot[c] = (int8_t) c; rot[nc + c] = (int8_t) c; }
    nrot = 1;
  }
  void upload()
  {
    drot.upload(rot.data(), rot.size());
    dht.upload(ht.data(), ht.size());
  }
  CurveDev dev() const { return CurveDev{drot.p, dht.p, nrot}; }
};

// Bits needed to store 0..nc (a child rank plus one sentinel).
__host__ __device__ inline int slot_bits(int dim) { return dim == 2 ? 3 : dim == 3 ? 4 : 5; }

// getMortonIndex(level) (include/treeNode.tcc:244-258) for coordinates < 2^(md+1).
__host__ __device__ inline unsigned morton_at(const uint32_t *x, int dim, int md, int lev)
{
  unsigned c = 0;
  const int sh = md - lev;
  for (int d = 0; d < dim; d++) c |= ((x[d] >> sh) & 1u) << d;
  return c;
}

// 128-bit builder: appends fields most-significant first.
struct KeyBuilder {
  uint64_t hi = 0, lo = 0;
  int used = 0;
  __host__ __device__ void push(uint64_t v, int bits)
  {
    if (bits == 0) return;
    hi = (hi << bits) | (bits < 64 ? (lo >> (64 - bits)) : lo);
    lo = (bits < 64) ? ((lo << bits) | v) : v;
    used += bits;
  }
  // Left-align to a total width W so keys with different layouts compare on
  // their first field.
  __host__ __device__ Key128 finish(int W)
  {
    const int s = W - used;
    if (s > 0) {
      if (s >= 64) { hi = lo << (s - 64); lo = 0; }
      else { hi = (hi << s) | (lo >> (64 - s)); lo <<= s; }
    }
    return Key128{lo, hi};
  }
};

// SFC tree-sort key of a cell (SFC_Tree::locTreeSort, include/tsort.tcc:14-80):
// for levels 1..md the SFC rank of the child taken at that level plus one, and
// 0 below the cell's own level, so ancestors precede descendants.
__host__ __device__ inline uint64_t tree_key(const uint32_t *x, int lev, int dim, int md, CurveDev cv)
{
  const int nc = 1 << dim, B = slot_bits(dim);
  uint64_t k = 0;
  int r = 0;
  for (int l = 1; l <= md; l++) {
    unsigned v = 0;
    if (l <= lev) {
      const unsigned m = morton_at(x, dim, md, l);
      v = (unsigned) cv.rot[r * 2 * nc + nc + m] + 1u;
      r = cv.ht[r * nc + m];
    }
    k = (k << B) | v;
  }
  return k;
}

// Node key used for exact coordinate lookups: coordinates concatenated with
// md+1 bits per axis (coordinates may equal 2^md on the upper boundary).
__host__ __device__ inline uint64_t coord_key(const uint32_t *x, int dim, int md)
{
  uint64_t k = 0;
  for (int d = dim - 1; d >= 0; d--) k = (k << (md + 1)) | x[d];
  return k;
}

// Cell key for set membership: level in the top bits, anchor below.
__host__ __device__ inline uint64_t cell_key(const uint32_t *a, int lev, int dim, int md)
{
  uint64_t k = (uint64_t) lev;
  for (int d = dim - 1; d >= 0; d--) k = (k << md) | a[d];
  return k;
}

// Status of the allocation-free product (dkt_matvec.cu).
enum { NOALLOC_OK = 0, NOALLOC_TOO_LARGE = 1, NOALLOC_CUDA = 2 };

// Device-resident distributed array (ot::DA on one rank).
struct DA {
  int dim = 3, order = 1, md = 10, curve = 0;
  int64_t n_elem = 0, n_nodes = 0, n_bdry = 0;
  CurveHost cv;
  DBuf<uint32_t> elem_x;     // [n_elem][dim], SFC order
  DBuf<uint8_t> elem_lev;
  DBuf<uint32_t> node_x;     // [n_nodes][dim], DA order
  DBuf<uint8_t> node_lev;
  DBuf<uint32_t> bdry;       // boundary node ids, ascending
};

// Elemental operator K_L = alpha[L] * A + beta[L] * B (dense nPe x nPe, the
// reference's lexicographic node order, x fastest), or one dense table per
// level when kind == custom.
enum OpKind { OP_IDENTITY = 0, OP_HEAT = 1, OP_LAPMASS = 2, OP_CUSTOM = 3, OP_LAPLACE = 4, OP_MASS = 5, OP_HEATVEC = 6 };
// operators whose feMatrix pre/post steps zero the domain-boundary entries
__host__ __device__ inline bool op_has_bc(int k)
{
  return k == OP_HEAT || k == OP_LAPMASS || k == OP_LAPLACE || k == OP_HEATVEC;
}

struct Operator {
  int kind = OP_LAPMASS;
  int npe = 8, nlev = 11;
  bool uses_scale = true;            // HeatMat ignores the scale argument
  std::vector<double> A, B;          // npe*npe each (row r = output, col c = input)
  std::vector<double> alpha, beta;   // per level
  std::vector<double> table;         // custom: nlev*npe*npe
};

// Flattened traversal: one record per leaf visit of fem::matvec.
struct Plan {
  int dim = 3, order = 1, md = 10, npe = 8;
  // false: the reference traversal (parent values only from level L-1 nodes,
  // transpose masked by the leaf fill mask); true: the conforming P^T K P
  bool conforming = false;
  int64_t n_nodes = 0, n_leaf = 0, n_hang = 0, n_bdry = 0;
  int64_t stale_slots = 0;           // parent slots read unfilled with nonzero weight
  DBuf<int32_t> e2n;                 // [n_leaf][npe]  node index or -1
  DBuf<uint32_t> info;               // [n_leaf] level | child<<8 | hanging<<16 | rank among the tile's hanging leaves<<17 | reads stale slots<<27
  DBuf<int32_t> hidx;                // [n_leaf] index into hanging arrays or -1
  DBuf<int32_t> p2n;                 // [n_hang][npe] parent node index (level L-1) or -1
  DBuf<uint32_t> fill;               // [n_hang][3] filled-rank bitmask of the leaf
  DBuf<uint32_t> bdry;               // boundary node ids
  DBuf<double> opA, opB, opAlpha, opBeta, opTable;
  DBuf<double> ip;                   // [2][M][M] child interpolation (ip_1D_0, ip_1D_1)
  Operator op;
  DBuf<double> xin;                  // scratch: boundary-zeroed input
  DBuf<double> xh, yh;               // device copies for the host-array entry point
  // Emulation of the reference's static parent buffer (dkt_stale.cu).
  bool st_ready = false;
  int64_t st_start = 0, st_n_ent = 0, st_n_runs = 0;
  DBuf<int32_t> st_row, st_idx, st_runs, st_hzoff, st_hztab, st_srow, st_sidx, st_gstart;
  // order 2: per group the child number and the need / take slot masks
  // ([G][6]: needed slots, slots taken from the previous group), walked as a
  // tensor-product interpolation instead of per-entry term lists
  bool st_tp = false;
  double st_pint[3] = {0, 0, 0};
  DBuf<int32_t> st_gchild;
  DBuf<uint32_t> st_gmask;
  DBuf<double> st_w, st_v, st_sw, st_f;
  DBuf<long long> st_vq;
  DBuf<int32_t> st_hleaves;          // leaves that read stale slots (info bit 27)
  int64_t st_n_hleaf = 0;
  cudaStream_t st_stream = nullptr;  // side stream of the chain, with its fork/join events
  cudaEvent_t st_fork = nullptr, st_join = nullptr;
  // Exact fixed-point path of the Q1 built-in operators (dkt_q1fx.cu).
  int arith = 0;                     // 0 auto, 1 native FP64, 2 fixed point
  bool fx_ready = false;
  int fx_c = 0;
  DBuf<long long> fx_fm, xq, yq;     // fx_fm: [unit level tau][leaf level L][mode] (q1fx_setup)
  DBuf<int> fx_sx;
  // Dyadic scaling (every level factor of the operator a power of two or
  // zero): 0 = multiply-high factors; 1 / 2 / 3 = the tiled kernel scales a
  // mode value with small integer multiples and shifts (Laplacian term, mass
  // term, both; fx_shift[L] = s_L | d_L << 8), and yq carries fx_div = 3^dim
  // times the product.  |xq| <= 2^fx_bx.
  int fx_scale = 0, fx_div = 1, fx_bx = 56;
  DBuf<uint32_t> fx_shift;
  // Per-level units: a level-L leaf's contributions are exact in a unit
  // 2^(-kappa L) times the level-0 unit, kappa the level exponent of the
  // operator's leading term (dim - 2 for the Laplacian, dim for the mass);
  // node n keeps its sum in the unit of fx_lam[n], the coarsest level of a
  // leaf adding into it, and a tile computes in the unit of tl_tau[t], its
  // coarsest leaf level.  kappa = 0: one unit for all.
  int fx_kappa = 0;
  DBuf<uint8_t> fx_lam;
  DBuf<unsigned long long> fx_amax;
  // Sum-factorised order-2 kernel (dkt_q2sf.cu): 1D transform T (row-major),
  // child-interpolation middle row, per-level diagonals, hanging-first order.
  bool sf_ready = false, sf_split = false;
  int64_t sf_n_main = 0;             // leaves of the main launch (all, or those reading no stale slot)
  double sf_T[9] = {0}, sf_pint[3] = {0};
  DBuf<double> sf_D;
  DBuf<float> sf_D32;
  DBuf<int32_t> sf_order;
  // binary32 variant of the same Q1 operators (inner solves).
  bool f32_ready = false;
  DBuf<float> f32_f, x32;
  // Tiles of the Q1 kernels (dkt_tile.cu): T leaves per tile, per-tile
  // distinct-node lists and 16-bit local maps.
  bool tl_ready = false;
  int tl_T = 0;
  int64_t tl_n = 0, tl_sum_u = 0;
  uint32_t tl_umax = 0;
  DBuf<int64_t> tl_off, tl_lstart, tl_hb;   // per tile: node-list offset, first leaf, first hanging index
  DBuf<uint32_t> tl_nodes, tl_fm;     // distinct nodes (| exclusive flag); reflected fill masks
  DBuf<uint16_t> tl_e2l, tl_p2l;
  DBuf<uint8_t> tl_tau;              // per tile: coarsest leaf level (its fixed-point unit)
  // the node entries again at fixed stride tl_cap per tile (padded with node
  // 0), and each tile's count: the leaf kernel reads a tile's entries without
  // first reading its offset (one dependent global load fewer per tile)
  DBuf<uint32_t> tl_pad;
  DBuf<int32_t> tl_ucnt;
  int tl_cap = 0;
  bool tl_ls_direct = false;         // tile t's leaves start at t * tl_T (false: tl_lstart, a batch)
  DBuf<int32_t> leaf_sfc;            // position in the traversal's (SFC) order of each leaf record, once tiled
  // persistent tiled launch (CTAs pull tiles from a counter) instead of one
  // CTA per tile; chosen by dkt_plan_autotune
  bool tl_persist = false;
  DBuf<unsigned long long> tl_counter;
  // Optional CUDA-event timing of the leaf kernel on its launching stream.
  bool timing = false;
  std::vector<cudaEvent_t> ev;       // start/stop pairs of the current window
  int64_t timed_launches = 0;
  // Kernels this plan's products have launched (all of them, cumulative).
  int64_t n_launch = 0;
  // mixed-precision solves that finished on the FP64 fallback
  int64_t fallbacks = 0;
  // batches (dkt_batch.cu): node offset of every mesh, plus the end; empty
  // for a single mesh
  std::vector<int64_t> seg, lseg;    // node and leaf offsets of the meshes
  DBuf<int32_t> tl_mlo, tl_mhi;      // per tile: first and last mesh it covers (batches)
  // While a batched solve captures its iterations: per-mesh converged flags
  // (stride in ints); tiles whose meshes have all converged are skipped.
  const int *skip_mesh = nullptr;
  int skip_stride = 1;
  // stale-chain shape: longest run in groups and in entries
  int64_t st_max_run_groups = 0, st_max_run_ents = 0;

  Plan() = default;
  Plan(const Plan &) = delete;
  Plan &operator=(const Plan &) = delete;
  ~Plan()
  {
    if (st_stream) cudaStreamDestroy(st_stream);
    if (st_fork) cudaEventDestroy(st_fork);
    if (st_join) cudaEventDestroy(st_join);
  }
};

}  // namespace dkt
