// Batches of independent meshes as one block-diagonal plan.
//
// The flattened traversals of P plans are concatenated with their node,
// hanging-leaf and tile numbers offset, so one launch of the leaf kernel
// (tiles never straddle two meshes) computes all P products, and the vector
// kernels of the solver work on the concatenated vectors with per-mesh
// segments (Plan::seg).  Plans of one batch share dimension, order, maximum
// depth, operator and traversal; the exact fixed-point scales and the tiles'
// shared-memory size are set for the whole batch.
#include <algorithm>
#include "dkt_internal.cuh"

namespace dkt {

bool q1fx_setup(Plan &pl, cudaStream_t s);
void tile_pad(Plan &pl, cudaStream_t s);
bool q2sf_setup(Plan &pl, cudaStream_t s);

__global__ void k_offset_ids(const int32_t *__restrict__ in, int32_t *__restrict__ out, int64_t n, int32_t base)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { const int32_t v = in[i]; out[i] = v >= 0 ? v + base : v; }
}
__global__ void k_offset_u32(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, int64_t n, uint32_t base,
                             uint32_t keep_mask)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { const uint32_t v = in[i]; out[i] = (v & keep_mask) | ((v & ~keep_mask) + base); }
}
__global__ void k_offset_i64(const int64_t *__restrict__ in, int64_t *__restrict__ out, int64_t n, int64_t base)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i] + base;
}

template <typename T>
static void copy_to(T *dst, const T *src, size_t n, cudaStream_t s)
{
  if (n) DKT_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
}

void batch_combine(const std::vector<const Plan *> &in, Plan &out, cudaStream_t s)
{
  if (in.empty()) throw std::invalid_argument("empty batch");
  const Plan &a = *in[0];
  int64_t nn = 0, nl = 0, nh = 0, nb = 0, nt = 0, su = 0;
  uint32_t umax = 0;
  for (const Plan *p : in) {
    if (p->dim != a.dim || p->order != a.order || p->md != a.md || p->op.kind != a.op.kind ||
        p->conforming != a.conforming)
      throw std::invalid_argument("plans of a batch must share dim, order, max_depth, operator and traversal");
    if (a.op.kind == OP_CUSTOM) throw std::invalid_argument("custom operators cannot be batched");
    if (p->st_ready && p->st_n_runs > 0) throw std::invalid_argument("plans with stale parent reads cannot be batched");
    if (p->tl_ready != a.tl_ready || p->tl_T != a.tl_T) throw std::invalid_argument("plans of a batch must share tiling");
    nn += p->n_nodes; nl += p->n_leaf; nh += p->n_hang; nb += p->n_bdry;
    nt += p->tl_n; su += p->tl_sum_u; umax = std::max(umax, p->tl_umax);
  }
  if (nn >= (int64_t) 0x7FFFFFFF || nh >= (int64_t) 0x7FFFFFFF) throw std::invalid_argument("batch too large");
  const int npe = a.npe;
  out.dim = a.dim; out.order = a.order; out.md = a.md; out.npe = npe; out.conforming = a.conforming;
  out.n_nodes = nn; out.n_leaf = nl; out.n_hang = nh; out.n_bdry = nb;
  out.e2n.alloc((size_t) nl * npe);
  out.info.alloc(std::max<int64_t>(nl, 1));
  out.hidx.alloc(std::max<int64_t>(nl, 1));
  out.p2n.alloc((size_t) std::max<int64_t>(nh, 1) * npe);
  out.fill.alloc((size_t) std::max<int64_t>(nh, 1) * 3);
  out.bdry.alloc(std::max<int64_t>(nb, 1));
  out.op = a.op;
  out.opA.upload(out.op.A.data(), out.op.A.size(), s);
  out.opB.upload(out.op.B.data(), out.op.B.size(), s);
  out.opAlpha.upload(out.op.alpha.data(), out.op.alpha.size(), s);
  out.opBeta.upload(out.op.beta.data(), out.op.beta.size(), s);
  if (a.ip.n) { out.ip.alloc(a.ip.n); copy_to(out.ip.p, a.ip.p, a.ip.n, s); }
  if (a.tl_ready) {
    out.tl_off.alloc(nt + 1);
    out.tl_lstart.alloc(nt + 1);
    out.tl_hb.alloc(nt + 1);
    out.tl_fm.alloc(std::max<int64_t>(nh, 1));
    out.tl_nodes.alloc(std::max<int64_t>(su, 1));
    out.tl_tau.alloc(std::max<int64_t>(nt, 1));
    out.tl_e2l.alloc((size_t) nl * npe);
    out.tl_p2l.alloc((size_t) std::max<int64_t>(nh, 1) * npe);
  }
  out.seg.assign(1, 0);
  out.lseg.assign(1, 0);
  std::vector<int32_t> mlo;
  int64_t bn = 0, bl = 0, bh = 0, bb = 0, bt = 0, bu = 0;
  for (const Plan *p : in) {
    const size_t ne = (size_t) p->n_leaf * npe, np_ = (size_t) p->n_hang * npe;
    if (ne) k_offset_ids<<<grid_for(ne), 256, 0, s>>>(p->e2n.p, out.e2n.p + bl * npe, ne, (int32_t) bn);
    copy_to(out.info.p + bl, p->info.p, p->n_leaf, s);
    if (p->n_leaf) k_offset_ids<<<grid_for(p->n_leaf), 256, 0, s>>>(p->hidx.p, out.hidx.p + bl, p->n_leaf, (int32_t) bh);
    if (np_) k_offset_ids<<<grid_for(np_), 256, 0, s>>>(p->p2n.p, out.p2n.p + bh * npe, np_, (int32_t) bn);
    copy_to(out.fill.p + bh * 3, p->fill.p, (size_t) p->n_hang * 3, s);
    if (p->n_bdry)
      k_offset_u32<<<grid_for(p->n_bdry), 256, 0, s>>>(p->bdry.p, out.bdry.p + bb, p->n_bdry, (uint32_t) bn, 0u);
    if (a.tl_ready) {
      k_offset_i64<<<grid_for(p->tl_n + 1), 256, 0, s>>>(p->tl_off.p, out.tl_off.p + bt, p->tl_n + 1, bu);
      k_offset_i64<<<grid_for(p->tl_n + 1), 256, 0, s>>>(p->tl_lstart.p, out.tl_lstart.p + bt, p->tl_n + 1, bl);
      k_offset_i64<<<grid_for(p->tl_n), 256, 0, s>>>(p->tl_hb.p, out.tl_hb.p + bt, p->tl_n, bh);
      copy_to(out.tl_fm.p + bh, p->tl_fm.p, (size_t) p->n_hang, s);
      if (p->tl_sum_u)
        k_offset_u32<<<grid_for(p->tl_sum_u), 256, 0, s>>>(p->tl_nodes.p, out.tl_nodes.p + bu, p->tl_sum_u,
                                                            (uint32_t) bn, 0xF8000000u);   // keep level + flag bits
      copy_to(out.tl_tau.p + bt, p->tl_tau.p, (size_t) p->tl_n, s);
      copy_to(out.tl_e2l.p + bl * npe, p->tl_e2l.p, ne, s);
      copy_to(out.tl_p2l.p + bh * npe, p->tl_p2l.p, np_, s);
    }
    check_launch("batch_combine");
    for (int64_t t = 0; t < p->tl_n; t++) mlo.push_back((int32_t) out.seg.size() - 1);
    bn += p->n_nodes; bl += p->n_leaf; bh += p->n_hang; bb += p->n_bdry; bt += p->tl_n; bu += p->tl_sum_u;
    out.seg.push_back(bn);
    out.lseg.push_back(bl);
  }
  if (a.tl_ready) {
    out.tl_T = a.tl_T; out.tl_n = nt; out.tl_sum_u = su; out.tl_umax = umax;
    out.tl_ls_direct = false;
    tile_pad(out, s);
    if (mlo.empty()) mlo.push_back(0);
    out.tl_mlo.upload(mlo.data(), mlo.size(), s);
    out.tl_mhi.upload(mlo.data(), mlo.size(), s);   // tiles of one plan never straddle meshes
  }
  DKT_CUDA(cudaStreamSynchronize(s));
  q1fx_setup(out, s);
  q2sf_setup(out, s);
  out.tl_ready = a.tl_ready;
}

}  // namespace dkt
