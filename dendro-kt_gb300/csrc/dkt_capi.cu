// C ABI (include/dkt_gb300.h): argument checking, error codes, object
// lifetimes, host<->device movement.  All compute runs in the kernels of
// dkt_da.cu, dkt_plan.cu and dkt_matvec.cu.
#include <algorithm>
#include <climits>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "dkt_internal.cuh"
#include "../../include/dkt_gb300.h"
#include "../../include/dkt_gb300_mesh.h"
#include "dkt_host.h"

namespace dkt {
void sort_tree(DA &da, cudaStream_t s);
void build_da_nodes(DA &da, cudaStream_t s);
void boundary_ids(const uint32_t *nx, int64_t n, int dim, int md, DBuf<uint32_t> &out, int64_t &nb, cudaStream_t s);
void build_plan(Plan &pl, const uint32_t *node_x, const uint8_t *node_lev, int64_t n_nodes, const CurveHost &cv,
                const double *ip_host, cudaStream_t s);
void matvec(Plan &pl, const double *x, double *y, double scale, cudaStream_t s);
void fematrix_matvec(Plan &pl, const double *x, double *y, double scale, cudaStream_t s);
void diagonal(const Plan &pl, double *diag, cudaStream_t s);
bool q1fx_setup(Plan &pl, cudaStream_t s);
bool q2sf_setup(Plan &pl, cudaStream_t s);
void tile_setup(Plan &pl, int T, cudaStream_t s);
bool tile_size_supported(int dim, int T);
// 4D: tiles of 128 leaves (level-8 moving ball, product 3.44 ms against 3.58 ms
// with 256; level 7 equal); 2D/3D: 256
inline int default_tile(int dim) { return dim == 4 ? 128 : 256; }
void sphere_shell_device(int dim, int md, int level, double R, double w, const double *c, DBuf<uint64_t> &out,
                         int64_t &n_out, cudaStream_t s);
void tree_from_points_device(const uint32_t *pts_host, int64_t n, int dim, int md, int64_t max_pts,
                             DBuf<uint64_t> &out, int64_t &n_out, cudaStream_t s);
void function2octree_device(FieldFn fn, void *user, int n_vars, int dim, int md, int p, double tol, bool balance,
                            DBuf<uint64_t> &out, int64_t &n_out, cudaStream_t s);
void moving_ball_device(int md, int level, double R, double w, const double *c0, const double *c1,
                        DBuf<uint64_t> &out, int64_t &n_out, cudaStream_t s);
void unpack_cells_to_host(const DBuf<uint64_t> &keys, int64_t n, int dim, int md, uint32_t *coords, uint8_t *levels,
                          cudaStream_t s);
void stale_setup(Plan &pl, const std::vector<double> &ip, cudaStream_t s);
int fematrix_matvec_noalloc(const Plan &pl, const double *x, double *y, double scale, cudaStream_t s,
                            std::string &err);
int pcg_solve(Plan &pl, const double *b, double *x, int precision, int max_iter, double tol, bool jacobi,
              int *iters, int *refinements, double *relres, cudaStream_t user);
void q1f32_apply(Plan &pl, const float *x, float *y, bool bc_in, bool bc_out, cudaStream_t s);
void batch_combine(const std::vector<const Plan *> &in, Plan &out, cudaStream_t s);
void fematrix_matvec(Plan &pl, const double *x, double *y, double scale, cudaStream_t s);
int cg_solve(Plan &pl, const double *b, double *x, int max_iter, double tol, bool jacobi, bool linf, int *iters,
             double *relres, cudaStream_t s);

}  // namespace dkt

#include "dkt_handles.cuh"

namespace {
thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
  g_err = msg;
  return code;
}

template <typename F>
int guarded(F &&f)
{
  try {
    return f();
  } catch (const std::bad_alloc &e) {
    return fail(DKT_E_NOMEM, std::string("host allocation failed: ") + e.what());
  } catch (const std::invalid_argument &e) {
    return fail(DKT_E_ARG, e.what());
  } catch (const std::runtime_error &e) {
    const std::string m = e.what();
    if (m.find("out of memory") != std::string::npos) return fail(DKT_E_NOMEM, m);
    if (m.find("CUDA") != std::string::npos || m.find("launch") != std::string::npos) return fail(DKT_E_CUDA, m);
    return fail(DKT_E_INTERNAL, m);
  } catch (...) {
    return fail(DKT_E_INTERNAL, "unknown exception");
  }
}

int check_cfg(int dim, int order, int curve, int md)
{
  if (dim < 2 || dim > 4) return fail(DKT_E_ARG, "dim must be 2, 3 or 4");
  if (order < 1 || order > 2) return fail(DKT_E_UNSUP, "element order must be 1 or 2");
  if (curve != DKT_CURVE_MORTON && curve != DKT_CURVE_HILBERT) return fail(DKT_E_ARG, "unknown curve");
  if (md < 1 || md > 30) return fail(DKT_E_ARG, "max_depth out of range");
  if (dim * md + 6 > 64) return fail(DKT_E_UNSUP, "dim * max_depth too large (cell keys are 64-bit)");
  return DKT_OK;
}

void set_curve(dkt::CurveHost &cv, int curve, int dim)
{
  if (curve == DKT_CURVE_HILBERT) {
    dkt::hilbert_tables(dim, cv.rot, cv.ht, cv.nrot);
  } else {
    cv.morton(dim);
  }
}

void setup_operator(dkt::Plan &pl, int op, const double *tables, cudaStream_t s)
{
  if (op < 0 || op > 6) throw std::invalid_argument("unknown operator");
  pl.op.kind = op;
  pl.op.npe = pl.npe;
  pl.op.nlev = pl.md + 1;
  if (op == DKT_OP_CUSTOM) {
    if (!tables) throw std::invalid_argument("custom operator needs tables");
    const size_t n = (size_t) (pl.md + 1) * pl.npe * pl.npe;
    pl.op.table.assign(tables, tables + n);
    pl.op.uses_scale = true;
    pl.opTable.upload(pl.op.table.data(), n, s);
    return;
  }
  dkt::builtin_operator(op, pl.dim, pl.order, pl.md, pl.op.A, pl.op.B, pl.op.alpha, pl.op.beta, pl.op.uses_scale);
  pl.opA.upload(pl.op.A.data(), pl.op.A.size(), s);
  pl.opB.upload(pl.op.B.data(), pl.op.B.size(), s);
  pl.opAlpha.upload(pl.op.alpha.data(), pl.op.alpha.size(), s);
  pl.opBeta.upload(pl.op.beta.data(), pl.op.beta.size(), s);
}

// out[i] = in[i] >= 0 ? map[in[i]] : -1; a referenced node the map leaves
// out (-1) raises *bad
__global__ void k_remap_ids(const int32_t *__restrict__ in, int32_t *__restrict__ out, int64_t n,
                            const int32_t *__restrict__ map, int *__restrict__ bad)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t v = in[i];
  int32_t r = -1;
  if (v >= 0) {
    r = map[v];
    if (r < 0) atomicExch(bad, 1);
  }
  out[i] = r;
}
// rows[k] of in (width w) to row k of out, node ids through map when given
template <typename T>
__global__ void k_gather_rows(const T *__restrict__ in, T *__restrict__ out, const int32_t *__restrict__ rows,
                              int64_t n_rows, int w, const int32_t *__restrict__ map, int *__restrict__ bad)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_rows * w) return;
  T v = in[(int64_t) rows[i / w] * w + i % w];
  if (map) {
    const int32_t id = (int32_t) v;
    int32_t r = -1;
    if (id >= 0) {
      r = map[id];
      if (r < 0) atomicExch(bad, 1);
    }
    v = (T) r;
  }
  out[i] = v;
}

std::vector<double> interp_tables(int p)
{
  const dkt::RefEl1D re = dkt::refel_1d(p);
  std::vector<double> ip(re.ip0);
  ip.insert(ip.end(), re.ip1.begin(), re.ip1.end());
  return ip;
}
}  // namespace

extern "C" {

const char *dkt_last_error(void) { return g_err.c_str(); }

int dkt_da_create(int dim, int order, int curve, int max_depth, const uint32_t *tree_coords,
                  const uint8_t *tree_levels, int64_t n_elem, int tree_is_sorted, dkt_da *out)
{
  if (!out || !tree_coords || !tree_levels || n_elem <= 0) return fail(DKT_E_ARG, "null or empty tree");
  if (int rc = check_cfg(dim, order, curve, max_depth)) return rc;
  return guarded([&]() {
    for (int64_t i = 0; i < n_elem; i++) {
      if ((int) tree_levels[i] > max_depth) throw std::invalid_argument("element level exceeds max_depth");
      const uint32_t len = 1u << (max_depth - tree_levels[i]);
      for (int d = 0; d < dim; d++) {
        const uint32_t x = tree_coords[i * dim + d];
        if (x >= (1u << max_depth) || (x & (len - 1u))) throw std::invalid_argument("element anchor not aligned or outside the domain");
      }
    }
    dkt_da_s *h = new dkt_da_s();
    dkt::DA &da = h->da;
    da.dim = dim; da.order = order; da.md = max_depth; da.curve = curve; da.n_elem = n_elem;
    set_curve(da.cv, curve, dim);
    da.cv.upload();
    cudaStream_t s = 0;
    try {
      da.elem_x.upload(tree_coords, (size_t) n_elem * dim, s);
      da.elem_lev.upload(tree_levels, (size_t) n_elem, s);
      if (!tree_is_sorted) dkt::sort_tree(da, s);
      dkt::build_da_nodes(da, s);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
    return DKT_OK;
  });
}

int64_t dkt_da_local_nodal_size(dkt_da da) { return da ? da->da.n_nodes : -1; }
int64_t dkt_da_num_elements(dkt_da da) { return da ? da->da.n_elem : -1; }
int64_t dkt_da_boundary_size(dkt_da da) { return da ? da->da.n_bdry : -1; }

int dkt_da_get_nodes(dkt_da da, uint32_t *coords, uint8_t *levels)
{
  if (!da || !coords || !levels) return fail(DKT_E_ARG, "null argument");
  return guarded([&]() {
    const dkt::DA &d = da->da;
    DKT_CUDA(cudaMemcpy(coords, d.node_x.p, (size_t) d.n_nodes * d.dim * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    DKT_CUDA(cudaMemcpy(levels, d.node_lev.p, (size_t) d.n_nodes, cudaMemcpyDeviceToHost));
    return DKT_OK;
  });
}

int dkt_da_get_boundary_ids(dkt_da da, uint32_t *ids)
{
  if (!da || (!ids && da->da.n_bdry > 0)) return fail(DKT_E_ARG, "null argument");
  return guarded([&]() {
    if (da->da.n_bdry > 0)
      DKT_CUDA(cudaMemcpy(ids, da->da.bdry.p, (size_t) da->da.n_bdry * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return DKT_OK;
  });
}

int dkt_da_get_tree(dkt_da da, uint32_t *coords, uint8_t *levels)
{
  if (!da || !coords || !levels) return fail(DKT_E_ARG, "null argument");
  return guarded([&]() {
    const dkt::DA &d = da->da;
    DKT_CUDA(cudaMemcpy(coords, d.elem_x.p, (size_t) d.n_elem * d.dim * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    DKT_CUDA(cudaMemcpy(levels, d.elem_lev.p, (size_t) d.n_elem, cudaMemcpyDeviceToHost));
    return DKT_OK;
  });
}

int dkt_da_set_vector_by_function(dkt_da da, dkt_field_fn fn, void *user, int dof, double *out)
{
  if (!da || !fn || !out || dof < 1) return fail(DKT_E_ARG, "bad argument");
  return guarded([&]() {
    const dkt::DA &d = da->da;
    const int64_t n = d.n_nodes;
    const int edim = d.dim < 3 ? d.dim : 3;
    std::vector<uint32_t> nx((size_t) n * d.dim);
    if (n) DKT_CUDA(cudaMemcpy(nx.data(), d.node_x.p, (size_t) n * d.dim * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    const double scale = 1.0 / (double) (1u << d.md);
    const int64_t batch = int64_t(1) << 20;
    std::vector<double> pts;
    for (int64_t b0 = 0; b0 < n; b0 += batch) {
      const int64_t nb = std::min(batch, n - b0);
      pts.resize((size_t) nb * edim);
      for (int64_t k = 0; k < nb; k++)
        for (int a = 0; a < edim; a++) pts[k * edim + a] = scale * (double) nx[(b0 + k) * d.dim + a];
      if (fn(pts.data(), nb, edim, out + b0 * dof, dof, user) != 0)
        throw std::runtime_error("setVectorByFunction: the field callback reported an error");
    }
    return DKT_OK;
  });
}

void dkt_da_destroy(dkt_da da) { delete da; }

static int plan_common(int dim, int order, int curve, int md, const uint32_t *node_x_dev, const uint8_t *node_lev_dev,
                       int64_t n, const uint32_t *bdry_dev, int64_t nb, int op, const double *tables, dkt_plan *out,
                       int traversal = DKT_TRAVERSAL_REFERENCE)
{
  dkt_plan_s *h = new dkt_plan_s();
  try {
    dkt::Plan &pl = h->pl;
    pl.dim = dim; pl.order = order; pl.md = md;
    pl.conforming = (traversal == DKT_TRAVERSAL_CONFORMING);
    cudaStream_t s = 0;
    dkt::CurveHost cv;
    set_curve(cv, curve, dim);
    cv.upload();
    const std::vector<double> ip = interp_tables(order);
    dkt::build_plan(pl, node_x_dev, node_lev_dev, n, cv, ip.data(), s);
    setup_operator(pl, op, tables, s);
    dkt::stale_setup(pl, ip, s);
    if (dkt::q1fx_setup(pl, s)) dkt::tile_setup(pl, dkt::default_tile(dim), s);
    dkt::q2sf_setup(pl, s);
    if (bdry_dev) {
      pl.bdry.alloc(nb > 0 ? nb : 1);
      if (nb > 0) DKT_CUDA(cudaMemcpyAsync(pl.bdry.p, bdry_dev, nb * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
      pl.n_bdry = nb;
    } else {
      dkt::boundary_ids(node_x_dev, n, dim, md, pl.bdry, pl.n_bdry, s);
    }
    DKT_CUDA(cudaStreamSynchronize(s));
  } catch (...) {
    delete h;
    throw;
  }
  *out = h;
  return DKT_OK;
}

int dkt_plan_create(dkt_da da, int op, const double *op_tables, dkt_plan *out)
{
  if (!da || !out) return fail(DKT_E_ARG, "null argument");
  return guarded([&]() {
    const dkt::DA &d = da->da;
    return plan_common(d.dim, d.order, d.curve, d.md, d.node_x.p, d.node_lev.p, d.n_nodes, d.bdry.p, d.n_bdry, op,
                       op_tables, out);
  });
}

int dkt_plan_create_ex(dkt_da da, int op, const double *op_tables, int traversal, dkt_plan *out)
{
  if (!da || !out) return fail(DKT_E_ARG, "null argument");
  if (traversal != DKT_TRAVERSAL_REFERENCE && traversal != DKT_TRAVERSAL_CONFORMING) return fail(DKT_E_ARG, "bad traversal");
  return guarded([&]() {
    const dkt::DA &d = da->da;
    return plan_common(d.dim, d.order, d.curve, d.md, d.node_x.p, d.node_lev.p, d.n_nodes, d.bdry.p, d.n_bdry, op,
                       op_tables, out, traversal);
  });
}

int dkt_plan_create_from_nodes(int dim, int order, int curve, int max_depth, const uint32_t *node_coords,
                               const uint8_t *node_levels, int64_t sz, int op, const double *op_tables,
                               dkt_plan *out)
{
  if (!out || !node_coords || !node_levels || sz <= 0) return fail(DKT_E_ARG, "null or empty node list");
  if (int rc = check_cfg(dim, order, curve, max_depth)) return rc;
  return guarded([&]() {
    for (int64_t i = 0; i < sz; i++) {
      if ((int) node_levels[i] > max_depth) throw std::invalid_argument("node level exceeds max_depth");
      for (int d = 0; d < dim; d++)
        if (node_coords[i * dim + d] > (1u << max_depth)) throw std::invalid_argument("node outside the domain");
    }
    dkt::DBuf<uint32_t> nx;
    dkt::DBuf<uint8_t> nl;
    nx.upload(node_coords, (size_t) sz * dim);
    nl.upload(node_levels, (size_t) sz);
    return plan_common(dim, order, curve, max_depth, nx.p, nl.p, sz, nullptr, 0, op, op_tables, out);
  });
}

int dkt_plan_create_part(dkt_plan full, int64_t leaf_begin, int64_t leaf_end, const int32_t *node_map,
                         int64_t n_local, dkt_plan *out)
{
  if (!full || !node_map || !out || n_local <= 0) return fail(DKT_E_ARG, "null argument or empty part");
  const dkt::Plan &f = full->pl;
  if (leaf_begin < 0 || leaf_end <= leaf_begin || leaf_end > f.n_leaf) return fail(DKT_E_ARG, "bad leaf range");
  if (f.seg.size() >= 2) return fail(DKT_E_UNSUP, "a batch plan is not partitioned");
  if (f.st_ready && f.st_n_runs > 0)
    return fail(DKT_E_UNSUP, "a plan that reads stale parent-buffer slots is not partitioned (the buffer is one "
                             "sequential chain over the whole traversal)");
  dkt_plan_s *h = new dkt_plan_s();
  const int rc = guarded([&]() {
    dkt::Plan &pl = h->pl;
    cudaStream_t s = 0;
    const int64_t nl = leaf_end - leaf_begin, npe = f.npe;
    // the part's hanging records, in the order of its leaves
    std::vector<int32_t> hid((size_t) nl), hrows;
    DKT_CUDA(cudaMemcpy(hid.data(), f.hidx.p + leaf_begin, nl * sizeof(int32_t), cudaMemcpyDeviceToHost));
    for (int32_t &v : hid)
      if (v >= 0) {
        hrows.push_back(v);
        v = (int32_t) hrows.size() - 1;
      }
    const int64_t nh = (int64_t) hrows.size();
    pl.dim = f.dim; pl.order = f.order; pl.md = f.md; pl.npe = f.npe; pl.conforming = f.conforming;
    pl.n_nodes = n_local; pl.n_leaf = nl; pl.n_hang = nh; pl.n_bdry = 0;
    pl.op = f.op;
    pl.arith = f.arith;
    if (f.opA.n) { pl.opA.alloc(f.opA.n); DKT_CUDA(cudaMemcpy(pl.opA.p, f.opA.p, f.opA.n * sizeof(double), cudaMemcpyDeviceToDevice)); }
    if (f.opB.n) { pl.opB.alloc(f.opB.n); DKT_CUDA(cudaMemcpy(pl.opB.p, f.opB.p, f.opB.n * sizeof(double), cudaMemcpyDeviceToDevice)); }
    if (f.opAlpha.n) { pl.opAlpha.alloc(f.opAlpha.n); DKT_CUDA(cudaMemcpy(pl.opAlpha.p, f.opAlpha.p, f.opAlpha.n * sizeof(double), cudaMemcpyDeviceToDevice)); }
    if (f.opBeta.n) { pl.opBeta.alloc(f.opBeta.n); DKT_CUDA(cudaMemcpy(pl.opBeta.p, f.opBeta.p, f.opBeta.n * sizeof(double), cudaMemcpyDeviceToDevice)); }
    if (f.opTable.n) { pl.opTable.alloc(f.opTable.n); DKT_CUDA(cudaMemcpy(pl.opTable.p, f.opTable.p, f.opTable.n * sizeof(double), cudaMemcpyDeviceToDevice)); }
    if (f.ip.n) { pl.ip.alloc(f.ip.n); DKT_CUDA(cudaMemcpy(pl.ip.p, f.ip.p, f.ip.n * sizeof(double), cudaMemcpyDeviceToDevice)); }
    dkt::DBuf<int32_t> map;
    map.upload(node_map, (size_t) f.n_nodes, s);
    dkt::DBuf<int> bad(1);
    DKT_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
    pl.e2n.alloc((size_t) nl * npe);
    k_remap_ids<<<dkt::grid_for(nl * npe), 256, 0, s>>>(f.e2n.p + leaf_begin * npe, pl.e2n.p, nl * npe, map.p, bad.p);
    pl.info.alloc(nl);
    DKT_CUDA(cudaMemcpyAsync(pl.info.p, f.info.p + leaf_begin, nl * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    pl.hidx.upload(hid.data(), hid.size(), s);
    pl.p2n.alloc((size_t) std::max<int64_t>(nh, 1) * npe);
    pl.fill.alloc((size_t) std::max<int64_t>(nh, 1) * 3);
    dkt::DBuf<int32_t> rows;
    if (nh) {
      rows.upload(hrows.data(), hrows.size(), s);
      k_gather_rows<int32_t><<<dkt::grid_for(nh * npe), 256, 0, s>>>(f.p2n.p, pl.p2n.p, rows.p, nh, (int) npe,
                                                                     map.p, bad.p);
      k_gather_rows<uint32_t><<<dkt::grid_for(nh * 3), 256, 0, s>>>(f.fill.p, pl.fill.p, rows.p, nh, 3, nullptr,
                                                                    bad.p);
    }
    dkt::check_launch("part_remap");
    pl.bdry.alloc(1);
    int hbad = 0;
    DKT_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    DKT_CUDA(cudaStreamSynchronize(s));
    if (hbad) throw std::invalid_argument("node_map leaves out a node that the part's leaves touch");
    if (dkt::q1fx_setup(pl, s)) dkt::tile_setup(pl, f.tl_ready ? f.tl_T : dkt::default_tile(pl.dim), s);
    dkt::q2sf_setup(pl, s);
    DKT_CUDA(cudaStreamSynchronize(s));
    return DKT_OK;
  });
  if (rc != DKT_OK) { delete h; return rc; }
  *out = h;
  return DKT_OK;
}

int64_t dkt_plan_num_nodes(dkt_plan plan) { return plan ? plan->pl.n_nodes : -1; }

int dkt_plan_stats(dkt_plan plan, int64_t *out4)
{
  if (!plan || !out4) return fail(DKT_E_ARG, "null argument");
  out4[0] = plan->pl.n_leaf;
  out4[1] = plan->pl.n_hang;
  out4[2] = plan->pl.stale_slots;
  out4[3] = plan->pl.n_bdry;
  return DKT_OK;
}

int dkt_plan_stats_ex(dkt_plan plan, int64_t *out, int n)
{
  if (!plan || !out || n < 0) return fail(DKT_E_ARG, "bad argument");
  const dkt::Plan &pl = plan->pl;
  const int64_t v[9] = {pl.n_leaf, pl.n_hang, pl.stale_slots, pl.n_bdry,
                        pl.st_ready ? pl.st_n_ent : 0, pl.st_ready ? pl.st_n_runs : 0,
                        pl.st_max_run_groups, pl.st_max_run_ents, pl.fallbacks};
  for (int k = 0; k < n && k < 9; k++) out[k] = v[k];
  return DKT_OK;
}

int dkt_plan_export(dkt_plan plan, int32_t *e2n, uint32_t *info, int32_t *hidx, int32_t *p2n, uint32_t *fill)
{
  if (!plan) return fail(DKT_E_ARG, "null argument");
  return guarded([&]() {
    const dkt::Plan &pl = plan->pl;
    const size_t nl = (size_t) pl.n_leaf, nh = (size_t) pl.n_hang, npe = (size_t) pl.npe;
    if (e2n) DKT_CUDA(cudaMemcpy(e2n, pl.e2n.p, npe * nl * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (info) DKT_CUDA(cudaMemcpy(info, pl.info.p, nl * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (hidx) DKT_CUDA(cudaMemcpy(hidx, pl.hidx.p, nl * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (p2n && nh) DKT_CUDA(cudaMemcpy(p2n, pl.p2n.p, npe * nh * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (fill && nh) DKT_CUDA(cudaMemcpy(fill, pl.fill.p, 3 * nh * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return DKT_OK;
  });
}

int dkt_matvec(dkt_plan plan, const double *x_dev, double *y_dev, double scale, void *stream)
{
  if (!plan || !x_dev || !y_dev) return fail(DKT_E_ARG, "null argument");
  return guarded([&]() {
    dkt::matvec(plan->pl, x_dev, y_dev, scale, (cudaStream_t) stream);
    return DKT_OK;
  });
}

int dkt_fematrix_matvec(dkt_plan plan, const double *x_dev, double *y_dev, double scale, void *stream)
{
  if (!plan || !x_dev || !y_dev) return fail(DKT_E_ARG, "null argument");
  return guarded([&]() {
    dkt::fematrix_matvec(plan->pl, x_dev, y_dev, scale, (cudaStream_t) stream);
    return DKT_OK;
  });
}

int dkt_fevector_compute_vec(dkt_plan plan, const double *in_dev, double *out_dev, double scale, void *stream)
{
  if (!plan || !in_dev || !out_dev) return fail(DKT_E_ARG, "null argument");
  const int k = plan->pl.op.kind;
  if (k != dkt::OP_HEATVEC && k != dkt::OP_MASS && k != dkt::OP_CUSTOM)
    return fail(DKT_E_ARG, "plan operator is not a vector (right-hand side) operator");
  return guarded([&]() {
    dkt::fematrix_matvec(plan->pl, in_dev, out_dev, scale, (cudaStream_t) stream);
    return DKT_OK;
  });
}

int dkt_fematrix_matvec_noalloc(dkt_plan plan, const double *x_dev, double *y_dev, double scale, void *stream)
{
  if (!plan || !x_dev || !y_dev) return fail(DKT_E_ARG, "null argument");
  try {
    std::string err;
    const int st = dkt::fematrix_matvec_noalloc(plan->pl, x_dev, y_dev, scale, (cudaStream_t) stream, err);
    if (st == dkt::NOALLOC_TOO_LARGE) return fail(DKT_E_ARG, err);
    if (st != dkt::NOALLOC_OK) return fail(DKT_E_CUDA, err);
  } catch (const std::exception &e) {
    return fail(DKT_E_CUDA, e.what());
  }
  return DKT_OK;
}

int dkt_fematrix_matvec_host(dkt_plan plan, const double *x_host, double *y_host, double scale)
{
  if (!plan || !x_host || !y_host) return fail(DKT_E_ARG, "null argument");
  return guarded([&]() {
    dkt::Plan &pl = plan->pl;
    const int64_t n = pl.n_nodes;
    if (pl.xh.n < (size_t) n) pl.xh.alloc(n);
    if (pl.yh.n < (size_t) n) pl.yh.alloc(n);
    DKT_CUDA(cudaMemcpyAsync(pl.xh.p, x_host, n * sizeof(double), cudaMemcpyHostToDevice, 0));
    dkt::fematrix_matvec(pl, pl.xh.p, pl.yh.p, scale, 0);
    DKT_CUDA(cudaMemcpyAsync(y_host, pl.yh.p, n * sizeof(double), cudaMemcpyDeviceToHost, 0));
    DKT_CUDA(cudaStreamSynchronize(0));
    return DKT_OK;
  });
}

int dkt_fematrix_matvec_host_many(dkt_plan plan, const double *const *x_host, double *const *y_host, int count,
                                  double scale)
{
  if (!plan || count < 0 || (count > 0 && (!x_host || !y_host))) return fail(DKT_E_ARG, "bad argument");
  for (int k = 0; k < count; k++)
    if (!x_host[k] || !y_host[k]) return fail(DKT_E_ARG, "null vector");
  return guarded([&]() {
    dkt::Plan &pl = plan->pl;
    const int64_t n = pl.n_nodes;
    const size_t bytes = (size_t) n * sizeof(double);
    dkt::DBuf<double> din[2], dout[2];
    for (int b = 0; b < 2; b++) { din[b].alloc(n); dout[b].alloc(n); }
    cudaStream_t sc = 0, si = nullptr, so = nullptr;   // compute: the caller thread's default stream
    cudaEvent_t in_ready[2], in_free[2], out_ready[2], out_free[2];
    DKT_CUDA(cudaStreamCreateWithFlags(&si, cudaStreamNonBlocking));
    DKT_CUDA(cudaStreamCreateWithFlags(&so, cudaStreamNonBlocking));
    for (int b = 0; b < 2; b++) {
      DKT_CUDA(cudaEventCreateWithFlags(&in_ready[b], cudaEventDisableTiming));
      DKT_CUDA(cudaEventCreateWithFlags(&in_free[b], cudaEventDisableTiming));
      DKT_CUDA(cudaEventCreateWithFlags(&out_ready[b], cudaEventDisableTiming));
      DKT_CUDA(cudaEventCreateWithFlags(&out_free[b], cudaEventDisableTiming));
    }
    auto cleanup = [&]() {
      cudaStreamSynchronize(si);
      cudaStreamSynchronize(so);
      cudaStreamSynchronize(sc);
      for (int b = 0; b < 2; b++) {
        cudaEventDestroy(in_ready[b]); cudaEventDestroy(in_free[b]);
        cudaEventDestroy(out_ready[b]); cudaEventDestroy(out_free[b]);
      }
      cudaStreamDestroy(si);
      cudaStreamDestroy(so);
    };
    try {
      // buffer b serves products b, b + 2, ...: its copy-in waits until the
      // product two steps back has read it, its copy-out until the product wrote it
      for (int k = 0; k < count; k++) {
        const int b = k & 1;
        if (k >= 2) DKT_CUDA(cudaStreamWaitEvent(si, in_free[b], 0));
        DKT_CUDA(cudaMemcpyAsync(din[b].p, x_host[k], bytes, cudaMemcpyHostToDevice, si));
        DKT_CUDA(cudaEventRecord(in_ready[b], si));
        DKT_CUDA(cudaStreamWaitEvent(sc, in_ready[b], 0));
        if (k >= 2) DKT_CUDA(cudaStreamWaitEvent(sc, out_free[b], 0));
        dkt::fematrix_matvec(pl, din[b].p, dout[b].p, scale, sc);
        DKT_CUDA(cudaEventRecord(in_free[b], sc));
        DKT_CUDA(cudaEventRecord(out_ready[b], sc));
        DKT_CUDA(cudaStreamWaitEvent(so, out_ready[b], 0));
        DKT_CUDA(cudaMemcpyAsync(y_host[k], dout[b].p, bytes, cudaMemcpyDeviceToHost, so));
        DKT_CUDA(cudaEventRecord(out_free[b], so));
      }
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
    DKT_CUDA(cudaGetLastError());
    return DKT_OK;
  });
}

int dkt_diagonal(dkt_plan plan, double *diag_dev, void *stream)
{
  if (!plan || !diag_dev) return fail(DKT_E_ARG, "null argument");
  return guarded([&]() {
    dkt::diagonal(plan->pl, diag_dev, (cudaStream_t) stream);
    return DKT_OK;
  });
}

int dkt_cg_solve(dkt_plan plan, const double *b_dev, double *x_dev, int max_iter, double tol, int flags,
                 int *iters, double *relres, void *stream)
{
  if (!plan || !b_dev || !x_dev || max_iter < 0 || !(tol > 0)) return fail(DKT_E_ARG, "bad argument");
  if (flags & ~(DKT_CG_JACOBI | DKT_CG_REFERENCE)) return fail(DKT_E_ARG, "unknown CG flags");
  return guarded([&]() {
    return dkt::cg_solve(plan->pl, b_dev, x_dev, max_iter, tol, (flags & DKT_CG_JACOBI) != 0,
                         (flags & DKT_CG_REFERENCE) != 0, iters, relres, (cudaStream_t) stream);
  });
}

int dkt_cg_solve_host(dkt_plan plan, const double *b_host, double *x_host, int max_iter, double tol, int flags,
                      int *iters, double *relres)
{
  if (!plan || !b_host || !x_host || max_iter < 0 || !(tol > 0)) return fail(DKT_E_ARG, "bad argument");
  if (flags & ~(DKT_CG_JACOBI | DKT_CG_REFERENCE)) return fail(DKT_E_ARG, "unknown CG flags");
  return guarded([&]() {
    dkt::Plan &pl = plan->pl;
    const int64_t n = pl.n_nodes;
    dkt::DBuf<double> b(n), x(n);
    DKT_CUDA(cudaMemcpyAsync(b.p, b_host, n * sizeof(double), cudaMemcpyHostToDevice, 0));
    DKT_CUDA(cudaMemcpyAsync(x.p, x_host, n * sizeof(double), cudaMemcpyHostToDevice, 0));
    const int rc = dkt::cg_solve(pl, b.p, x.p, max_iter, tol, (flags & DKT_CG_JACOBI) != 0,
                                 (flags & DKT_CG_REFERENCE) != 0, iters, relres, 0);
    DKT_CUDA(cudaMemcpyAsync(x_host, x.p, n * sizeof(double), cudaMemcpyDeviceToHost, 0));
    DKT_CUDA(cudaStreamSynchronize(0));
    return rc;
  });
}

int dkt_batch_create(const dkt_plan *plans, int n, dkt_plan *out)
{
  if (!plans || n <= 0 || !out) return fail(DKT_E_ARG, "bad argument");
  for (int k = 0; k < n; k++)
    if (!plans[k]) return fail(DKT_E_ARG, "null plan");
  dkt_plan_s *h = new dkt_plan_s();
  const int rc = guarded([&]() {
    std::vector<const dkt::Plan *> in;
    for (int k = 0; k < n; k++) in.push_back(&plans[k]->pl);
    dkt::batch_combine(in, h->pl, 0);
    return DKT_OK;
  });
  if (rc != DKT_OK) { delete h; return rc; }
  *out = h;
  return DKT_OK;
}

int dkt_plan_num_meshes(dkt_plan plan, int *n)
{
  if (!plan || !n) return fail(DKT_E_ARG, "null argument");
  *n = plan->pl.seg.size() >= 2 ? (int) plan->pl.seg.size() - 1 : 1;
  return DKT_OK;
}

int dkt_plan_mesh_offsets(dkt_plan plan, int64_t *offsets)
{
  if (!plan || !offsets) return fail(DKT_E_ARG, "null argument");
  if (plan->pl.seg.size() >= 2) std::copy(plan->pl.seg.begin(), plan->pl.seg.end(), offsets);
  else { offsets[0] = 0; offsets[1] = plan->pl.n_nodes; }
  return DKT_OK;
}

namespace {
// x_i = uniform[-1,1) from a counter hash (the autotuner's input: every
// product path, global atomics included, does its real work)
__global__ void k_fill_pm1(double *__restrict__ x, float *__restrict__ x32, int64_t n)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t z = (uint64_t) i * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  const double v = 2.0 * ((double) (z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
  x[i] = v;
  x32[i] = (float) v;
}
}  // namespace

int dkt_plan_autotune_ex(dkt_plan plan, int arith, int *best_tile, int *best_persist, double *best_ms,
                         double *times)
{
  if (!plan || arith < 0 || arith > 1) return fail(DKT_E_ARG, "bad argument");
  if (!plan->pl.fx_ready) return fail(DKT_E_UNSUP, "tiles need a Q1 built-in operator");
  if (arith == 1 && !plan->pl.f32_ready)
    return fail(DKT_E_UNSUP, "binary32 product needs a plan without stale parent reads");
  return guarded([&]() {
    dkt::Plan &pl = plan->pl;
    const int sizes[3] = {pl.dim == 4 ? 64 : 128, pl.dim == 4 ? 128 : 256, pl.dim == 4 ? 256 : 512};
    const int64_t n = pl.n_nodes;
    dkt::DBuf<double> x(n), y(n);
    dkt::DBuf<float> x32(n), y32(n);
    k_fill_pm1<<<dkt::grid_for(n), 256>>>(x.p, x32.p, n);
    dkt::check_launch("autotune_input");
    cudaEvent_t e0, e1;
    DKT_CUDA(cudaEventCreate(&e0));
    DKT_CUDA(cudaEventCreate(&e1));
    const bool saved = pl.timing;
    pl.timing = false;
    auto product = [&]() {
      if (arith == 0) dkt::fematrix_matvec(pl, x.p, y.p, 1.0, 0);
      else dkt::q1f32_apply(pl, x32.p, y32.p, false, true, 0);
    };
    // candidates: the untiled kernel, then per tile size the plain grid and
    // the persistent launch (dims 2 and 3)
    struct Cand { int T; bool persist; };
    std::vector<Cand> cands{{0, false}};
    for (int T : sizes) {
      cands.push_back({T, false});
      cands.push_back({T, true});
    }
    int best = 0;
    double bms = 1e300;
    for (size_t c = 0; c < cands.size(); c++) {
      double ms_c = -1.0;
      if (!(cands[c].persist && pl.dim > 3)) {
        dkt::tile_setup(pl, cands[c].T, 0);
        pl.tl_persist = cands[c].persist;
        product();
        DKT_CUDA(cudaEventRecord(e0, 0));
        for (int k = 0; k < 5; k++) product();
        DKT_CUDA(cudaEventRecord(e1, 0));
        DKT_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        DKT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        ms_c = ms / 5;
        if (ms_c < bms) { bms = ms_c; best = (int) c; }
      }
      if (times) times[c] = ms_c;
    }
    pl.timing = saved;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    dkt::tile_setup(pl, cands[best].T, 0);
    pl.tl_persist = cands[best].persist;
    if (best_tile) *best_tile = cands[best].T;
    if (best_persist) *best_persist = cands[best].persist ? 1 : 0;
    if (best_ms) *best_ms = bms;
    return DKT_OK;
  });
}

int dkt_plan_autotune(dkt_plan plan, int *best_tile, double *best_ms)
{
  return dkt_plan_autotune_ex(plan, 0, best_tile, nullptr, best_ms, nullptr);
}

int dkt_pcg_solve(dkt_plan plan, const double *b_dev, double *x_dev, int precision, int max_iter, double tol,
                  int jacobi, int *iters, int *refinements, double *relres, void *stream)
{
  if (!plan || !b_dev || !x_dev || max_iter < 0 || !(tol > 0) || precision < 0 || precision > 1)
    return fail(DKT_E_ARG, "bad argument");
  if (precision == 1 && !plan->pl.f32_ready)
    return fail(DKT_E_UNSUP, "mixed precision needs a Q1 or Q2 built-in operator without stale parent reads");
  return guarded([&]() {
    return dkt::pcg_solve(plan->pl, b_dev, x_dev, precision, max_iter, tol, jacobi != 0, iters, refinements,
                          relres, (cudaStream_t) stream);
  });
}

int dkt_matvec_f32(dkt_plan plan, const float *x_dev, float *y_dev, void *stream)
{
  if (!plan || !x_dev || !y_dev) return fail(DKT_E_ARG, "null argument");
  if (!plan->pl.f32_ready)
    return fail(DKT_E_UNSUP, "binary32 product needs a Q1 or Q2 built-in operator without stale parent reads");
  return guarded([&]() {
    const bool bc = dkt::op_has_bc(plan->pl.op.kind);
    dkt::q1f32_apply(plan->pl, x_dev, y_dev, bc, bc, (cudaStream_t) stream);
    return DKT_OK;
  });
}

int dkt_plan_set_arithmetic(dkt_plan plan, int mode)
{
  if (!plan || mode < 0 || mode > 2) return fail(DKT_E_ARG, "bad argument");
  if (mode == 2 && !plan->pl.fx_ready) return fail(DKT_E_UNSUP, "fixed-point arithmetic needs a Q1 built-in operator");
  plan->pl.arith = mode;
  return DKT_OK;
}

int dkt_plan_kernel_timing(dkt_plan plan, int enable, double *total_ms, int64_t *launches)
{
  if (!plan) return fail(DKT_E_ARG, "null argument");
  return guarded([&]() {
    dkt::Plan &pl = plan->pl;
    double tot = 0.0;
    for (size_t k = 0; k + 1 < pl.ev.size(); k += 2) {
      DKT_CUDA(cudaEventSynchronize(pl.ev[k + 1]));
      float ms = 0.f;
      DKT_CUDA(cudaEventElapsedTime(&ms, pl.ev[k], pl.ev[k + 1]));
      tot += ms;
    }
    for (cudaEvent_t e : pl.ev) cudaEventDestroy(e);
    pl.ev.clear();
    if (total_ms) *total_ms = tot;
    if (launches) *launches = pl.timed_launches;
    pl.timed_launches = 0;
    pl.timing = enable != 0;
    return DKT_OK;
  });
}

int dkt_plan_set_tile(dkt_plan plan, int tile_leaves)
{
  if (!plan || tile_leaves < 0) return fail(DKT_E_ARG, "bad argument");
  if (tile_leaves > 0 && !dkt::tile_size_supported(plan->pl.dim, tile_leaves))
    return fail(DKT_E_ARG, "unsupported tile size");
  if (tile_leaves > 0 && !plan->pl.fx_ready) return fail(DKT_E_UNSUP, "tiles need a Q1 built-in operator");
  return guarded([&]() {
    dkt::tile_setup(plan->pl, tile_leaves, 0);
    return DKT_OK;
  });
}

int dkt_plan_launch_count(dkt_plan plan, int64_t *count)
{
  if (!plan || !count) return fail(DKT_E_ARG, "null argument");
  *count = plan->pl.n_launch;
  return DKT_OK;
}

void dkt_plan_destroy(dkt_plan plan)
{
  if (!plan) return;
  for (cudaEvent_t e : plan->pl.ev) cudaEventDestroy(e);
  delete plan;
}

// ---- mesh generation (include/dkt_gb300_mesh.h) ----
int dkt_mesh_gaussian_points(int64_t n, int dim, int max_depth, double mean, double sd, uint64_t seed,
                             uint32_t *out)
{
  if (!out || n < 0 || dim < 2 || dim > 4 || max_depth < 1 || max_depth > 30) return fail(DKT_E_ARG, "bad argument");
  return guarded([&]() {
    dkt::gaussian_points(n, dim, max_depth, mean, sd, seed, out);
    return DKT_OK;
  });
}

static int export_cells(const std::vector<dkt::Cell> &cells, int dim, int64_t *n_out, uint32_t **coords,
                        uint8_t **levels)
{
  const size_t n = cells.size();
  uint32_t *c = (uint32_t *) std::malloc(n * dim * sizeof(uint32_t) + 1);
  uint8_t *l = (uint8_t *) std::malloc(n + 1);
  if (!c || !l) { std::free(c); std::free(l); return fail(DKT_E_NOMEM, "host allocation failed"); }
  for (size_t i = 0; i < n; i++) {
    for (int d = 0; d < dim; d++) c[i * dim + d] = cells[i].x[d];
    l[i] = (uint8_t) cells[i].lev;
  }
  *n_out = (int64_t) n;
  *coords = c;
  *levels = l;
  return DKT_OK;
}

int dkt_mesh_tree_from_points(const uint32_t *pts, int64_t n, int dim, int max_depth, int64_t max_pts,
                              int64_t *n_out, uint32_t **coords, uint8_t **levels)
{
  if (!pts || !n_out || !coords || !levels || n <= 0 || dim < 2 || dim > 4 || max_pts < 1)
    return fail(DKT_E_ARG, "bad argument");
  return guarded([&]() {
    const auto cells = dkt::tree_from_points(pts, n, dim, max_depth, max_pts);
    return export_cells(cells, dim, n_out, coords, levels);
  });
}

int dkt_mesh_moving_ball(int max_depth, int level, double radius, double halfwidth, const double *c0,
                         const double *c1, int64_t *n_out, uint32_t **coords, uint8_t **levels)
{
  if (!c0 || !c1 || !n_out || !coords || !levels || level < 1 || level > max_depth) return fail(DKT_E_ARG, "bad argument");
  return guarded([&]() {
    const auto cells = dkt::moving_ball_tree(max_depth, level, radius, halfwidth, c0, c1);
    return export_cells(cells, 4, n_out, coords, levels);
  });
}

int dkt_mesh_moving_ball_device(int max_depth, int level, double radius, double halfwidth, const double *c0,
                                const double *c1, int64_t *n_out, uint32_t **coords, uint8_t **levels)
{
  if (!c0 || !c1 || !n_out || !coords || !levels || level < 1 || level > max_depth || 4 * max_depth + 6 > 64)
    return fail(DKT_E_ARG, "bad argument");
  return guarded([&]() {
    dkt::DBuf<uint64_t> keys;
    int64_t n = 0;
    dkt::moving_ball_device(max_depth, level, radius, halfwidth, c0, c1, keys, n, 0);
    uint32_t *c = (uint32_t *) std::malloc((size_t) n * 4 * sizeof(uint32_t) + 1);
    uint8_t *l = (uint8_t *) std::malloc((size_t) n + 1);
    if (!c || !l) { std::free(c); std::free(l); return fail(DKT_E_NOMEM, "host allocation failed"); }
    dkt::unpack_cells_to_host(keys, n, 4, max_depth, c, l, 0);
    *n_out = n;
    *coords = c;
    *levels = l;
    return DKT_OK;
  });
}

int dkt_curve_tables(int curve, int dim, int8_t *rot, int32_t *ht, int *nrot)
{
  if (!rot || !ht || !nrot || dim < 2 || dim > 4) return fail(DKT_E_ARG, "bad argument");
  if (curve != DKT_CURVE_MORTON && curve != DKT_CURVE_HILBERT) return fail(DKT_E_ARG, "unknown curve");
  return guarded([&]() {
    dkt::CurveHost cv;
    set_curve(cv, curve, dim);
    std::copy(cv.rot.begin(), cv.rot.end(), rot);
    std::copy(cv.ht.begin(), cv.ht.end(), ht);
    *nrot = cv.nrot;
    return DKT_OK;
  });
}

int dkt_mesh_sphere_shell(int dim, int max_depth, int level, double radius, double halfwidth, const double *centre,
                          int64_t *n_out, uint32_t **coords, uint8_t **levels)
{
  if (!centre || !n_out || !coords || !levels || dim < 2 || dim > 4 || level < 1 || level > max_depth ||
      dim * max_depth + 6 > 64)
    return fail(DKT_E_ARG, "bad argument");
  return guarded([&]() {
    const auto cells = dkt::sphere_shell_tree(dim, max_depth, level, radius, halfwidth, centre);
    return export_cells(cells, dim, n_out, coords, levels);
  });
}

int dkt_mesh_sphere_shell_device(int dim, int max_depth, int level, double radius, double halfwidth,
                                 const double *centre, int64_t *n_out, uint32_t **coords, uint8_t **levels)
{
  if (!centre || !n_out || !coords || !levels || dim < 2 || dim > 4 || level < 1 || level > max_depth ||
      dim * max_depth + 6 > 64)
    return fail(DKT_E_ARG, "bad argument");
  return guarded([&]() {
    dkt::DBuf<uint64_t> keys;
    int64_t n = 0;
    dkt::sphere_shell_device(dim, max_depth, level, radius, halfwidth, centre, keys, n, 0);
    uint32_t *c = (uint32_t *) std::malloc((size_t) n * dim * sizeof(uint32_t) + 1);
    uint8_t *l = (uint8_t *) std::malloc((size_t) n + 1);
    if (!c || !l) { std::free(c); std::free(l); return fail(DKT_E_NOMEM, "host allocation failed"); }
    dkt::unpack_cells_to_host(keys, n, dim, max_depth, c, l, 0);
    *n_out = n;
    *coords = c;
    *levels = l;
    return DKT_OK;
  });
}

int dkt_mesh_tree_from_points_device(const uint32_t *pts, int64_t n, int dim, int max_depth, int64_t max_pts,
                                     int64_t *n_out, uint32_t **coords, uint8_t **levels)
{
  if (!pts || !n_out || !coords || !levels || n <= 0 || dim < 2 || dim > 4 || max_pts < 1 || max_depth < 1 ||
      dim * max_depth + 6 > 64)
    return fail(DKT_E_ARG, "bad argument");
  return guarded([&]() {
    for (int64_t i = 0; i < n * dim; i++)
      if (pts[i] >= (1u << max_depth)) throw std::invalid_argument("point outside the domain");
    dkt::DBuf<uint64_t> keys;
    int64_t nc = 0;
    dkt::tree_from_points_device(pts, n, dim, max_depth, max_pts, keys, nc, 0);
    uint32_t *c = (uint32_t *) std::malloc((size_t) nc * dim * sizeof(uint32_t) + 1);
    uint8_t *l = (uint8_t *) std::malloc((size_t) nc + 1);
    if (!c || !l) { std::free(c); std::free(l); return fail(DKT_E_NOMEM, "host allocation failed"); }
    dkt::unpack_cells_to_host(keys, nc, dim, max_depth, c, l, 0);
    *n_out = nc;
    *coords = c;
    *levels = l;
    return DKT_OK;
  });
}

int dkt_mesh_function2octree(dkt_field_fn fn, void *user, int n_vars, int dim, int max_depth, int order,
                             double interp_tol, int balance, int64_t *n_out, uint32_t **coords, uint8_t **levels)
{
  if (!fn || !n_out || !coords || !levels || n_vars < 1 || n_vars > 64 || dim < 2 || dim > 4 || order < 1 ||
      order > 2 || max_depth < 1 || dim * max_depth + 6 > 64 || !(interp_tol >= 0))
    return fail(DKT_E_ARG, "bad argument");
  return guarded([&]() {
    dkt::DBuf<uint64_t> keys;
    int64_t nc = 0;
    dkt::function2octree_device(fn, user, n_vars, dim, max_depth, order, interp_tol, balance != 0, keys, nc, 0);
    uint32_t *c = (uint32_t *) std::malloc((size_t) nc * dim * sizeof(uint32_t) + 1);
    uint8_t *l = (uint8_t *) std::malloc((size_t) nc + 1);
    if (!c || !l) { std::free(c); std::free(l); return fail(DKT_E_NOMEM, "host allocation failed"); }
    dkt::unpack_cells_to_host(keys, nc, dim, max_depth, c, l, 0);
    *n_out = nc;
    *coords = c;
    *levels = l;
    return DKT_OK;
  });
}

int dkt_write_vtu(const char *path, int dim, int max_depth, const uint32_t *coords, const uint8_t *levels,
                  int64_t n_cells, const double *cell_values, const char *cell_values_name)
{
  if (!path || (n_cells > 0 && (!coords || !levels)) || n_cells < 0 || (dim != 2 && dim != 3) || max_depth < 1 ||
      max_depth > 30)
    return fail(DKT_E_ARG, "bad argument");
  return guarded([&]() {
    dkt::write_vtu(path, dim, max_depth, coords, levels, n_cells, cell_values, cell_values_name);
    return DKT_OK;
  });
}

void dkt_free(void *p) { std::free(p); }

}  // extern "C"
