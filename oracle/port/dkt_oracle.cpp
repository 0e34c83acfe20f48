// CPU oracle: a restatement of Dendro-KT's adaptive k-tree matvec path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product links, loads or calls this
// library; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg use it, as the checker.  It follows the reference's algorithms step by
// step (recursive SFC bucketing, countCGNodes, the recursive mesh-free
// traversal with its static buffers) so that it can be timed as the
// reference's own CPU algorithm on a machine where the reference sources are
// absent, and so that its outputs can be pinned against the reference build
// (oracle/ref) on golden fixtures.
//
// Reference citations are paths inside the Dendro-KT project.
#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Global configuration of one call (the reference keeps these as globals:
// m_uiMaxDepth src/treeNode.cpp:4, rotations/HILBERT_TABLE src/KDhcurvedata.cpp:22-23).
// ---------------------------------------------------------------------------
struct Curve {
  int nc = 0;
  std::vector<int8_t> rot;   // rot[r*2*nc + 0*nc + sfc] = morton child; [.. + 1*nc + morton] = sfc rank
  std::vector<int32_t> ht;   // ht[r*nc + morton] = child orientation
};

unsigned g_md = 10;
Curve g_curve;

void set_curve(int dim, const int8_t *rot, const int32_t *ht, int nrot)
{
  const int nc = 1 << dim;
  g_curve.nc = nc;
  if (rot == nullptr) {   // Morton: identity tables (src/KDhcurvedata.cpp:47-59)
    g_curve.rot.assign(2 * nc, 0);
    g_curve.ht.assign(nc, 0);
    for (int c = 0; c < nc; c++) { g_curve.rot[c] = (int8_t) c; g_curve.rot[nc + c] = (int8_t) c; }
  } else {
    g_curve.rot.assign(rot, rot + (size_t) nrot * 2 * nc);
    g_curve.ht.assign(ht, ht + (size_t) nrot * nc);
  }
}
inline const int8_t *rot_perm(int r) { return &g_curve.rot[(size_t) r * 2 * g_curve.nc]; }
inline const int8_t *rot_inv(int r) { return &g_curve.rot[(size_t) r * 2 * g_curve.nc + g_curve.nc]; }
inline const int32_t *orient(int r) { return &g_curve.ht[(size_t) r * g_curve.nc]; }

// ---------------------------------------------------------------------------
// TreeNode / TNPoint restated (include/treeNode.h:36-253, include/nsort.h:79-176)
// ---------------------------------------------------------------------------
template <int dim>
struct TN {
  uint32_t x[dim];
  uint32_t lev;
  // transient fields of TNPoint (include/nsort.h:171-174)
  uint8_t sel = 1;      // 0 No, 1 Maybe, 2 Yes
  uint8_t ninst = 1;
};

inline uint32_t cell_len(unsigned lev) { return 1u << (g_md - lev); }

// TreeNode(coords, level) masks low bits (include/treeNode.tcc:60-80).
template <int dim>
TN<dim> make_cell(const uint32_t *c, unsigned lev)
{
  TN<dim> t;
  const uint32_t mask = ~(cell_len(lev) - 1u);
  for (int d = 0; d < dim; d++) t.x[d] = c[d] & mask;
  t.lev = lev;
  return t;
}

// getMortonIndex(level) (include/treeNode.tcc:244-258)
template <int dim>
inline unsigned morton_index(const TN<dim> &t, unsigned lev)
{
  const uint64_t len = 1ull << (g_md - lev), lenp = len << 1;
  unsigned c = 0;
  for (int d = 0; d < dim; d++) c += (unsigned) (((t.x[d] % lenp) / len) << d);
  return c;
}

template <int dim>
inline bool same_coords(const TN<dim> &a, const TN<dim> &b)
{
  for (int d = 0; d < dim; d++) if (a.x[d] != b.x[d]) return false;
  return true;
}
template <int dim>
inline bool tn_equal(const TN<dim> &a, const TN<dim> &b) { return a.lev == b.lev && same_coords(a, b); }

// isAncestor (include/treeNode.tcc:636-660)
template <int dim>
inline bool is_ancestor(const TN<dim> &a, const TN<dim> &b)
{
  if (!(a.lev < b.lev)) return false;
  const uint64_t la = cell_len(a.lev), lb = cell_len(b.lev);
  for (int d = 0; d < dim; d++)
    if (!(b.x[d] >= a.x[d] && (uint64_t) b.x[d] + lb <= (uint64_t) a.x[d] + la)) return false;
  return true;
}

template <int dim>
inline TN<dim> get_parent(const TN<dim> &t)
{
  const unsigned pl = t.lev > 0 ? t.lev - 1 : 0;
  TN<dim> p;
  for (int d = 0; d < dim; d++) p.x[d] = (t.x[d] >> (g_md - pl)) << (g_md - pl);
  p.lev = pl;
  return p;
}

template <int dim>
inline TN<dim> child_morton(const TN<dim> &t, unsigned child)
{
  TN<dim> c;
  const uint32_t clen = cell_len(t.lev + 1);
  for (int d = 0; d < dim; d++) c.x[d] = (t.x[d] & ~(cell_len(t.lev) - 1u)) | ((child >> d) & 1u ? clen : 0u);
  c.lev = t.lev + 1;
  return c;
}

// isOnDomainBoundary (include/treeNode.tcc:616-624)
template <int dim>
inline bool on_domain_boundary(const TN<dim> &t)
{
  const uint32_t mask = (1u << g_md) - 1u;
  for (int d = 0; d < dim; d++) if (!(t.x[d] & mask)) return true;
  return false;
}

// TNPoint::get_cellType(lev) (include/nsort.tcc:163-184): bit d set iff the
// coordinate is interior to the level-lev cell along axis d.
template <int dim>
inline void cell_type(const TN<dim> &t, unsigned lev, unsigned &orient, unsigned &cdim)
{
  const uint32_t mask = cell_len(lev) - 1u;
  orient = 0; cdim = 0;
  for (int d = 0; d < dim; d++) { bool in = (t.x[d] & mask) != 0; orient |= (unsigned) in << d; cdim += in; }
}

// get_firstIncidentHyperplane (include/nsort.tcc:137-151)
template <int dim>
inline unsigned first_incident_hyperplane(const TN<dim> &t, unsigned hlev)
{
  const uint32_t mask = cell_len(hlev) - 1u;
  for (int d = 0; d < dim; d++) if (!(t.x[d] & mask)) return d;
  return dim;
}

// getFinestOpenContainer (include/nsort.tcc:203-230)
template <int dim>
inline TN<dim> finest_open_container(const TN<dim> &t)
{
  unsigned h = 0;
  for (int d = 0; d < dim; d++) {
    unsigned v = t.x[d], pos = 0;
    while (!(v & 1u)) { v >>= 1; pos++; }
    if (pos > h) h = pos;
  }
  const unsigned level = g_md - h - 1;
  return make_cell<dim>(t.x, level);
}

// get_lexNodeRank (include/nsort.tcc:283-303)
template <int dim>
inline unsigned lex_node_rank(const TN<dim> &pt, const TN<dim> &host, unsigned p)
{
  const uint64_t len = cell_len(host.lev);
  unsigned rank = 0, stride = 1;
  for (int d = 0; d < dim; d++) {
    unsigned idx = p - (unsigned) ((uint64_t) p * ((uint64_t) host.x[d] + len - pt.x[d]) / len);
    rank += idx * stride;
    stride *= (p + 1);
  }
  return rank;
}

inline unsigned ipow(unsigned b, unsigned e) { unsigned r = 1; while (e--) r *= b; return r; }

// ---------------------------------------------------------------------------
// SFC bucketing (include/tsort.tcc:162-334).  A stable counting sort: the
// reference's in-place cycle-leader move orders equal keys differently, but
// equal keys are equal TreeNodes everywhere this is used, so outputs match.
// ---------------------------------------------------------------------------
template <int dim, typename KeyFun>
void sfc_bucketing(TN<dim> *pts, size_t begin, size_t end, unsigned lev, int pRot, KeyFun key,
                   bool sepAnc, bool ancFirst, std::array<size_t, 17> &split, size_t &ancS, size_t &ancE)
{
  const int nc = 1 << dim;
  std::array<size_t, 16> counts{};
  size_t nAnc = 0;
  std::vector<int> bucket(end - begin);
  for (size_t i = begin; i < end; i++) {
    TN<dim> k = key(pts[i]);
    int b;
    if (sepAnc && k.lev < lev) { b = nc; nAnc++; }
    else { b = (int) morton_index(k, lev); counts[b]++; }
    bucket[i - begin] = b;
  }
  size_t acc = ancFirst ? begin + nAnc : begin;
  const int8_t *rp = rot_perm(pRot);
  std::array<size_t, 17> off{};
  for (int s = 0; s < nc; s++) { int m = rp[s]; split[s] = acc; off[m] = acc; acc += counts[m]; }
  split[nc] = acc;
  if (ancFirst) { ancS = begin; ancE = begin + nAnc; } else { ancS = acc; ancE = acc + nAnc; }
  off[nc] = ancS;
  std::vector<TN<dim>> tmp(pts + begin, pts + end);
  for (size_t i = 0; i < tmp.size(); i++) pts[off[bucket[i]]++] = tmp[i];
}

template <int dim>
struct IdKey { TN<dim> operator()(const TN<dim> &t) const { return t; } };

// SFC_Tree::locTreeSort (include/tsort.tcc:14-80)
template <int dim>
void loc_tree_sort(TN<dim> *pts, size_t begin, size_t end, unsigned sLev, unsigned eLev, int pRot)
{
  if (end <= begin) return;
  const int nc = 1 << dim;
  std::array<size_t, 17> sp; size_t a0, a1;
  sfc_bucketing<dim>(pts, begin, end, sLev, pRot, IdKey<dim>(), true, true, sp, a0, a1);
  if (sLev < eLev) {
    const int8_t *rp = rot_perm(pRot);
    const int32_t *ol = orient(pRot);
    for (int s = 0; s < nc; s++) {
      int cRot = ol[(int) rp[s]];
      if (sp[s + 1] - sp[s] <= 1) continue;
      loc_tree_sort<dim>(pts, sp[s], sp[s + 1], sLev + 1, eLev, sLev > 0 ? cRot : pRot);
    }
  }
}

// SFC_Tree::locTreeConstruction (src/tsort.cpp:566-645)
template <int dim>
void loc_tree_construction(TN<dim> *pts, std::vector<TN<dim>> &tree, size_t maxPts, size_t begin, size_t end,
                           unsigned sLev, unsigned eLev, int pRot, TN<dim> pNode)
{
  if (end <= begin) return;
  const int nc = 1 << dim;
  std::array<size_t, 17> sp; size_t a0, a1;
  sfc_bucketing<dim>(pts, begin, end, sLev, pRot, IdKey<dim>(), true, true, sp, a0, a1);
  const int8_t *rp = rot_perm(pRot);
  const int32_t *ol = orient(pRot);
  if (sLev < eLev) {
    for (int s = 0; s < nc; s++) {
      int child = rp[s];
      TN<dim> cNode = child_morton(pNode, child);
      if (sp[s + 1] - sp[s] > maxPts)
        loc_tree_construction<dim>(pts, tree, maxPts, sp[s], sp[s + 1], sLev + 1, eLev, ol[child], cNode);
      else
        tree.push_back(cNode);
    }
  } else {
    for (int s = 0; s < nc; s++) tree.push_back(child_morton(pNode, rp[s]));
  }
}

// SFC_Tree::locRemoveDuplicates (src/tsort.cpp:720-744)
template <int dim>
void loc_remove_duplicates(std::vector<TN<dim>> &t)
{
  size_t nu = 0, cur = 0;
  const size_t n = t.size();
  while (cur < n) {
    while (cur + 1 < n && (tn_equal(t[cur], t[cur + 1]) || is_ancestor(t[cur], t[cur + 1]))) cur++;
    t[nu++] = t[cur];
    cur++;
  }
  t.resize(nu);
}

// TreeNode::appendAllNeighbours (include/treeNode.tcc:525-586), includeDomBdry = false
template <int dim>
void append_all_neighbours(const TN<dim> &t, std::vector<TN<dim>> &out)
{
  const uint64_t len = cell_len(t.lev), top = 1ull << g_md;
  const unsigned n3 = ipow(3, dim);
  for (unsigned idx = 1; idx < n3; idx++) {
    bool ok = true;
    TN<dim> nb = t;
    unsigned r = idx;
    for (int d = 0; d < dim && ok; d++) {
      unsigned delta = r % 3; r /= 3;   // 0: same, 1: +1, 2: -1
      if (delta == 1) { if ((uint64_t) t.x[d] >= top - len) ok = false; else nb.x[d] = t.x[d] + (uint32_t) len; }
      else if (delta == 2) { if ((uint64_t) t.x[d] < len) ok = false; else nb.x[d] = t.x[d] - (uint32_t) len; }
    }
    if (ok) out.push_back(nb);
  }
}

// SFC_Tree::propagateNeighbours (src/tsort.cpp:777-820)
template <int dim>
void propagate_neighbours(std::vector<TN<dim>> &nodes)
{
  std::vector<std::vector<TN<dim>>> lv(g_md + 1);
  for (auto &t : nodes) lv[t.lev].push_back(t);
  nodes.clear();
  for (unsigned l = g_md; l > 0; l--) {
    const unsigned lp = l - 1;
    for (const auto &t : lv[l]) {
      TN<dim> p = get_parent(t);
      lv[lp].push_back(p);
      append_all_neighbours(p, lv[lp]);
    }
    loc_tree_sort<dim>(lv[lp].data(), 0, lv[lp].size(), 1, lp, 0);
    loc_remove_duplicates(lv[lp]);
  }
  for (auto &v : lv) nodes.insert(nodes.end(), v.begin(), v.end());
}

// SFC_Tree::locTreeBalancing (src/tsort.cpp:826-854)
template <int dim>
std::vector<TN<dim>> loc_tree_balancing(std::vector<TN<dim>> pts, size_t maxPts)
{
  std::vector<TN<dim>> tree, nt;
  TN<dim> root{}; root.lev = 0;
  loc_tree_construction<dim>(pts.data(), tree, maxPts, 0, pts.size(), 1, g_md, 0, root);
  propagate_neighbours(tree);
  loc_tree_construction<dim>(tree.data(), nt, 1, 0, tree.size(), 1, g_md, 0, root);
  return nt;
}

// ---------------------------------------------------------------------------
// Node generation (include/nsort.tcc:311-389)
// ---------------------------------------------------------------------------
template <int dim>
void append_exterior_nodes(const TN<dim> &e, unsigned p, std::vector<TN<dim>> &out)
{
  const uint64_t len = cell_len(e.lev);
  const unsigned n = ipow(p + 1, dim);
  std::array<unsigned, dim> idx{};
  for (unsigned node = 0; node < n; node++) {
    bool ext = false;
    for (int d = 0; d < dim; d++) if (idx[d] == 0 || idx[d] == p) ext = true;
    if (ext) {
      TN<dim> t;
      for (int d = 0; d < dim; d++) t.x[d] = (uint32_t) (len * idx[d] / p) + e.x[d];
      t.lev = e.lev;
      out.push_back(t);
    }
    for (int d = 0; d < dim; d++) { if (++idx[d] <= p) break; idx[d] = 0; }
  }
}

template <int dim>
void append_interior_nodes(const TN<dim> &e, unsigned p, std::vector<TN<dim>> &out)
{
  if (p < 2) return;
  const uint64_t len = cell_len(e.lev);
  const unsigned n = ipow(p - 1, dim);
  std::array<unsigned, dim> idx{};
  for (unsigned node = 0; node < n; node++) {
    TN<dim> t;
    for (int d = 0; d < dim; d++) t.x[d] = (uint32_t) (len * (idx[d] + 1) / p) + e.x[d];
    t.lev = e.lev;
    out.push_back(t);
    for (int d = 0; d < dim; d++) { if (++idx[d] < p - 1) break; idx[d] = 0; }
  }
}

// Lexicographic element nodes (Element::appendNodes, include/nsort.tcc:311-334)
template <int dim>
void element_node_coords(const TN<dim> &e, unsigned p, std::vector<double> &coords)
{
  const uint64_t len = cell_len(e.lev);
  const unsigned n = ipow(p + 1, dim);
  coords.resize((size_t) n * dim);
  const double sc = 1.0 / (double) (1u << g_md);
  std::array<unsigned, dim> idx{};
  for (unsigned node = 0; node < n; node++) {
    for (int d = 0; d < dim; d++) coords[(size_t) node * dim + d] = sc * (double) ((uint32_t) (len * idx[d] / p) + e.x[d]);
    for (int d = 0; d < dim; d++) { if (++idx[d] <= p) break; idx[d] = 0; }
  }
}

// ---------------------------------------------------------------------------
// countCGNodes (include/nsort.tcc:878-944) with the low-order resolver
// ---------------------------------------------------------------------------
template <int dim>
void loc_tree_sort_as_points(TN<dim> *pts, size_t begin, size_t end, unsigned sLev, unsigned eLev, int pRot)
{
  if (end <= begin) return;
  const int nc = 1 << dim;
  std::array<size_t, 17> sp; size_t a0, a1;
  sfc_bucketing<dim>(pts, begin, end, sLev, pRot, IdKey<dim>(), false, true, sp, a0, a1);
  if (sLev < eLev) {
    const int8_t *rp = rot_perm(pRot);
    const int32_t *ol = orient(pRot);
    for (int s = 0; s < nc; s++) {
      if (sp[s + 1] - sp[s] <= 1) continue;
      int cRot = ol[(int) rp[s]];
      bool ident = true;
      for (size_t i = sp[s] + 1; i < sp[s + 1]; i++) if (!same_coords(pts[i], pts[sp[s]])) { ident = false; break; }
      if (!ident) loc_tree_sort_as_points<dim>(pts, sp[s], sp[s + 1], sLev + 1, eLev, sLev > 0 ? cRot : pRot);
      // identical coordinates: the reference only regroups by level here
      // (include/nsort.tcc:1064-1101); no output depends on that order.
    }
  }
}

// scanForDuplicates (include/nsort.tcc:1111-1139)
template <int dim>
void scan_for_duplicates(TN<dim> *start, TN<dim> *end, TN<dim> *&firstCoarsest, TN<dim> *&next, unsigned &numDups)
{
  next = start + 1;
  firstCoarsest = start;
  unsigned ninst = start->ninst;
  bool same = true;
  while (next < end && same_coords(*next, *start)) {
    ninst += next->ninst;
    if (same && next->lev != firstCoarsest->lev) same = false;
    if (next->lev < firstCoarsest->lev) firstCoarsest = next;
    next++;
  }
  numDups = same ? ninst : 0;
}

// resolveInterface_lowOrder (include/nsort.tcc:1266-1313)
template <int dim>
size_t resolve_low_order(TN<dim> *start, TN<dim> *end)
{
  for (TN<dim> *p = start; p < end; p++) p->sel = 0;
  size_t total = 0;
  TN<dim> *it = start;
  while (it < end) {
    TN<dim> *fc, *nx; unsigned nd;
    scan_for_duplicates(it, end, fc, nx, nd);
    if (!nd) { fc->sel = 2; total++; }
    else {
      unsigned orient, cdim;
      cell_type(*fc, fc->lev, orient, cdim);
      if (nd == (1u << (dim - cdim))) { fc->sel = 2; total++; }
    }
    it = nx;
  }
  return total;
}

template <int dim>
struct ContainerKey { TN<dim> operator()(const TN<dim> &t) const { return finest_open_container(t); } };

// countCGNodes_impl (include/nsort.tcc:1153-1231)
template <int dim>
size_t count_cg_nodes_impl(TN<dim> *start, TN<dim> *end, unsigned sLev, int pRot)
{
  if (!(start < end)) return 0;
  const int nc = 1 << dim;
  size_t nu = 0;
  std::array<size_t, 17> sp; size_t a0, a1;
  sfc_bucketing<dim>(start, 0, end - start, sLev, pRot, ContainerKey<dim>(), true, false, sp, a0, a1);
  const int8_t *rp = rot_perm(pRot);
  const int32_t *ol = orient(pRot);
  for (int s = 0; s < nc; s++) {
    if (sp[s + 1] - sp[s] == 0) continue;
    int cRot = ol[(int) rp[s]];
    nu += count_cg_nodes_impl<dim>(start + sp[s], start + sp[s + 1], sLev + 1, cRot);
  }
  // Own interface: bucketByHyperplane (include/nsort.tcc:1237-1260), stable.
  TN<dim> *as = start + a0, *ae = start + a1;
  std::array<size_t, dim + 1> hc{};
  for (TN<dim> *p = as; p < ae; p++) hc[first_incident_hyperplane(*p, sLev)]++;
  std::array<size_t, dim + 1> ho{};
  size_t acc = 0;
  for (int d = 0; d <= dim; d++) { ho[d] = acc; acc += hc[d]; }
  std::vector<TN<dim>> buf(ae - as);
  std::array<size_t, dim + 1> hw = ho;
  for (TN<dim> *p = as; p < ae; p++) buf[hw[first_incident_hyperplane(*p, sLev)]++] = *p;
  std::copy(buf.begin(), buf.end(), as);
  for (int d = 0; d < dim; d++) {
    loc_tree_sort_as_points<dim>(as, ho[d], ho[d] + hc[d], sLev, g_md, pRot);
    nu += resolve_low_order<dim>(as + ho[d], as + ho[d] + hc[d]);
  }
  return nu;
}

template <int dim>
size_t count_cg_nodes(TN<dim> *start, TN<dim> *end)
{
  const int nc = 1 << dim;
  // filterDomainBoundary: stable, boundary points to the end (include/nsort.tcc:950-989)
  std::vector<TN<dim>> in, bd;
  for (TN<dim> *p = start; p < end; p++) (on_domain_boundary(*p) ? bd : in).push_back(*p);
  std::copy(in.begin(), in.end(), start);
  std::copy(bd.begin(), bd.end(), start + in.size());
  const size_t nB = bd.size();
  TN<dim> *bs = end - nB;
  if (!(end > start)) return 0;
  // Boundary points: root bucketing with rotation 0, then sort as points (nsort.tcc:889-906)
  std::array<size_t, 17> sp; size_t a0, a1;
  sfc_bucketing<dim>(bs, 0, nB, 0, 0, IdKey<dim>(), false, true, sp, a0, a1);
  for (int s = 0; s < nc; s++) {
    if (sp[s + 1] - sp[s] <= 1) continue;
    loc_tree_sort_as_points<dim>(bs, sp[s], sp[s + 1], 1, g_md, 0);
  }
  size_t total = 0;
  for (TN<dim> *p = bs; p < end; p++) p->sel = 0;
  TN<dim> *it = bs;
  while (it < end) {
    TN<dim> *fc, *nx; unsigned nd;
    scan_for_duplicates(it, end, fc, nx, nd);
    fc->sel = 2;
    total++;
    it = nx;
  }
  total += count_cg_nodes_impl<dim>(start, end - nB, 1, 0);
  return total;
}

// ---------------------------------------------------------------------------
// 1D reference-element operators (FEM/src/refel.cpp:75-220), from the
// mathematics: Lagrange basis on the equispaced nodes u_k = -1 + 2k/p,
// Gauss-Legendre points/weights by Newton iteration on P_{p+1}.
// Layout as the reference stores them: A[k*M + j] = basis k at point j.
// ---------------------------------------------------------------------------
struct RefEl {
  unsigned p = 1, M = 2;
  std::vector<double> ip0, ip1, Q, D, W;
};

double lagrange(const std::vector<double> &u, unsigned k, double x)
{
  double v = 1.0;
  for (unsigned m = 0; m < u.size(); m++) if (m != k) v *= (x - u[m]) / (u[k] - u[m]);
  return v;
}
double lagrange_d(const std::vector<double> &u, unsigned k, double x)
{
  double s = 0.0;
  for (unsigned i = 0; i < u.size(); i++) {
    if (i == k) continue;
    double t = 1.0 / (u[k] - u[i]);
    for (unsigned m = 0; m < u.size(); m++) if (m != k && m != i) t *= (x - u[m]) / (u[k] - u[m]);
    s += t;
  }
  return s;
}

RefEl make_refel(unsigned p)
{
  RefEl r; r.p = p; r.M = p + 1;
  const unsigned M = r.M;
  std::vector<double> u(M), g(M), w(M);
  for (unsigned k = 0; k < M; k++) u[k] = -1.0 + 2.0 * k / p;
  for (unsigned i = 0; i < M; i++) {   // roots of P_M, ascending
    double x = -std::cos(M_PI * (i + 0.75) / (M + 0.5));
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = x;
      for (unsigned n = 2; n <= M; n++) { double p2 = ((2.0 * n - 1) * x * p1 - (n - 1.0) * p0) / n; p0 = p1; p1 = p2; }
      double dp = M * (x * p1 - p0) / (x * x - 1.0);
      double dx = p1 / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-17) break;
    }
    double p0 = 1.0, p1 = x;
    for (unsigned n = 2; n <= M; n++) { double p2 = ((2.0 * n - 1) * x * p1 - (n - 1.0) * p0) / n; p0 = p1; p1 = p2; }
    double dp = M * (x * p1 - p0) / (x * x - 1.0);
    g[i] = x;
    w[i] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
  if (M == 1) { g[0] = 0.0; w[0] = 2.0; }
  r.ip0.resize(M * M); r.ip1.resize(M * M); r.Q.resize(M * M); r.D.resize(M * M); r.W = w;
  for (unsigned k = 0; k < M; k++)
    for (unsigned j = 0; j < M; j++) {
      r.ip0[k * M + j] = lagrange(u, k, 0.5 * (u[j] - 1.0));
      r.ip1[k * M + j] = lagrange(u, k, 0.5 * (u[j] + 1.0));
      r.Q[k * M + j] = lagrange(u, k, g[j]);
      r.D[k * M + j] = lagrange_d(u, k, g[j]);
    }
  return r;
}

// y[..j..] = sum_k A[k*M+j] x[..k..] along `axis`; with `transpose` the
// matrix is applied as A[j*M+k] (the reference's *T1d arrays).
void apply_axis(unsigned dim, unsigned M, const double *A, bool transpose, const double *x, double *y, unsigned axis)
{
  unsigned stride = 1, n = 1;
  for (unsigned a = 0; a < axis; a++) stride *= M;
  for (unsigned a = 0; a < dim; a++) n *= M;
  for (unsigned idx = 0; idx < n; idx++) {
    const unsigned j = (idx / stride) % M;
    const unsigned base = idx - j * stride;
    double s = 0.0;
    for (unsigned k = 0; k < M; k++) s += (transpose ? A[j * M + k] : A[k * M + j]) * x[base + k * stride];
    y[idx] = s;
  }
}

// RefElement::IKD_Parent2Child / IKD_Child2Parent (FEM/include/refel.h:214-271)
void ikd_interp(unsigned dim, const RefEl &re, const double *in, double *out, unsigned child, bool transpose)
{
  const unsigned n = ipow(re.M, dim);
  std::vector<double> a(in, in + n), b(n);
  for (unsigned d = 0; d < dim; d++) {
    const double *A = ((child >> d) & 1u) ? re.ip1.data() : re.ip0.data();
    apply_axis(dim, re.M, A, transpose, a.data(), b.data(), d);
    std::swap(a, b);
  }
  std::copy(a.begin(), a.end(), out);
}

// ---------------------------------------------------------------------------
// Elemental operators
//   op 0: identity (test/testMatvec.cpp:187-198)
//   op 1: HeatMat<dim>::elementalMatVec, 3-axis stiffness with J = h/2
//         (FEM/examples/src/heatMat.cpp:45-117)
//   op 2: Laplacian + mass, J^(d-2) K_ref + J^d M_ref (restated operator)
//   op 4 / op 5: its Laplacian / its mass term alone
//   op 6: HeatVec<dim>::elementalComputeVec, J^d M_ref with the scale ignored
//         (FEM/examples/src/heatVec.cpp:30-78), Dirichlet zeroing of input
//         and output as pre/postComputeVec (:83-105)
// ---------------------------------------------------------------------------
void ele_op(int op, unsigned dim, const RefEl &re, const double *in, double *out, const double *coords, double scale)
{
  const unsigned M = re.M, n = ipow(M, dim);
  if (op == 0) { for (unsigned i = 0; i < n; i++) out[i] = in[i]; return; }
  std::vector<double> wq(n), acc(n, 0.0), a(n), b(n);
  for (unsigned idx = 0; idx < n; idx++) {
    double w = 1.0; unsigned r = idx;
    for (unsigned d = 0; d < dim; d++) { w *= re.W[r % M]; r /= M; }
    wq[idx] = w;
  }
  if (op == 1) {
    // Element size from the first and last element node, first three axes
    // (heatMat.cpp:61-86); the quadrature weights cover three axes only.
    const unsigned nax = dim < 3 ? dim : 3;
    double J[3] = {1, 1, 1};
    for (unsigned d = 0; d < nax; d++) J[d] = (coords[(n - 1) * dim + d] - coords[d]) / 2.0;
    for (unsigned t = 0; t < nax; t++) {
      std::copy(in, in + n, a.begin());
      for (unsigned d = 0; d < nax; d++) { apply_axis(dim, M, d == t ? re.D.data() : re.Q.data(), false, a.data(), b.data(), d); std::swap(a, b); }
      double f = 1.0;
      for (unsigned d = 0; d < nax; d++) f *= (d == t) ? 1.0 / J[d] : J[d];
      for (unsigned idx = 0; idx < n; idx++) {
        double w = 1.0; unsigned r = idx;
        for (unsigned d = 0; d < nax; d++) { w *= re.W[r % M]; r /= M; }
        a[idx] *= f * w;
      }
      for (unsigned d = 0; d < nax; d++) { apply_axis(dim, M, d == t ? re.D.data() : re.Q.data(), true, a.data(), b.data(), d); std::swap(a, b); }
      for (unsigned idx = 0; idx < n; idx++) acc[idx] += a[idx];
    }
    for (unsigned i = 0; i < n; i++) out[i] = acc[i];
    return;
  }
  const double h = coords[(n - 1) * dim + 0] - coords[0];
  const double J = 0.5 * h;
  double Jdm2 = 1.0, Jd = 1.0;
  for (unsigned k = 0; k + 2 < dim; k++) Jdm2 *= J;
  for (unsigned k = 0; k < dim; k++) Jd *= J;
  if (dim < 2) Jdm2 = 1.0 / J;
  for (int term = -1; term < (int) dim; term++) {
    std::copy(in, in + n, a.begin());
    for (unsigned d = 0; d < dim; d++) { apply_axis(dim, M, (int) d == term ? re.D.data() : re.Q.data(), false, a.data(), b.data(), d); std::swap(a, b); }
    for (unsigned idx = 0; idx < n; idx++) a[idx] *= wq[idx];
    for (unsigned d = 0; d < dim; d++) { apply_axis(dim, M, (int) d == term ? re.D.data() : re.Q.data(), true, a.data(), b.data(), d); std::swap(a, b); }
    double f = term < 0 ? Jd : Jdm2;
    if (op == 4 && term < 0) f = 0.0;   // Laplacian only
    if ((op == 5 || op == 6) && term >= 0) f = 0.0;  // mass only
    for (unsigned idx = 0; idx < n; idx++) acc[idx] += f * a[idx];
  }
  if (op == 6) scale = 1.0;   // HeatVec ignores the scale argument
  for (unsigned i = 0; i < n; i++) out[i] = scale * acc[i];
}

// ---------------------------------------------------------------------------
// fem::matvec (FEM/include/matvec.h:74-548), restated with the same
// function-static buffer semantics (matvec.h:275-299): the parent buffer keeps
// values from earlier leaves in slots that are not refilled.
// ---------------------------------------------------------------------------
struct MatvecStats {
  int64_t leaves = 0, hanging_leaves = 0, stale_reads = 0, aliased = 0, max_depth_seen = 0, ref_errors = 0;
};
// 0: parent-buffer slots keep earlier leaves' values, as the reference's
// function-static buffer does; 1: unfilled slots read as zero.
int g_stale_mode = 0;
// Conforming variant (not the reference's behaviour): the parent values are
// taken from every node on the parent's lattice whatever its level, and the
// transpose adds to every such parent node, which makes the operator the
// symmetric P^T K P.  Used as the oracle of the conforming device mode.
int g_conforming = 0;

template <int dim>
inline bool on_lattice(const TN<dim> &pt, const TN<dim> &host, unsigned p)
{
  const uint64_t len = cell_len(host.lev);
  for (int d = 0; d < dim; d++) {
    const uint64_t off = (uint64_t) pt.x[d] - host.x[d];
    if ((off * p) % len) return false;
  }
  return true;
}

template <int dim>
struct Traversal {
  unsigned p;
  int op;
  const RefEl *re;
  TN<dim> partFront, partBack;
  struct Buf { std::vector<TN<dim>> coords; std::vector<double> vin, vout; std::vector<int8_t> smap; };
  std::vector<Buf> ibufs;
  std::vector<double> parentBuf, leafIn, leafOut, coordBuf;
  std::vector<uint8_t> parentFill, leafFill, parentFresh;
  MatvecStats st;

  // top_down (matvec.h:74-199)
  bool top_down(const TN<dim> *coords, const double *vec, size_t sz, std::array<size_t, 16> &offsets,
                std::array<size_t, 16> &counts, Buf &B, const TN<dim> &root, int pRot)
  {
    const unsigned pLev = root.lev, nc = 1u << dim;
    bool leaf = true;
    for (size_t i = 0; i < sz; i++) if (coords[i].lev > pLev) { leaf = false; break; }
    if (leaf) return true;
    counts.fill(0); offsets.fill(0);
    B.smap.assign(sz * nc, (int8_t) -1);
    const int8_t *ri = rot_inv(pRot);
    const unsigned rootM = morton_index(root, pLev);
    for (size_t i = 0; i < sz; i++) {
      unsigned base = (morton_index(coords[i], pLev) ^ rootM) | morton_index(coords[i], pLev + 1);
      unsigned po, pd, co, cd;
      cell_type(coords[i], pLev, po, pd);
      cell_type(coords[i], pLev + 1, co, cd);
      const unsigned dupO = po & ~co, dupD = pd - cd;
      base &= ~dupO;
      unsigned strides[dim];
      for (unsigned d = 0, k = 0; d < dim; d++) { strides[k] = 1u << d; k += (dupO >> d) & 1u; }
      for (unsigned j = 0; j < (1u << dupD); j++) {
        unsigned cm = base;
        for (unsigned k = 0; k < dupD; k++) cm += strides[k] * ((j >> k) & 1u);
        const int cs = ri[cm];
        B.smap[i * nc + j] = (int8_t) cs;
        counts[cs]++;
      }
    }
    size_t acc = 0;
    for (unsigned c = 0; c < nc; c++) { offsets[c] = acc; acc += counts[c]; }
    if (B.coords.size() < acc) B.coords.resize(acc);
    if (B.vin.size() < acc) B.vin.resize(acc);
    std::array<size_t, 16> w = offsets;
    for (size_t i = 0; i < sz; i++)
      for (unsigned j = 0; j < nc; j++) {
        int cs = B.smap[i * nc + j];
        if (cs < 0) break;
        B.coords[w[cs]] = coords[i];
        B.vin[w[cs]] = vec[i];
        w[cs]++;
      }
    return false;
  }

  void rec(const double *vin, double *vout, const TN<dim> *coords, const TN<dim> &root, int pRot, size_t sz,
           const double *pVin, double *pVout, const TN<dim> *pCoords, size_t pSz)
  {
    if (sz == 0) return;
    const unsigned pLev = root.lev, nc = 1u << dim;
    const unsigned nPe = ipow(p + 1, dim);
    if ((int64_t) pLev > st.max_depth_seen) st.max_depth_seen = pLev;
    std::array<size_t, 16> offset, counts;
    Buf &B = ibufs[pLev];
    const bool leaf = top_down(coords, vin, sz, offset, counts, B, root, pRot);
    if (!leaf) {
      // vec_out_contrib sized like vec_in_dup (matvec.h:320-321); it is a
      // separate vector per level, so deeper levels never alias it.
      std::vector<double> &contrib = B.vout;
      contrib.assign(B.vin.size(), 0.0);
      const int8_t *rp = rot_perm(pRot);
      const int32_t *ol = orient(pRot);
      bool before = is_ancestor(root, partFront);
      bool after = false;
      for (unsigned s = 0; s < nc; s++) {
        const int cm = rp[s];
        const int cRot = ol[cm];
        TN<dim> ch = child_morton(root, cm);
        before = before && !(tn_equal(ch, partFront) || is_ancestor(ch, partFront));
        if (!before && !after)
          rec(B.vin.data() + offset[s], contrib.data() + offset[s], B.coords.data() + offset[s], ch, cRot, counts[s],
              vin, vout, coords, sz);
        after = after || (tn_equal(ch, partBack) || is_ancestor(ch, partBack));
      }
      // bottom_up (matvec.h:202-216)
      std::array<size_t, 16> w = offset;
      for (size_t i = 0; i < sz; i++)
        for (unsigned j = 0; j < nc; j++) {
          int cs = B.smap[i * nc + j];
          if (cs < 0) break;
          vout[i] += contrib[w[cs]++];
        }
      return;
    }
    // Leaf (matvec.h:378-522)
    st.leaves++;
    std::fill(leafFill.begin(), leafFill.end(), 0);
    for (size_t i = 0; i < sz; i++) {
      unsigned r = lex_node_rank(coords[i], root, p);
      if (leafFill[r]) st.aliased++;
      leafFill[r] = 1;
      leafIn[r] = vin[i];
    }
    bool all = true;
    for (unsigned r = 0; r < nPe; r++) all = all && leafFill[r];
    if (!all) {
      st.hanging_leaves++;
      if (pVin == nullptr || pCoords == nullptr || pSz == 0) { fprintf(stderr, "oracle: parent has no nodes\n"); return; }
      TN<dim> par = get_parent(root);
      std::fill(parentFill.begin(), parentFill.end(), 0);
      if (g_stale_mode == 1) std::fill(parentBuf.begin(), parentBuf.end(), 0.0);
      for (size_t i = 0; i < pSz; i++) {
        if (g_conforming ? !on_lattice(pCoords[i], par, p) : pCoords[i].lev != pLev - 1) continue;
        unsigned r = lex_node_rank(pCoords[i], par, p);
        parentFill[r] = 1;
        parentBuf[r] = pVin[i];
      }
      // The reference's own consistency check (matvec.h:439-447): every rank
      // is filled in the leaf or in the parent buffer.
      for (unsigned r = 0; r < nPe; r++)
        if (!leafFill[r] && !parentFill[r]) { st.ref_errors++; break; }
      // Instrumentation: does any unfilled leaf rank read a stale parent slot
      // with nonzero weight?
      {
        const unsigned child = morton_index(root, root.lev);
        for (unsigned q = 0; q < nPe; q++) {
          if (parentFill[q]) continue;
          std::vector<double> e(nPe, 0.0), z(nPe);
          e[q] = 1.0;
          ikd_interp(dim, *re, e.data(), z.data(), child, false);
          for (unsigned r = 0; r < nPe; r++) if (!leafFill[r] && z[r] != 0.0) { st.stale_reads++; break; }
        }
      }
      ikd_interp(dim, *re, parentBuf.data(), parentBuf.data(), morton_index(root, root.lev), false);
      for (unsigned r = 0; r < nPe; r++) if (!leafFill[r]) leafIn[r] = parentBuf[r];
    }
    element_node_coords(root, p, coordBuf);
    ele_op(op, dim, *re, leafIn.data(), leafOut.data(), coordBuf.data(), 1.0);
    for (size_t i = 0; i < sz; i++) vout[i] = leafOut[lex_node_rank(coords[i], root, p)];
    if (!all) {
      for (unsigned r = 0; r < nPe; r++) if (leafFill[r]) leafOut[r] = 0.0;
      ikd_interp(dim, *re, leafOut.data(), leafOut.data(), morton_index(root, root.lev), true);
      TN<dim> par = get_parent(root);
      for (size_t i = 0; i < pSz; i++) {
        if (g_conforming ? !on_lattice(pCoords[i], par, p) : pCoords[i].lev != pLev - 1) continue;
        unsigned r = lex_node_rank(pCoords[i], par, p);
        if (g_conforming || !leafFill[r]) pVout[i] += leafOut[r];
      }
    }
  }

  void run(const double *vin, double *vout, const TN<dim> *coords, size_t sz)
  {
    const unsigned nPe = ipow(p + 1, dim);
    ibufs.resize(g_md + 2);
    parentBuf.resize(nPe); parentFill.resize(nPe); leafIn.resize(nPe); leafOut.resize(nPe); leafFill.resize(nPe);
    std::fill(vout, vout + sz, 0.0);
    TN<dim> root{}; root.lev = 0;
    rec(vin, vout, coords, root, 0, sz, nullptr, nullptr, nullptr, 0);
  }
};

// ---------------------------------------------------------------------------
// Handle that keeps a DA and its traversal state between calls, like the
// reference's DA object plus the function-static matvec buffers.
// ---------------------------------------------------------------------------
struct OracleDA {
  int dim = 3;
  unsigned p = 1;
  int op = 2;
  std::vector<uint32_t> treeC; std::vector<uint8_t> treeL;
  std::vector<uint32_t> nodeC; std::vector<uint8_t> nodeL;
  std::vector<uint32_t> bdry;
  RefEl re;
  void *trav = nullptr;
  MatvecStats stats;
};

template <int dim>
void da_construct(OracleDA &h)
{
  const size_t ne = h.treeL.size();
  std::vector<TN<dim>> tree(ne);
  for (size_t i = 0; i < ne; i++) { for (int d = 0; d < dim; d++) tree[i].x[d] = h.treeC[i * dim + d]; tree[i].lev = h.treeL[i]; }
  std::vector<TN<dim>> nodes;
  for (auto &e : tree) append_exterior_nodes(e, h.p, nodes);
  count_cg_nodes<dim>(nodes.data(), nodes.data() + nodes.size());
  std::vector<TN<dim>> sel;
  for (auto &t : nodes) if (t.sel == 2) sel.push_back(t);
  for (auto &e : tree) append_interior_nodes(e, h.p, sel);
  h.nodeC.resize(sel.size() * dim); h.nodeL.resize(sel.size()); h.bdry.clear();
  for (size_t i = 0; i < sel.size(); i++) {
    for (int d = 0; d < dim; d++) h.nodeC[i * dim + d] = sel[i].x[d];
    h.nodeL[i] = (uint8_t) sel[i].lev;
    if (on_domain_boundary(sel[i])) h.bdry.push_back((uint32_t) i);
  }
}

template <int dim>
void matvec_raw(OracleDA &h, const double *x, double *y)
{
  const size_t n = h.nodeL.size();
  std::vector<TN<dim>> nodes(n);
  for (size_t i = 0; i < n; i++) { for (int d = 0; d < dim; d++) nodes[i].x[d] = h.nodeC[i * dim + d]; nodes[i].lev = h.nodeL[i]; }
  Traversal<dim> *t = (Traversal<dim> *) h.trav;
  if (!t) { t = new Traversal<dim>(); h.trav = t; }
  t->p = h.p; t->op = h.op; t->re = &h.re;
  for (int d = 0; d < dim; d++) { t->partFront.x[d] = h.treeC[d]; t->partBack.x[d] = h.treeC[(h.treeL.size() - 1) * dim + d]; }
  t->partFront.lev = h.treeL.front(); t->partBack.lev = h.treeL.back();
  t->st = MatvecStats();
  t->run(x, y, nodes.data(), n);
  h.stats = t->st;
}

std::string g_err;

}  // namespace

// ===========================================================================
// C API (ctypes).  All functions return 0 on success, nonzero on error.
// ===========================================================================
extern "C" {

const char *dkto_last_error() { return g_err.c_str(); }

// Morton (rot == nullptr) or caller-supplied rotation tables.
int dkto_set_curve(int dim, int max_depth, const int8_t *rot, const int32_t *ht, int nrot)
{
  if (dim < 2 || dim > 4 || max_depth < 1 || max_depth > 30) { g_err = "bad dim/max_depth"; return 1; }
  g_md = (unsigned) max_depth;
  set_curve(dim, rot, ht, nrot);
  return 0;
}

// Points (level max_depth) -> 2:1-balanced tree (SFC_Tree::locTreeBalancing, maxPts).
// Two-phase: call with out == nullptr to get the count, then with buffers.
static std::vector<uint32_t> s_treeC;
static std::vector<uint8_t> s_treeL;
int dkto_tree_balance(int dim, const uint32_t *pts, int64_t n, int64_t max_pts, int64_t *n_out)
{
  s_treeC.clear(); s_treeL.clear();
  auto go = [&](auto tag) {
    constexpr int D = decltype(tag)::value;
    std::vector<TN<D>> v(n);
    for (int64_t i = 0; i < n; i++) v[i] = make_cell<D>(pts + i * D, g_md);
    auto t = loc_tree_balancing<D>(v, (size_t) max_pts);
    for (auto &e : t) { for (int d = 0; d < D; d++) s_treeC.push_back(e.x[d]); s_treeL.push_back((uint8_t) e.lev); }
  };
  if (dim == 2) go(std::integral_constant<int, 2>());
  else if (dim == 3) go(std::integral_constant<int, 3>());
  else if (dim == 4) go(std::integral_constant<int, 4>());
  else { g_err = "bad dim"; return 1; }
  *n_out = (int64_t) s_treeL.size();
  return 0;
}
// The benchmark's spacetime moving-ball mesh (dim 4: x, y, z, t), restated
// for the CPU side: every cell whose box meets the shell
// | |(x,y,z) - c(t)| - R | <= w, c(t) = c0 + (c1 - c0) t, is refined down to
// `level`, then the tree is 2:1 balanced with propagateNeighbours +
// reconstruction (src/tsort.cpp:777-854, as loc_tree_balancing).  For a cell
// [lo,hi]^3 x [t0,t1] the distance from c(t) to the spatial box is convex in t,
// so its minimum over [t0,t1] is found by golden-section search (80 steps);
// the largest distance is convex too and peaks at t0 or t1.  The cell meets
// the shell iff min-distance <= R + w and max-distance >= R - w.
// With part_level > 0 only the cell of Morton index part_index at level
// part_level is refined (the rest of the domain stays at the coarsest cells
// on the path to it before balancing): one partition of the mesh.
namespace {
double mb_box_dist(const double *lo, const double *hi, const double *c)
{
  double s = 0.0;
  for (int d = 0; d < 3; d++) {
    const double g = c[d] < lo[d] ? lo[d] - c[d] : (c[d] > hi[d] ? c[d] - hi[d] : 0.0);
    s += g * g;
  }
  return std::sqrt(s);
}
double mb_box_far(const double *lo, const double *hi, const double *c)
{
  double s = 0.0;
  for (int d = 0; d < 3; d++) {
    const double f = std::max(std::fabs(c[d] - lo[d]), std::fabs(hi[d] - c[d]));
    s += f * f;
  }
  return std::sqrt(s);
}
bool mb_meets(const TN<4> &c, double R, double w, const double *c0, const double *c1)
{
  const double s = std::ldexp(1.0, -(int) g_md), h = std::ldexp(1.0, -(int) c.lev);
  double lo[3], hi[3];
  for (int d = 0; d < 3; d++) { lo[d] = c.x[d] * s; hi[d] = lo[d] + h; }
  const double t0 = c.x[3] * s, t1 = t0 + h;
  auto centre = [&](double t, double *out) { for (int d = 0; d < 3; d++) out[d] = c0[d] + (c1[d] - c0[d]) * t; };
  double ca[3], cb[3];
  centre(t0, ca);
  centre(t1, cb);
  const double dmax = std::max(mb_box_far(lo, hi, ca), mb_box_far(lo, hi, cb));
  double a = t0, b = t1;
  const double gr = 0.5 * (std::sqrt(5.0) - 1.0);
  for (int it = 0; it < 80; it++) {
    const double m1 = b - gr * (b - a), m2 = a + gr * (b - a);
    double p1[3], p2[3];
    centre(m1, p1);
    centre(m2, p2);
    if (mb_box_dist(lo, hi, p1) <= mb_box_dist(lo, hi, p2)) b = m2; else a = m1;
  }
  double pm[3];
  centre(0.5 * (a + b), pm);
  const double dmin = std::min({mb_box_dist(lo, hi, pm), mb_box_dist(lo, hi, ca), mb_box_dist(lo, hi, cb)});
  return dmin <= R + w && dmax >= R - w;
}
void mb_refine(const TN<4> &c, unsigned level, double R, double w, const double *c0, const double *c1,
               unsigned part_level, const TN<4> &part, std::vector<TN<4>> &leaves)
{
  // inside the partition cell (or on the path of cells down to it): the
  // cell and the partition cell agree on their common levels
  const unsigned common = std::min(c.lev, part_level);
  bool inside = true;
  for (int d = 0; d < 4; d++)
    if ((part.x[d] >> (g_md - common)) != (c.x[d] >> (g_md - common))) inside = false;
  const bool split = inside && (c.lev < part_level || (c.lev < level && mb_meets(c, R, w, c0, c1)));
  if (!split) { leaves.push_back(c); return; }
  for (int ch = 0; ch < 16; ch++) {
    TN<4> k = c;
    k.lev = c.lev + 1;
    const uint32_t cl = 1u << (g_md - k.lev);
    for (int d = 0; d < 4; d++) k.x[d] = c.x[d] | (((ch >> d) & 1) ? cl : 0u);
    mb_refine(k, level, R, w, c0, c1, part_level, part, leaves);
  }
}
}  // namespace

int dkto_moving_ball(int level, double R, double w, const double *c0, const double *c1, int part_level,
                     int64_t part_index, int64_t *n_out)
{
  if (level < 1 || level > (int) g_md || part_level < 0 || part_level > level) { g_err = "bad level"; return 1; }
  s_treeC.clear(); s_treeL.clear();
  TN<4> part{};
  part.lev = (uint32_t) part_level;
  for (int l = 0; l < part_level; l++) {
    const int64_t digit = (part_index >> (4 * (part_level - 1 - l))) & 15;
    for (int d = 0; d < 4; d++)
      if ((digit >> d) & 1) part.x[d] |= 1u << (g_md - 1 - l);
  }
  TN<4> root{};
  root.lev = 0;
  std::vector<TN<4>> leaves, nt;
  mb_refine(root, (unsigned) level, R, w, c0, c1, (unsigned) part_level, part, leaves);
  propagate_neighbours(leaves);
  loc_tree_construction<4>(leaves.data(), nt, 1, 0, leaves.size(), 1, g_md, 0, root);
  for (auto &e : nt) { for (int d = 0; d < 4; d++) s_treeC.push_back(e.x[d]); s_treeL.push_back((uint8_t) e.lev); }
  *n_out = (int64_t) s_treeL.size();
  return 0;
}

int dkto_tree_fetch(uint32_t *coords, uint8_t *levels)
{
  std::copy(s_treeC.begin(), s_treeC.end(), coords);
  std::copy(s_treeL.begin(), s_treeL.end(), levels);
  return 0;
}

// SFC_Tree::locTreeSort over cells (in place).
int dkto_tree_sort(int dim, uint32_t *coords, uint8_t *levels, int64_t n)
{
  auto go = [&](auto tag) {
    constexpr int D = decltype(tag)::value;
    std::vector<TN<D>> v(n);
    for (int64_t i = 0; i < n; i++) { for (int d = 0; d < D; d++) v[i].x[d] = coords[i * D + d]; v[i].lev = levels[i]; }
    loc_tree_sort<D>(v.data(), 0, v.size(), 1, g_md, 0);
    for (int64_t i = 0; i < n; i++) { for (int d = 0; d < D; d++) coords[i * D + d] = v[i].x[d]; levels[i] = (uint8_t) v[i].lev; }
  };
  if (dim == 2) go(std::integral_constant<int, 2>());
  else if (dim == 3) go(std::integral_constant<int, 3>());
  else if (dim == 4) go(std::integral_constant<int, 4>());
  else { g_err = "bad dim"; return 1; }
  return 0;
}

// ot::DA construction from a sorted, balanced tree.
int dkto_da_create(int dim, int order, int op, const uint32_t *coords, const uint8_t *levels, int64_t n, void **out)
{
  if (order < 1 || order > 2) { g_err = "oracle supports order 1 and 2 (low-order resolver)"; return 1; }
  if (n <= 0) { g_err = "empty tree"; return 1; }
  OracleDA *h = new OracleDA();
  h->dim = dim; h->p = (unsigned) order; h->op = op;
  h->treeC.assign(coords, coords + n * dim);
  h->treeL.assign(levels, levels + n);
  h->re = make_refel((unsigned) order);
  if (dim == 2) da_construct<2>(*h);
  else if (dim == 3) da_construct<3>(*h);
  else if (dim == 4) da_construct<4>(*h);
  else { delete h; g_err = "bad dim"; return 1; }
  *out = h;
  return 0;
}
int64_t dkto_da_num_nodes(void *hp) { return (int64_t) ((OracleDA *) hp)->nodeL.size(); }
int64_t dkto_da_num_bdry(void *hp) { return (int64_t) ((OracleDA *) hp)->bdry.size(); }
int dkto_da_nodes(void *hp, uint32_t *coords, uint8_t *levels, uint32_t *bdry)
{
  OracleDA *h = (OracleDA *) hp;
  std::copy(h->nodeC.begin(), h->nodeC.end(), coords);
  std::copy(h->nodeL.begin(), h->nodeL.end(), levels);
  if (bdry) std::copy(h->bdry.begin(), h->bdry.end(), bdry);
  return 0;
}
int dkto_da_refel(void *hp, double *ip0, double *ip1, double *Q, double *D, double *W)
{
  OracleDA *h = (OracleDA *) hp;
  std::copy(h->re.ip0.begin(), h->re.ip0.end(), ip0);
  std::copy(h->re.ip1.begin(), h->re.ip1.end(), ip1);
  std::copy(h->re.Q.begin(), h->re.Q.end(), Q);
  std::copy(h->re.D.begin(), h->re.D.end(), D);
  std::copy(h->re.W.begin(), h->re.W.end(), W);
  return 0;
}
void dkto_da_destroy(void *hp)
{
  OracleDA *h = (OracleDA *) hp;
  if (!h) return;
  if (h->trav) {
    if (h->dim == 2) delete (Traversal<2> *) h->trav;
    else if (h->dim == 3) delete (Traversal<3> *) h->trav;
    else delete (Traversal<4> *) h->trav;
  }
  delete h;
}

// fem::matvec over the DA's node list (no boundary handling).
int dkto_matvec_raw(void *hp, const double *x, double *y)
{
  OracleDA *h = (OracleDA *) hp;
  if (h->dim == 2) matvec_raw<2>(*h, x, y);
  else if (h->dim == 3) matvec_raw<3>(*h, x, y);
  else matvec_raw<4>(*h, x, y);
  return 0;
}

// feMatrix::matVec (FEM/include/feMatrix.h:189-259): operators 1 and 2 zero
// the boundary entries of the input before and of the output after
// (heatMat.cpp:119-139); the identity operator has no pre/post step.
int dkto_fematrix_matvec(void *hp, const double *x, double *y)
{
  OracleDA *h = (OracleDA *) hp;
  const size_t n = h->nodeL.size();
  std::vector<double> xin(x, x + n);
  const bool bc = (h->op == 1 || h->op == 2 || h->op == 4 || h->op == 6);
  if (bc) for (uint32_t b : h->bdry) xin[b] = 0.0;
  dkto_matvec_raw(hp, xin.data(), y);
  if (bc) for (uint32_t b : h->bdry) y[b] = 0.0;
  return 0;
}

// Counters from the last traversal: leaves, hanging leaves, stale parent
// slots read with nonzero weight, aliased leaf ranks, deepest level.
int dkto_last_stats(void *hp, int64_t *out6)
{
  OracleDA *h = (OracleDA *) hp;
  out6[0] = h->stats.leaves; out6[1] = h->stats.hanging_leaves; out6[2] = h->stats.stale_reads;
  out6[3] = h->stats.aliased; out6[4] = h->stats.max_depth_seen; out6[5] = h->stats.ref_errors;
  return 0;
}

// Select how unfilled parent-buffer slots are read (see g_stale_mode).
int dkto_set_stale_mode(int mode) { g_stale_mode = mode; return 0; }

// Select the reference traversal (0) or its conforming variant (1).
int dkto_set_conforming(int on) { g_conforming = on; return 0; }

// Unpreconditioned or Jacobi-preconditioned CG in the form of
// HeatMat::cgSolve (FEM/examples/src/heatMat.cpp:164-325), stopping on
// ||r||_2 / ||b||_2 <= tol.  diag == nullptr: unpreconditioned.
int dkto_cg(void *hp, const double *b, double *x, const double *diag, int max_iter, double tol, int *iters, double *relres)
{
  OracleDA *h = (OracleDA *) hp;
  const size_t n = h->nodeL.size();
  std::vector<double> r(n), z(n), p(n), Ap(n), Ax(n);
  auto dot = [&](const std::vector<double> &a, const std::vector<double> &c) { long double s = 0; for (size_t i = 0; i < n; i++) s += (long double) a[i] * c[i]; return (double) s; };
  dkto_fematrix_matvec(hp, x, Ax.data());
  double nb = 0; for (size_t i = 0; i < n; i++) nb += b[i] * b[i];
  nb = std::sqrt(nb); if (nb == 0) nb = 1;
  for (size_t i = 0; i < n; i++) r[i] = b[i] - Ax[i];
  auto prec = [&]() { for (size_t i = 0; i < n; i++) z[i] = diag ? (diag[i] != 0 ? r[i] / diag[i] : r[i]) : r[i]; };
  prec();
  p = z;
  double rz = dot(r, z);
  int it = 0;
  double res = std::sqrt(dot(r, r)) / nb;
  while (res > tol && it < max_iter) {
    dkto_fematrix_matvec(hp, p.data(), Ap.data());
    const double alpha = rz / dot(p, Ap);
    for (size_t i = 0; i < n; i++) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
    res = std::sqrt(dot(r, r)) / nb;
    it++;
    if (res <= tol) break;
    prec();
    const double rz2 = dot(r, z);
    const double beta = rz2 / rz;
    rz = rz2;
    for (size_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
  }
  *iters = it; *relres = res;
  return 0;
}

// HeatMat::cgSolve itself (FEM/examples/src/heatMat.cpp:164-325): no
// preconditioner, alpha = <r0,r0>/<p,Ap>, beta = <r1,r1>/<r0,r0>, stopping
// when ||r||_inf / ||b||_inf <= tol (||b||_inf = 0 counts as 1); dots are plain
// sums in index order (include/mathUtils.tcc:205-212) and the L-infinity norm
// is NaN if any entry is NaN (include/mathUtils.tcc:69-80).  iters = the
// iteration at which it stopped (0 when the initial guess already meets tol,
// max_iter when it did not converge); resid = the last relative residual;
// status 0 on convergence, 1 otherwise.
int dkto_cg_ref(void *hp, const double *b, double *x, int max_iter, double tol, int *iters, double *resid,
                int *status)
{
  OracleDA *h = (OracleDA *) hp;
  const size_t n = h->nodeL.size();
  std::vector<double> p(n), Ax(n), Ap(n), r0(n), r1(n);
  auto dot = [&](const std::vector<double> &a, const std::vector<double> &c) {
    double s = 0.0;
    for (size_t i = 0; i < n; i++) s += a[i] * c[i];
    return s;
  };
  auto linf = [&](const double *v) {
    if (n == 0) return 0.0;
    if (std::isnan(v[0])) return (double) NAN;
    double m = std::fabs(v[0]);
    for (size_t i = 1; i < n; i++) {
      if (std::isnan(v[i])) return (double) NAN;
      if (m < std::fabs(v[i])) m = std::fabs(v[i]);
    }
    return m;
  };
  double normb = linf(b);
  dkto_fematrix_matvec(hp, x, Ax.data());
  for (size_t i = 0; i < n; i++) { r0[i] = b[i] - Ax[i]; p[i] = r0[i]; }
  if (normb == 0.0) normb = 1;
  double res = linf(r0.data()) / normb;
  *iters = 0;
  *status = 1;
  if (res <= tol) { *resid = res; *status = 0; return 0; }
  for (int i = 1; i <= max_iter; i++) {
    dkto_fematrix_matvec(hp, p.data(), Ap.data());
    const double alpha = dot(r0, r0) / dot(p, Ap);
    for (size_t e = 0; e < n; e++) { x[e] += alpha * p[e]; r1[e] = r0[e] - alpha * Ap[e]; }
    res = linf(r1.data()) / normb;
    *iters = i;
    if (res <= tol) { *status = 0; break; }
    const double beta = dot(r1, r1) / dot(r0, r0);
    for (size_t e = 0; e < n; e++) { p[e] = r1[e] + beta * p[e]; r0[e] = r1[e]; }
  }
  *resid = res;
  return 0;
}

}  // extern "C"
