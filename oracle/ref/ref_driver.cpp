// Reference-side driver for the CPU oracle.
//
// Test infrastructure only.  Compiled (by oracle/ref/Makefile) against the
// unmodified Dendro-KT sources, a single-rank MPI stand-in and two LAPACK
// routines; writes everything the parity tests pin:
//   * the balanced tree      SFC_Tree::locTreeBalancing   (src/tsort.cpp:826-854),
//     or (input kind 3) the tree of ot::DA<dim>::DA(func, ...) (include/oda.tcc:67-88):
//     function2Octree (include/octUtils.h:180-417) of the two test fields
//     below, then distTreeBalancing with one point per region
//   * the DA node list       ot::DA::construct            (src/oda.cpp:52-151)
//   * boundary node ids      (src/oda.cpp:145-150)
//   * feMatrix::matVec output (FEM/include/feMatrix.h:189-259) for
//       op 0: identity eleOp as in test/testMatvec.cpp:187-198
//       op 1: HeatEq::HeatMat<dim> (FEM/examples/src/heatMat.cpp:45-139)
//       op 2: Laplacian + mass, a restatement built from the reference's
//             RefElement 1D operators (the reference has no valid 4D operator)
//       op 6: feVector::computeVec (FEM/include/feVector.h:122-168) of
//             HeatEq::HeatVec<dim> (FEM/examples/src/heatVec.cpp:30-104), the
//             mass right-hand side with boundary zeroing; a 3D operator
//   * the raw fem::matvec output (FEM/include/matvec.h:231-240), no pre/post
//   * the RefElement 1D matrices (FEM/src/refel.cpp:75-220)
//   * op 8 (dim 3): io::vtk::oct2vtu (IO/vtk/src/oct2vtk.cpp:1570-1760) of the
//     tree in SFC order, written beside the output file as <out>_vtu_0_1.vtu;
//     the matVec outputs are the identity's (as op 0)
//   * op 7: HeatEq::HeatMat<dim>::cgSolve (FEM/examples/src/heatMat.cpp:164-325)
//     from x = 0 on b = the HeatVec<dim> right-hand side of the input vector
//     (feVector::computeVec, as FEM/examples/src/heatEq.cpp:112-118 builds
//     it), with the tolerance and iteration cap of the input; the matVec
//     outputs are HeatMat's (as op 1)
//
// The binary formats are the ones tests/golden/refio.py writes and reads.
#include <mpi.h>
#include "treeNode.h"
#include "tsort.h"
#include "nsort.h"
#include "oda.h"
#include "hcurvedata.h"
#include "feMatrix.h"
#include "matvec.h"
#include "refel.h"
#include "heatMat.h"
#include "heatVec.h"
#include "oct2vtk.h"

#include <chrono>
#include <iostream>
#include <sstream>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <functional>
#include <vector>
#include <string>
#include <cmath>

namespace {

// Counter-based uniform in [-1,1): the same function the product, the port
// oracle and the tests use to make nodal vectors from a seed.
inline uint64_t splitmix64(uint64_t z)
{
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline double uniform_pm1(uint64_t seed, uint64_t i)
{
  uint64_t r = splitmix64(seed * 0xD1B54A32D192ED03ull + i);
  return 2.0 * ((double) (r >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
}

struct Reader {
  FILE *f;
  template <typename X> X get() { X x; if (fread(&x, sizeof(X), 1, f) != 1) { fprintf(stderr, "short read\n"); exit(2); } return x; }
  template <typename X> void arr(X *p, size_t n) { if (n && fread(p, sizeof(X), n, f) != n) { fprintf(stderr, "short read\n"); exit(2); } }
};
struct Writer {
  FILE *f;
  template <typename X> void put(X x) { fwrite(&x, sizeof(X), 1, f); }
  template <typename X> void arr(const X *p, size_t n) { if (n) fwrite(p, sizeof(X), n, f); }
};

// Identity eleOp (test/testMatvec.cpp:187-198).
template <unsigned int dim>
class IdentityMat : public feMatrix<IdentityMat<dim>, dim> {
 public:
  using feMatrix<IdentityMat<dim>, dim>::feMatrix;
  void elementalMatVec(const VECType *in, VECType *out, double *, double) override
  {
    const RefElement *refEl = feMat<dim>::m_uiOctDA->getReferenceElement();
    const unsigned int nPe = intPow(refEl->getOrder() + 1, dim);
    for (unsigned int i = 0; i < nPe; i++) out[i] = in[i];
  }
};

// y[..j..] = sum_k A[k*M+j] x[..k..] along `axis` (axis 0 varies fastest), the
// convention of DENDRO_TENSOR_IIAX_APPLY_ELEM (FEM/src/tensor.cpp:44-60).
template <unsigned int dim>
void apply_axis(unsigned M, const double *A, const double *x, double *y, unsigned axis)
{
  unsigned stride = 1;
  for (unsigned a = 0; a < axis; a++) stride *= M;
  unsigned n = 1;
  for (unsigned a = 0; a < dim; a++) n *= M;
  for (unsigned idx = 0; idx < n; idx++) {
    unsigned j = (idx / stride) % M;
    unsigned base = idx - j * stride;
    double s = 0.0;
    for (unsigned k = 0; k < M; k++) s += A[k * M + j] * x[base + k * stride];
    y[idx] = s;
  }
}

// Laplacian + mass on a cube element of side h, J = h/2:
//   K_e = J^(d-2) sum_a (Dg^T W Dg)_a (x) (Q^T W Q)_others  +  J^d (Q^T W Q)^(x)d
// using the reference's Gauss quadrature 1D operators (RefElement::getQ1d,
// getDg1d, getWgq), with HeatMat's boundary conditions (heatMat.cpp:119-139).
template <unsigned int dim>
class LapMassMat : public feMatrix<LapMassMat<dim>, dim> {
 public:
  using feMatrix<LapMassMat<dim>, dim>::feMatrix;
  void elementalMatVec(const VECType *in, VECType *out, double *coords, double scale) override
  {
    const RefElement *refEl = feMat<dim>::m_uiOctDA->getReferenceElement();
    const unsigned p = refEl->getOrder(), M = p + 1;
    const unsigned nPe = intPow(M, dim);
    const double *Q = refEl->getQ1d(), *QT = refEl->getQT1d();
    const double *D = refEl->getDg1d(), *DT = refEl->getDgT1d();
    const double *W = refEl->getWgq();
    const double h = coords[(nPe - 1) * dim + 0] - coords[0];
    const double J = 0.5 * h;
    double Jdm2 = 1.0, Jd = 1.0;
    for (unsigned a = 0; a + 2 < dim; a++) Jdm2 *= J;
    for (unsigned a = 0; a < dim; a++) Jd *= J;
    if (dim < 2) Jdm2 = 1.0 / J;
    std::vector<double> a(nPe), b(nPe), acc(nPe, 0.0), wq(nPe);
    for (unsigned idx = 0; idx < nPe; idx++) {
      double w = 1.0; unsigned r = idx;
      for (unsigned d = 0; d < dim; d++) { w *= W[r % M]; r /= M; }
      wq[idx] = w;
    }
    for (int term = -1; term < (int) dim; term++) {
      std::copy(in, in + nPe, a.begin());
      for (unsigned d = 0; d < dim; d++) {
        apply_axis<dim>(M, ((int) d == term) ? D : Q, a.data(), b.data(), d);
        std::swap(a, b);
      }
      for (unsigned idx = 0; idx < nPe; idx++) a[idx] *= wq[idx];
      for (unsigned d = 0; d < dim; d++) {
        apply_axis<dim>(M, ((int) d == term) ? DT : QT, a.data(), b.data(), d);
        std::swap(a, b);
      }
      const double f = (term < 0) ? Jd : Jdm2;
      for (unsigned idx = 0; idx < nPe; idx++) acc[idx] += f * a[idx];
    }
    for (unsigned idx = 0; idx < nPe; idx++) out[idx] = scale * acc[idx];
  }
  bool preMatVec(const VECType *, VECType *out, double)
  {
    std::vector<unsigned int> bdy;
    feMat<dim>::m_uiOctDA->getBoundaryNodeIndices(bdy);
    for (unsigned int i : bdy) out[i] = 0.0;
    return true;
  }
  bool postMatVec(const VECType *, VECType *out, double)
  {
    std::vector<unsigned int> bdy;
    feMat<dim>::m_uiOctDA->getBoundaryNodeIndices(bdy);
    for (unsigned int i : bdy) out[i] = 0.0;
    return true;
  }
};

// The two test fields of input kind 3: 1 / (eps + |x - c|^2), summed left to
// right so that other implementations reproduce the values bit for bit.
void test_fields(const double *x, double *out, unsigned dim)
{
  static const double c0[4] = {0.3, 0.6, 0.45, 0.5}, c1[4] = {0.7, 0.25, 0.55, 0.4};
  double s0 = 0.01, s1 = 0.02;
  for (unsigned d = 0; d < dim; d++) {
    const double a = x[d] - c0[d], b = x[d] - c1[d];
    s0 = s0 + a * a;
    s1 = s1 + b * b;
  }
  out[0] = 1.0 / s0;
  out[1] = 1.0 / s1;
}

// io::vtk::oct2vtu is defined for dim 3 only (IO/vtk/src/oct2vtk.cpp:1892)
template <unsigned int dim>
void write_oct_vtu(const std::vector<ot::TreeNode<unsigned int, dim>> &, const char *)
{
}
template <>
void write_oct_vtu<3>(const std::vector<ot::TreeNode<unsigned int, 3>> &tree, const char *prefix)
{
  io::vtk::oct2vtu<unsigned int, 3>(tree.data(), (unsigned int) tree.size(), prefix, MPI_COMM_WORLD);
}

double now_s()
{
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

template <unsigned int dim>
int run(Reader &in, Writer &out, int maxDepth, int order, int op, int inputKind, int nCalls, uint64_t seed,
        const char *outPath)
{
  using TN = ot::TreeNode<unsigned int, dim>;
  m_uiMaxDepth = maxDepth;
  _InitializeHcurve(dim);

  const uint64_t n = in.get<uint64_t>();
  std::vector<unsigned int> c(n * dim);
  std::vector<uint8_t> lev(n, (uint8_t) maxDepth);
  in.arr(c.data(), c.size());
  if (inputKind != 0) in.arr(lev.data(), lev.size());
  const uint64_t nxIn = in.get<uint64_t>();
  std::vector<double> xIn(nxIn);
  in.arr(xIn.data(), nxIn);
  const double interpTol = inputKind == 3 ? in.get<double>() : 0.0;
  // op 7: the cgSolve tolerance and iteration cap
  const double cgTol = op == 7 ? in.get<double>() : 0.0;
  const int cgMaxIter = op == 7 ? in.get<int32_t>() : 0;

  std::vector<TN> tree;
  double t0 = now_s();
  if (inputKind == 3) {
    std::function<void(const double *, double *)> fx = [](const double *x, double *o) { test_fields(x, o, dim); };
    const unsigned varIndex[2] = {0, 1};
    std::vector<TN> complete;
    ot::function2Octree<unsigned int, dim>(fx, 2, varIndex, 2, complete, maxDepth, interpTol, 0.3, order,
                                           MPI_COMM_WORLD);
    ot::SFC_Tree<unsigned int, dim>::distTreeBalancing(complete, tree, 1, 0.3, MPI_COMM_WORLD);
  } else if (inputKind == 0) {
    std::vector<TN> pts;
    pts.reserve(n);
    for (uint64_t i = 0; i < n; i++) {
      std::array<unsigned int, dim> a;
      for (unsigned d = 0; d < dim; d++) a[d] = c[i * dim + d];
      pts.push_back(TN(a, maxDepth));
    }
    ot::SFC_Tree<unsigned int, dim>::locTreeBalancing(pts, tree, 1);
  } else {
    for (uint64_t i = 0; i < n; i++) {
      std::array<unsigned int, dim> a;
      for (unsigned d = 0; d < dim; d++) a[d] = c[i * dim + d];
      tree.push_back(TN(a, lev[i]));
    }
    if (inputKind == 2)
      ot::SFC_Tree<unsigned int, dim>::locTreeSort(tree.data(), 0, (ot::RankI) tree.size(), 1, maxDepth, 0);
  }
  double t1 = now_s();

  ot::DA<dim> *da = new ot::DA<dim>(tree.data(), (unsigned int) tree.size(), MPI_COMM_WORLD, order);
  double t2 = now_s();

  const unsigned nLocal = da->getLocalNodalSz();
  const unsigned nTotal = da->getTotalNodalSz();
  const TN *nodes = da->getTNCoords() + da->getLocalNodeBegin();
  std::vector<unsigned int> bdy;
  da->getBoundaryNodeIndices(bdy);

  std::vector<double> x(nLocal), y(nLocal, 0.0), yraw(nTotal, 0.0);
  if (nxIn == nLocal) x = xIn;
  else for (unsigned i = 0; i < nLocal; i++) x[i] = uniform_pm1(seed, i);

  std::function<void(const double *, double *)> mv;
  IdentityMat<dim> idm(da, 1);
  HeatEq::HeatMat<dim> heat(da, 1);
  LapMassMat<dim> lm(da, 1);
  HeatEq::HeatVec<dim> hv(da, 1);
  std::array<double, dim> lo, hi;
  lo.fill(0.0);
  hi.fill(1.0);
  Point<dim> pmin(lo), pmax(hi);   // problem domain [0,1]^dim
  heat.setProblemDimensions(pmin, pmax);
  lm.setProblemDimensions(pmin, pmax);
  hv.setProblemDimensions(pmin, pmax);
  if (op == 0 || op == 8) mv = [&](const double *a, double *b) { idm.matVec(a, b, 1.0); };
  else if (op == 1 || op == 7) mv = [&](const double *a, double *b) { heat.matVec(a, b, 1.0); };
  else if (op == 6) mv = [&](const double *a, double *b) { hv.computeVec(a, b, 1.0); };
  else mv = [&](const double *a, double *b) { lm.matVec(a, b, 1.0); };

  std::vector<double> times;
  for (int k = 0; k < std::max(nCalls, 1); k++) {
    double ta = now_s();
    mv(x.data(), y.data());
    times.push_back(now_s() - ta);
  }
  std::sort(times.begin(), times.end());
  const double tMed = times[times.size() / 2];

  // Raw traversal, no boundary zeroing, on the ghosted layout (1 rank: identity).
  {
    std::vector<double> xg(nTotal, 0.0);
    std::copy(x.begin(), x.end(), xg.begin() + da->getLocalNodeBegin());
    using namespace std::placeholders;
    fem::EleOpT<double> eop;
    if (op == 0 || op == 8) eop = std::bind(&IdentityMat<dim>::elementalMatVec, &idm, _1, _2, _3, _4);
    else if (op == 1 || op == 7) eop = std::bind(&HeatEq::HeatMat<dim>::elementalMatVec, &heat, _1, _2, _3, _4);
    else if (op == 6) eop = std::bind(&HeatEq::HeatVec<dim>::elementalComputeVec, &hv, _1, _2, _3, _4);
    else eop = std::bind(&LapMassMat<dim>::elementalMatVec, &lm, _1, _2, _3, _4);
    fem::matvec(xg.data(), yraw.data(), da->getTNCoords(), nTotal, *da->getTreePartFront(), *da->getTreePartBack(),
                eop, 1.0, da->getReferenceElement());
  }

  out.put<char>('D'); out.put<char>('K'); out.put<char>('T'); out.put<char>('O');
  out.put<uint64_t>(tree.size());
  for (const TN &t : tree) for (unsigned d = 0; d < dim; d++) out.put<uint32_t>(t.getX(d));
  for (const TN &t : tree) out.put<uint8_t>((uint8_t) t.getLevel());
  out.put<uint64_t>(nLocal);
  for (unsigned i = 0; i < nLocal; i++) for (unsigned d = 0; d < dim; d++) out.put<uint32_t>(nodes[i].getX(d));
  for (unsigned i = 0; i < nLocal; i++) out.put<uint8_t>((uint8_t) nodes[i].getLevel());
  out.put<uint64_t>(bdy.size());
  for (unsigned i : bdy) out.put<uint32_t>(i);
  out.put<uint64_t>(nLocal); out.arr(x.data(), nLocal);
  out.put<uint64_t>(nLocal); out.arr(y.data(), nLocal);
  out.put<uint64_t>(nTotal); out.arr(yraw.data(), nTotal);
  out.put<double>(t1 - t0); out.put<double>(t2 - t1); out.put<double>(tMed);
  const RefElement *re = da->getReferenceElement();
  const int M = order + 1;
  out.put<int32_t>(M);
  out.arr(re->getIMChild0(), M * M);
  out.arr(re->getIMChild1(), M * M);
  out.arr(re->getQ1d(), M * M);
  out.arr(re->getDg1d(), M * M);
  out.arr(re->getWgq(), M);
  if (op == 8) write_oct_vtu<dim>(tree, (std::string(outPath) + "_vtu").c_str());
  if (op == 7) {
    // b = HeatVec right-hand side of x; x0 = 0; cgSolve writes its final
    // relative L-infinity residual into tol and prints the iteration at
    // which it stopped, which is read back from its output
    std::vector<double> rhs(nLocal, 0.0), sol(nLocal, 0.0);
    hv.computeVec(x.data(), rhs.data(), 1.0);
    double tol = cgTol;
    std::ostringstream log;
    std::streambuf *saved = std::cout.rdbuf(log.rdbuf());
    const int status = heat.cgSolve(sol.data(), rhs.data(), cgMaxIter, tol);
    std::cout.rdbuf(saved);
    int iters = 0;
    std::istringstream lines(log.str());
    std::string line;
    while (std::getline(lines, line)) {
      int k = 0;
      if (std::sscanf(line.c_str(), " iteration : %d", &k) == 1) iters = k;
    }
    if (status != 0) iters = cgMaxIter;
    out.put<int32_t>(status);
    out.put<double>(tol);
    out.put<int32_t>(iters);
    out.put<uint64_t>(nLocal); out.arr(rhs.data(), nLocal);
    out.put<uint64_t>(nLocal); out.arr(sol.data(), nLocal);
  }
  delete da;
  return 0;
}

}  // namespace

int main(int argc, char **argv)
{
  if (argc != 3) { fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]); return 1; }
  MPI_Init(&argc, &argv);
  FILE *fi = fopen(argv[1], "rb");
  FILE *fo = fopen(argv[2], "wb");
  if (!fi || !fo) { fprintf(stderr, "cannot open files\n"); return 1; }
  Reader in{fi};
  Writer out{fo};
  char magic[4];
  in.arr(magic, 4);
  if (std::memcmp(magic, "DKTI", 4) != 0) { fprintf(stderr, "bad magic\n"); return 1; }
  const int dim = in.get<int32_t>(), maxDepth = in.get<int32_t>(), order = in.get<int32_t>();
  const int op = in.get<int32_t>(), inputKind = in.get<int32_t>(), nCalls = in.get<int32_t>();
  const uint64_t seed = in.get<uint64_t>();
  int rc = 1;
  if (dim == 2) rc = run<2>(in, out, maxDepth, order, op, inputKind, nCalls, seed, argv[2]);
  else if (dim == 3) rc = run<3>(in, out, maxDepth, order, op, inputKind, nCalls, seed, argv[2]);
  else if (dim == 4) rc = run<4>(in, out, maxDepth, order, op, inputKind, nCalls, seed, argv[2]);
  fclose(fi);
  fclose(fo);
  MPI_Finalize();
  return rc;
}
