/* feMatrixGpu: the reference-side binding of the GB300 matvec path.
 *
 * A maintainer of Dendro-KT adds this header to FEM/include/ of the
 * reference tree.  It is a subclass of the operator whose product it
 * replaces (e.g. HeatEq::HeatMat<3>, FEM/examples/include/heatMat.h), so the
 * ot::DA / feMatrix API stays as it is:
 *   - matVec (feMatrix::matVec, FEM/include/feMatrix.h:189-259) goes through
 *     dkt_fematrix_matvec_host on a device plan built once per DA;
 *   - cgSolve (HeatMat::cgSolve, FEM/examples/src/heatMat.cpp:164-325, same
 *     signature and return convention) goes through dkt_cg_solve_host with
 *     DKT_CG_REFERENCE: the same iteration, stopping rule and results.
 * Every other member (elementalMatVec, setProblemDimensions, pre/postMatVec,
 * the PETSc shell of FEM/include/feMat.h:84-103) is the operator's own.
 * The DA's node order, levels and boundary ids equal the reference DA's, so
 * vectors made by ot::DA::createVector are passed through unchanged.
 *
 * Needs the reference's headers on the include path (feMatrix.h and the
 * operator's header) and this directory; link with
 * -L dendro-kt_gb300/_build -ldkt_gb300 -lcudart.
 *
 *   HeatEq::HeatMat<3> A(da, 1);                                    // before
 *   feMatrixGpu<HeatEq::HeatMat<3>, 3> A(da, tree, DKT_OP_HEAT);     // after
 */
#ifndef DKT_FEMATRIX_GPU_H
#define DKT_FEMATRIX_GPU_H

#include <stdexcept>
#include <vector>
#include "feMatrix.h"
#include "dkt_gb300.h"

/* Op: the feMatrix subclass whose product is replaced; op: the matching
 * built-in operator (DKT_OP_HEAT for HeatMat<3>, DKT_OP_LAPMASS, ...). */
template <typename Op, unsigned int dim>
class feMatrixGpu : public Op {
  dkt_da da_ = nullptr;
  dkt_plan plan_ = nullptr;

 public:
  /* tree: the complete, 2:1-balanced tree the DA was built from */
  feMatrixGpu(ot::DA<dim> *da, const std::vector<ot::TreeNode<unsigned, dim>> &tree, int op) : Op(da, 1)
  {
    std::vector<uint32_t> c(tree.size() * dim);
    std::vector<uint8_t> l(tree.size());
    for (size_t i = 0; i < tree.size(); i++) {
      for (unsigned d = 0; d < dim; d++) c[i * dim + d] = tree[i].getX(d);
      l[i] = (uint8_t) tree[i].getLevel();
    }
#ifdef HILBERT_ORDERING
    const int curve = DKT_CURVE_HILBERT;
#else
    const int curve = DKT_CURVE_MORTON;
#endif
    if (dkt_da_create(dim, da->getElementOrder(), curve, m_uiMaxDepth, c.data(), l.data(), (int64_t) tree.size(), 1,
                      &da_) != DKT_OK)
      throw std::runtime_error(dkt_last_error());
    if (dkt_plan_create(da_, op, nullptr, &plan_) != DKT_OK) throw std::runtime_error(dkt_last_error());
  }
  ~feMatrixGpu()
  {
    dkt_plan_destroy(plan_);
    dkt_da_destroy(da_);
  }
  feMatrixGpu(const feMatrixGpu &) = delete;
  feMatrixGpu &operator=(const feMatrixGpu &) = delete;

  void matVec(const VECType *in, VECType *out, double scale = 1.0) override
  {
    if (dkt_fematrix_matvec_host(plan_, in, out, scale) != DKT_OK) throw std::runtime_error(dkt_last_error());
  }

  /* HeatMat::cgSolve: x holds the initial guess and receives the solution;
   * tol receives the final relative L-infinity residual; returns 0 when it
   * converged within max_iter iterations, 1 otherwise. */
  int cgSolve(double *x, double *b, int max_iter, double &tol, unsigned int var = 0)
  {
    (void) var;
    int it = 0;
    double rr = 0.0;
    const int rc = dkt_cg_solve_host(plan_, b, x, max_iter, tol, DKT_CG_REFERENCE, &it, &rr);
    if (rc != DKT_OK && rc != DKT_E_NOCONV) throw std::runtime_error(dkt_last_error());
    tol = rr;
    return rc == DKT_OK ? 0 : 1;
  }
};

#endif
