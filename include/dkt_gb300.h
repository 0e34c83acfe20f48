/*
 * dkt_gb300.h -- C ABI of the GB300 (sm_103a) implementation of Dendro-KT's
 * adaptive k-tree finite-element matvec, dim 2-4, element order 1-2.
 *
 * Plain pointers and sizes only.  Every function returns DKT_OK (0) on
 * success or a negative DKT_E* code; dkt_last_error() describes the last
 * failure of the calling thread.  No exception crosses the ABI.
 *
 * Coordinates follow the reference's integer convention: an orthant or node
 * is a dim-vector of uint32 in [0, 2^max_depth] plus a level (the reference's
 * TreeNode<unsigned,dim>, include/treeNode.h:36-253; m_uiMaxDepth is
 * max_depth).  Arrays of coordinates are row-major [n][dim].
 *
 * Device pointers ("_dev") are CUDA global-memory addresses on the current
 * device; "stream" is a cudaStream_t passed as void* (NULL = legacy stream).
 */
#ifndef DKT_GB300_H
#define DKT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DKT_OK 0
#define DKT_E_ARG (-1)      /* invalid argument */
#define DKT_E_CUDA (-2)     /* CUDA runtime error */
#define DKT_E_NOMEM (-3)    /* device allocation failed */
#define DKT_E_UNSUP (-4)    /* configuration not supported */
#define DKT_E_NOCONV (-5)   /* iterative solve did not converge */
#define DKT_E_INTERNAL (-6)

#define DKT_CURVE_MORTON 0
#define DKT_CURVE_HILBERT 1

/* Elemental operators.  IDENTITY is the test operator of
 * test/testMatvec.cpp:187-198; HEAT is HeatEq::HeatMat<3>::elementalMatVec
 * (FEM/examples/src/heatMat.cpp:45-117, scale ignored, Dirichlet zeroing in
 * pre/postMatVec :119-139); LAPMASS is the Laplacian + mass operator
 * K_e = J^(d-2) K_ref + J^d M_ref (J = h/2) with the same boundary zeroing;
 * CUSTOM takes one dense nPe x nPe table per level, tabulated by the caller
 * from its own feMatrix::elementalMatVec (an arbitrary host callback cannot
 * run on the device). */
#define DKT_OP_IDENTITY 0
#define DKT_OP_HEAT 1
#define DKT_OP_LAPMASS 2
#define DKT_OP_CUSTOM 3
/* Laplacian alone (J^(d-2) K_ref, Dirichlet zeroing as HeatMat) and mass
 * alone (J^d M_ref in any dim, no boundary step: the right-hand side b = M f
 * of the Poisson problems, whose boundary rows the caller zeroes). */
#define DKT_OP_LAPLACE 4
#define DKT_OP_MASS 5
/* HeatEq::HeatVec<3>::elementalComputeVec (FEM/examples/src/heatVec.cpp:30-78):
 * the mass right-hand side J^3 M_ref, scale ignored, with the Dirichlet
 * zeroing of input and output of pre/postComputeVec (:83-105); the operator
 * that feVector::computeVec applies (FEM/include/feVector.h:122-168).  dim 3
 * only, as in the reference (its 3D tensor kernels). */
#define DKT_OP_HEATVEC 6

typedef struct dkt_da_s *dkt_da;
typedef struct dkt_plan_s *dkt_plan;

/* ---- ot::DA<dim> --------------------------------------------------------
 * dkt_da_create replaces ot::DA<dim>::DA(inTree, nEle, comm, order)
 * (include/oda.h:150-167, src/oda.cpp:45-151) on one rank.  The tree must be
 * complete and 2:1 balanced; unless tree_is_sorted, it is first put into SFC
 * order exactly as SFC_Tree::locTreeSort does (include/tsort.tcc:14-80).  The
 * node list, its order, the node levels and the boundary ids equal the
 * reference's bit for bit (SFC_NodeSort::dist_countCGNodes,
 * include/nsort.tcc:492-533).  Runs on the device. */
int dkt_da_create(int dim, int order, int curve, int max_depth, const uint32_t *tree_coords,
                  const uint8_t *tree_levels, int64_t n_elem, int tree_is_sorted, dkt_da *out);
/* ot::DA::getLocalNodalSz (include/oda.h:180); equals getTotalNodalSz on one rank. */
int64_t dkt_da_local_nodal_size(dkt_da da);
int64_t dkt_da_num_elements(dkt_da da);
/* Number of domain-boundary nodes (size of getBoundaryNodeIndices, oda.h:264). */
int64_t dkt_da_boundary_size(dkt_da da);
/* Host copies of getTNCoords (oda.h:252): coords [n][dim], levels [n]. */
int dkt_da_get_nodes(dkt_da da, uint32_t *coords, uint8_t *levels);
/* Host copy of getBoundaryNodeIndices (oda.h:264). */
int dkt_da_get_boundary_ids(dkt_da da, uint32_t *ids);
/* Host copy of the SFC-ordered tree the DA was built on. */
int dkt_da_get_tree(dkt_da da, uint32_t *coords, uint8_t *levels);

/* Fields evaluated by the caller on batches of points: x [n][dim] with
 * coordinates in [0, 1], out [n][n_vars]; a nonzero return is a failure. */
typedef int (*dkt_field_fn)(const double *x, int64_t n, int dim, double *out, int n_vars, void *user);

/* DA<dim>::setVectorByFunction (include/oda.tcc:437-470) on a host nodal
 * vector: out [n][dof] (interleaved, [abc][abc]) gets fn at every DA node.
 * As in the reference, the function sees the first min(dim, 3) coordinates
 * of the node, scaled by 1/2^max_depth (dim passed to fn accordingly).  fn is
 * called on batches of about 1 M nodes. */
int dkt_da_set_vector_by_function(dkt_da da, dkt_field_fn fn, void *user, int dof, double *out);
void dkt_da_destroy(dkt_da da);

/* ---- fem::matvec -----------------------------------------------------------
 * A plan is the flattened form of the recursive traversal
 * fem::matvec(vecIn, vecOut, coords, sz, partFront, partBack, eleOp, scale,
 * refElement) (FEM/include/matvec.h:37-38, 231-548): built once per node list,
 * reused for every product.  op_tables is NULL except for DKT_OP_CUSTOM, where
 * it holds (max_depth+1) tables of nPe*nPe doubles (row = output rank,
 * column = input rank; rank = lexicographic element node index, x fastest).
 */
int dkt_plan_create(dkt_da da, int op, const double *op_tables, dkt_plan *out);
/* Traversal variants.  REFERENCE reproduces fem::matvec exactly, including
 * its parent-buffer reads (matvec.h:411-456) and its transpose mask
 * (matvec.h:497-521), which make the operator non-symmetric.  CONFORMING
 * takes the parent values from every node on the parent lattice and adds the
 * transpose to all of them: the symmetric P^T K P, for Krylov solvers (no
 * counterpart in the reference). */
#define DKT_TRAVERSAL_REFERENCE 0
#define DKT_TRAVERSAL_CONFORMING 1
int dkt_plan_create_ex(dkt_da da, int op, const double *op_tables, int traversal, dkt_plan *out);
/* Same, from a bare node list (the `coords, sz` arguments of fem::matvec). */
int dkt_plan_create_from_nodes(int dim, int order, int curve, int max_depth, const uint32_t *node_coords,
                               const uint8_t *node_levels, int64_t sz, int op, const double *op_tables,
                               dkt_plan *out);
int64_t dkt_plan_num_nodes(dkt_plan plan);
/* Counters of the flattened traversal: [0] leaf visits, [1] hanging leaves,
 * [2] parent-buffer slots that the reference would read without refilling
 * (nonzero means its result depends on earlier leaves; the device path uses
 * zero there), [3] boundary nodes. */
int dkt_plan_stats(dkt_plan plan, int64_t *out4);

/* Extended counts, up to n of: leaves, hanging leaves, stale slots, boundary
 * nodes, stale-chain entries, stale-chain runs, longest run (hanging leaves),
 * longest run (entries), mixed-precision solves on the plan that finished
 * some mesh with FP64 PCG (its binary32 recursion had stopped tracking the
 * true residual).  Instrumentation, no reference counterpart. */
int dkt_plan_stats_ex(dkt_plan plan, int64_t *out, int n);

/* Host copy of the flattened traversal (for inspection and tests):
 * e2n [leaves][nPe] node of each lexicographic rank or -1; info [leaves]
 * level | child<<8 | hanging<<16; hidx [leaves] hanging record or -1;
 * p2n [hanging][nPe] parent node of level L-1 per rank or -1; fill
 * [hanging][3] filled-rank bit masks.  Any pointer may be NULL. */
int dkt_plan_export(dkt_plan plan, int32_t *e2n, uint32_t *info, int32_t *hidx, int32_t *p2n, uint32_t *fill);

/* fem::matvec on device arrays: y = sum over leaves of the elemental products
 * (no boundary handling).  y is overwritten (matvec.h:235). */
int dkt_matvec(dkt_plan plan, const double *x_dev, double *y_dev, double scale, void *stream);

/* feMatrix<LeafT,dim>::matVec(in, out, scale) (FEM/include/feMatrix.h:189-259)
 * on device arrays: pre-matvec boundary zeroing of the input copy, fem::matvec,
 * post-matvec boundary zeroing of the output (for HEAT and LAPMASS, the
 * reference's HeatMat::preMatVec/postMatVec; IDENTITY and CUSTOM have no
 * pre/post step).  x_dev is not modified. */
int dkt_fematrix_matvec(dkt_plan plan, const double *x_dev, double *y_dev, double scale, void *stream);

/* feMatrix::matVec that allocates no device memory (no counterpart in the
 * reference).  For callers that must not allocate during a product: a solver
 * or serving loop that reserved its device-memory budget up front, or host
 * code that must not let cudaMalloc/cudaFree stall the device.  Same result
 * as dkt_fematrix_matvec with DKT_ARITH_FP64 (the dense native-FP64 kernel).
 * Its one scratch buffer, the boundary-zeroed input copy, is a fixed array in
 * device global memory of 1,048,576 doubles (8 MiB) that every GPU loading
 * this library holds until the process exits; plans with more nodes are
 * rejected with DKT_E_ARG.  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  All calls share the array:
 * calls whose work overlaps on the GPU (different streams, or different
 * threads) race on it and must be serialised by the caller.  A plan with
 * static-parent-buffer reads (stale slots, see dkt_plan_stats_ex) also keeps
 * the chain of those reads in buffers of its own, made when the plan was
 * created, which every product on that plan rewrites: a call on a plan must
 * not overlap any other product on the same plan either. */
int dkt_fematrix_matvec_noalloc(dkt_plan plan, const double *x_dev, double *y_dev, double scale, void *stream);

/* One part of a partitioned mesh (the rank-local plan of a multi-rank ot::DA,
 * src/oda.cpp:52-151 with SFC_NodeSort::dist_countCGNodes,
 * include/nsort.tcc:492-803): the leaves [leaf_begin, leaf_end) of `full`'s
 * flattened traversal, their node indices renumbered by node_map (host
 * array of full's node count: the part's local index of every node its
 * leaves touch, -1 elsewhere; n_local local nodes, ghosts included).  Its
 * dkt_matvec is the part's share of fem::matvec (include/matvec.h:231-548) on
 * the part's ghosted layout; the partition, ownership and ghost exchange
 * around it are the host's (dendro-kt_gb300/partition.py).  Plans that read
 * stale parent-buffer slots and batch plans are refused (DKT_E_UNSUP). */
int dkt_plan_create_part(dkt_plan full, int64_t leaf_begin, int64_t leaf_end, const int32_t *node_map,
                         int64_t n_local, dkt_plan *out);

/* Same with host arrays: copies in, computes, copies out, synchronises. */
int dkt_fematrix_matvec_host(dkt_plan plan, const double *x_host, double *y_host, double scale);

/* count products y_k = A x_k with host arrays (no counterpart in the
 * reference), pipelined: while product k runs, x_{k+1} is copied in and
 * y_{k-1} copied out, on separate streams with two device buffers each way.
 * With pinned host arrays the copies overlap the compute.  Returns when every
 * y_k is on the host; each is what dkt_fematrix_matvec_host would give. */
int dkt_fematrix_matvec_host_many(dkt_plan plan, const double *const *x_host, double *const *y_host, int count,
                                  double scale);

/* feVector<T,dim>::computeVec(in, out, scale) (FEM/include/feVector.h:122-168):
 * preComputeVec on the input copy, fem::matvec with elementalComputeVec,
 * postComputeVec on the output.  The plan's operator is the vector's
 * elemental operator: DKT_OP_HEATVEC for HeatEq::HeatVec<3>, DKT_OP_MASS for
 * the mass right-hand side in any dim (no boundary step), or DKT_OP_CUSTOM
 * tables.  Device arrays; same traversal and result as dkt_fematrix_matvec. */
int dkt_fevector_compute_vec(dkt_plan plan, const double *in_dev, double *out_dev, double scale, void *stream);

/* Diagonal of the operator (for Jacobi preconditioning), on device. */
int dkt_diagonal(dkt_plan plan, double *diag_dev, void *stream);

/* CG on feMatrix::matVec in the form of HeatMat::cgSolve
 * (FEM/examples/src/heatMat.cpp:164-325).  flags:
 *   0                  unpreconditioned, stopping when ||r||_2 <= tol ||b||_2,
 *                      confirmed on the true residual b - A x (the iteration
 *                      restarts from x while that is above tol);
 *   DKT_CG_JACOBI      the same, Jacobi-preconditioned;
 *   DKT_CG_REFERENCE   HeatMat::cgSolve itself: no preconditioner,
 *                      alpha = <r0,r0>/<p,Ap>, beta = <r1,r1>/<r0,r0>, stopping
 *                      when ||r||_inf <= tol ||b||_inf (||b||_inf = 0 counts as 1,
 *                      heatMat.cpp:207-227) on the plan's own traversal; relres
 *                      is then the final relative L-infinity residual (the tol
 *                      that cgSolve writes back) and iters the iteration at
 *                      which it stopped (0 if x already met tol).
 * x_dev holds the initial guess and receives the solution.  iters/relres may
 * be NULL.  Returns DKT_OK on convergence, -5 when max_iter was reached
 * (cgSolve's status 1). */
#define DKT_CG_JACOBI 1
#define DKT_CG_REFERENCE 2
int dkt_cg_solve(dkt_plan plan, const double *b_dev, double *x_dev, int max_iter, double tol, int flags,
                 int *iters, double *relres, void *stream);

/* The same with host arrays (b, and x in and out; copies in and out, then
 * synchronises): with DKT_CG_REFERENCE the drop-in for HeatMat::cgSolve
 * (FEM/examples/src/heatMat.cpp:164-325) in the feMatrixGpu binding
 * (include/feMatrixGpu.h). */
int dkt_cg_solve_host(dkt_plan plan, const double *b_host, double *x_host, int max_iter, double tol, int flags,
                      int *iters, double *relres);

#define DKT_PREC_FP64 0
#define DKT_PREC_MIXED 1

/* Device-resident CG on the same operator: scalars stay on the device and
 * blocks of 16 iterations run as one CUDA graph.  For a batch plan every
 * mesh converges on its own (relative to its own ||b||); iters, refinements
 * and relres are then arrays with one entry per mesh.  DKT_PREC_FP64: Jacobi-PCG
 * in FP64.  DKT_PREC_MIXED: Jacobi-PCG on binary32 vectors with the binary32
 * product and reliable updates -- the correction is folded into x in FP64
 * and the residual recomputed with the FP64 product (b - A x) each
 * time the binary32 residual has fallen 100x, or after 512 binary32
 * iterations without that, the search direction kept while the binary32
 * recursion still tracks b - A x -- until ||b - A x||_2 <= tol ||b||_2
 * (FP64 residual); refinements counts the updates.  A mesh on which binary32
 * stops making progress is finished by FP64 PCG from its x.  Dot products
 * accumulate in FP64 in both.  Mixed needs a Q1 or Q2 built-in operator without
 * stale parent reads (a conforming plan, or a mesh without them); it is the
 * solver of HeatMat::cgSolve (FEM/examples/src/heatMat.cpp:164-325) with the
 * precision split that the reference does not have.  iters = CG iterations
 * (all inner iterations for mixed), refinements = outer steps (0 for FP64).
 * Returns DKT_OK on convergence, -5 when max_iter was reached. */
int dkt_pcg_solve(dkt_plan plan, const double *b_dev, double *x_dev, int precision, int max_iter, double tol,
                  int jacobi, int *iters, int *refinements, double *relres, void *stream);

/* Batch of independent meshes as one block-diagonal plan: the flattened
 * traversals (and tiles) of n plans are concatenated, so one launch of the
 * leaf kernel computes all n products and dkt_pcg_solve solves all n
 * systems at once, each mesh with its own scalars and convergence test.
 * Vectors are the meshes' vectors one after another (dkt_plan_mesh_offsets).
 * The plans must share dim, order, max_depth, operator (built-in), traversal
 * and tile size, and have no stale parent reads; they stay valid and
 * independent.  No counterpart in the reference (one mesh per ot::DA). */
int dkt_batch_create(const dkt_plan *plans, int n, dkt_plan *out);

/* Meshes in a plan (1 unless it is a batch) and their node offsets (n+1). */
int dkt_plan_num_meshes(dkt_plan plan, int *n);
int dkt_plan_mesh_offsets(dkt_plan plan, int64_t *offsets);

/* Times the product on this plan (uniform[-1,1] input) for every launch
 * shape and keeps the fastest: the untiled kernel, then for each supported
 * tile size (leaves, i.e. elements, per CTA) the plain grid of one CTA per
 * tile and the persistent launch whose CTAs pull tiles from a counter (dims 2
 * and 3).  arith: 0 the FP64 feMatrix product, 1 the binary32 product of the
 * mixed-precision solver.  times (may be NULL): 7 entries, ms per product of
 * the candidates in that order (untiled; then per tile size, ascending, plain
 * and persistent), -1 where not available.  No counterpart in the reference. */
int dkt_plan_autotune_ex(dkt_plan plan, int arith, int *best_tile, int *best_persist, double *best_ms,
                         double *times);
/* The same for the FP64 product, without the per-candidate times. */
int dkt_plan_autotune(dkt_plan plan, int *best_tile, double *best_ms);

/* Binary32 feMatrix product y = A x with the Q1 or Q2 built-in operator of
 * the plan (boundary entries zeroed in and out as feMatrix::matVec does for
 * the operators with Dirichlet steps).  No counterpart in the reference, which is
 * FP64 only; accuracy about 1e-6 relative. */
int dkt_matvec_f32(dkt_plan plan, const float *x_dev, float *y_dev, void *stream);

/* Arithmetic of the leaf kernel.  AUTO (default) uses FIXED where it applies:
 * the Q1 built-in operators are diagonal in the Hadamard basis and run in
 * exact int64 fixed point (deterministic, ~2^-50 relative to max|x|*|K|,
 * well inside the 1e-12 parity tolerance), and the Q2 built-in operators run
 * on the sum-factorised FP64 kernel; FP64 forces the dense native-FP64
 * kernel (always used for custom operators). */
#define DKT_ARITH_AUTO 0
#define DKT_ARITH_FP64 1
#define DKT_ARITH_FIXED 2
int dkt_plan_set_arithmetic(dkt_plan plan, int mode);

/* Measurement hook: with enable = 1 the leaf kernel of every later product
 * is bracketed by CUDA events on its launching stream.  Each call first
 * closes the current window, returning the summed kernel time (ms) and the
 * number of timed launches since the previous call (synchronising on the
 * last event), then sets the new state. */
int dkt_plan_kernel_timing(dkt_plan plan, int enable, double *total_ms, int64_t *launches);

/* Leaf tiling of the Q1 built-in operators: tile_leaves consecutive leaves
 * (64/128/256 in 4D, 128/256/512 in 2D/3D) share one CTA, a per-tile list of
 * distinct nodes and 16-bit local maps; 0 selects the untiled kernel.  The
 * result does not depend on it (fixed point: bitwise).  A tuning knob with no
 * reference counterpart; plans start with 128 in 4D and 256 in 2D and 3D. */
int dkt_plan_set_tile(dkt_plan plan, int tile_leaves);

/* Number of kernels this plan's matrix-vector products and solves have
 * launched so far (cumulative; every kernel of the library, not only the
 * leaf kernel).  Instrumentation with no counterpart in the reference. */
int dkt_plan_launch_count(dkt_plan plan, int64_t *count);

void dkt_plan_destroy(dkt_plan plan);

/* Throughput probes of the current device (no counterpart in the reference):
 * out4 = {FP64 FMA TFLOP/s, FP64 add Tops/s, FP32 FMA TFLOP/s, int64 add Tops/s}. */
int dkt_probe_device(double *out4);

const char *dkt_last_error(void);

/* ---------------------------------------------------------------------------
 * Serving: a request loop for Q1 Poisson solves (-Laplace u = f, homogeneous
 * Dirichlet, conforming traversal).  No counterpart in the reference, which
 * solves one mesh per process.  Requests are admitted against a device-memory
 * budget in arrival order and run concurrently on `workers` host threads,
 * each on its own stream, so kernels of different requests overlap; a
 * finished request frees its memory and admits the next ones.  The right-hand
 * side is b = uniform[-1,1] (counter-based, seeded) with Dirichlet rows
 * zeroed; the solver is dkt_pcg_solve with the server's precision and
 * tolerance.  Times are seconds since dkt_server_create.
 * ------------------------------------------------------------------------- */
typedef struct dkt_server_s *dkt_server;

typedef struct {
  int rc;                       /* DKT_OK, -5 (not converged) or an error */
  int dim;
  int64_t n_elem, n_nodes;
  int iterations, refinements;
  double relres;                /* ||b - A x||_2 / ||b||_2 */
  double t_submit, t_admit, t_start, t_done;
  int64_t device_bytes;         /* peak device bytes of the request */
  double est_bytes;             /* footprint the admission used */
} dkt_solve_report;

/* precision: DKT_PREC_FP64, DKT_PREC_MIXED, or 2 = FP64 PCG with the dense
 * native-FP64 leaf kernel (DKT_ARITH_FP64: the plain FP64 path). */
int dkt_server_create(int workers, double budget_bytes, int precision, double tol, dkt_server *out);
/* Copies the tree; returns at once with a ticket. */
int dkt_server_submit(dkt_server srv, int dim, int max_depth, const uint32_t *tree_coords, const uint8_t *tree_levels,
                      int64_t n_elem, uint64_t rhs_seed, int64_t *ticket);
/* Blocks until the request is done. */
int dkt_server_wait(dkt_server srv, int64_t ticket, dkt_solve_report *report);
/* Copies the solution (n_nodes values, DA node order) of a finished request. */
int dkt_server_solution(dkt_server srv, int64_t ticket, double *x_host, int64_t capacity);
/* The error message of a request that failed (empty when it did not). */
int dkt_server_error(dkt_server srv, int64_t ticket, char *buf, int capacity);
/* Drops a finished request's stored result. */
int dkt_server_release(dkt_server srv, int64_t ticket);
/* Finishes the admitted requests, drops the queued ones, joins the workers. */
void dkt_server_destroy(dkt_server srv);

#ifdef __cplusplus
}
#endif

#endif /* DKT_GB300_H */
