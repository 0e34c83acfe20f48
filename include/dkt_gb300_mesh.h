/*
 * dkt_gb300_mesh.h -- C ABI of the host-side mesh generators that produce
 * the input trees of the matvec path (the reference's ot::getPts,
 * include/octUtils.h:29-65, and SFC_Tree::locTreeBalancing /
 * distTreeBalancing on one rank, src/tsort.cpp:826-878).  Return codes as in
 * dkt_gb300.h.  Arrays returned through pointer-to-pointer arguments are
 * allocated with malloc and released with dkt_free.
 */
#ifndef DKT_GB300_MESH_H
#define DKT_GB300_MESH_H

#include <stdint.h>
#include "dkt_gb300.h"   /* dkt_field_fn */

#ifdef __cplusplus
extern "C" {
#endif

/* n points, each coordinate N(mean, sd) on the unit cube (clipped), drawn from
 * a counter-based stream of the given seed, quantised to level max_depth;
 * out is [n][dim]. */
int dkt_mesh_gaussian_points(int64_t n, int dim, int max_depth, double mean, double sd, uint64_t seed,
                             uint32_t *out);

/* Complete tree with at most max_pts points per leaf, then 2:1 balanced over
 * all 3^dim - 1 neighbours; cells are returned unsorted (dkt_da_create sorts). */
int dkt_mesh_tree_from_points(const uint32_t *pts, int64_t n, int dim, int max_depth, int64_t max_pts,
                              int64_t *n_out, uint32_t **coords, uint8_t **levels);
/* Same tree, built on the current device: the points' Morton keys are sorted
 * once, cells are refined level by level (a cell's point count is a key
 * range), then balanced as above; cells returned sorted by level. */
int dkt_mesh_tree_from_points_device(const uint32_t *pts, int64_t n, int dim, int max_depth, int64_t max_pts,
                                     int64_t *n_out, uint32_t **coords, uint8_t **levels);

/* dim 4 (x,y,z,t): every cell whose box meets the shell
 * | |(x,y,z) - c(t)| - radius | <= halfwidth, c(t) = c0 + (c1 - c0) t, is refined
 * down to `level`; the result is 2:1 balanced. */
int dkt_mesh_moving_ball(int max_depth, int level, double radius, double halfwidth, const double *c0,
                         const double *c1, int64_t *n_out, uint32_t **coords, uint8_t **levels);

/* Same mesh, built on the current device (refinement frontier level by level,
 * balancing by sorted cell-key sets); cells returned sorted by level. */
int dkt_mesh_moving_ball_device(int max_depth, int level, double radius, double halfwidth, const double *c0,
                                const double *c1, int64_t *n_out, uint32_t **coords, uint8_t **levels);

/* ot::function2Octree (include/octUtils.h:180-417) and, with balance = 1,
 * the tree of ot::DA<dim>::DA(func, dofSz, comm, order, interp_tol)
 * (include/oda.tcc:67-88), built on the current device.  From the root's
 * children, level by level up to max_depth, a cell is split when
 * interpolating any of the n_vars fields from its element nodes (order 1 or
 * 2) to the element nodes of one of its children misses the field's values
 * there by more than interp_tol (max norm).  The fields are evaluated by `fn`
 * on the host, on batches of points (about 4 M per call): x [n][dim] with
 * coordinates in [0, 1], out [n][n_vars]; a nonzero return aborts with
 * DKT_E_INTERNAL.  With balance = 1 the tree is then 2:1 balanced.  Arrays
 * are freed with dkt_free. */
int dkt_mesh_function2octree(dkt_field_fn fn, void *user, int n_vars, int dim, int max_depth, int order,
                             double interp_tol, int balance, int64_t *n_out, uint32_t **coords, uint8_t **levels);

/* Rotation tables of a space-filling curve, the data that _InitializeHcurve
 * (src/KDhcurvedata.cpp:23-57) loads: per orientation, the Morton children
 * in curve order then the curve rank of every Morton child (rot, 2^(dim+1)
 * bytes), and the orientation of every Morton child (ht, 2^dim ints).
 * DKT_CURVE_HILBERT is the harmonious Hilbert curve, generated here from
 * Haverkort's refinement rule (not copied tables); orientations may be
 * numbered differently from the reference's, the curve is the same.
 * Buffers: rot >= 192*32 bytes, ht >= 192*16 ints for dim 4. */
int dkt_curve_tables(int curve, int dim, int8_t *rot, int32_t *ht, int *nrot);

/* Sphere-shell refinement in dim 2..4, built on the device: every cell of
 * level < `level` whose box meets | ||x - centre|| - radius | <= halfwidth is
 * split (exact box distance interval), then the tree is 2:1 balanced.  The
 * workload generator of the served request stream (refinement on a random
 * sphere); no reference counterpart beyond SFC_Tree::locTreeBalancing
 * (src/tsort.cpp:826-854) for the balance.  Arrays are freed with dkt_free. */
int dkt_mesh_sphere_shell(int dim, int max_depth, int level, double radius, double halfwidth, const double *centre,
                          int64_t *n_out, uint32_t **coords, uint8_t **levels);   /* host build, same tree */
int dkt_mesh_sphere_shell_device(int dim, int max_depth, int level, double radius, double halfwidth,
                                 const double *centre, int64_t *n_out, uint32_t **coords, uint8_t **levels);

/* io::vtk::oct2vtu (IO/vtk/include/oct2vtk.h:272-273): the tree as a VTK XML
 * unstructured grid with the reference's arrays: one hexahedron (3D) or quad
 * (2D) per cell with its own corner points in integer lattice coordinates
 * (Position, UInt32, 0..2^max_depth), UInt64 connectivity and offsets, UInt8
 * types, and the cell data mpi_rank (0) and cell_level (UInt32), as inline
 * base64 binary arrays.  cell_values (one double per cell, named
 * cell_values_name) may be NULL.  The reference instantiates dim 3 only;
 * dim 2 here as quads; DKT_E_ARG for other dims (VTK has no 4D cells). */
int dkt_write_vtu(const char *path, int dim, int max_depth, const uint32_t *coords, const uint8_t *levels,
                  int64_t n_cells, const double *cell_values, const char *cell_values_name);

void dkt_free(void *p);

#ifdef __cplusplus
}
#endif

#endif
