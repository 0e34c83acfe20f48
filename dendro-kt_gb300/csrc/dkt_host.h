// Host-side declarations shared by the C ABI and dkt_host.cpp.
#pragma once
#include <cstdint>
#include <vector>

namespace dkt {

struct RefEl1D {
  int p = 1, M = 2;
  std::vector<double> ip0, ip1, Q, D, W;
};
RefEl1D refel_1d(int p);
void builtin_operator(int kind, int dim, int p, int md, std::vector<double> &A, std::vector<double> &B,
                      std::vector<double> &alpha, std::vector<double> &beta, bool &uses_scale);
// Order-2 factors: M1 = T^T T, K1 = T^T diag(lam) T (T row-major 3x3), and the
// middle row (a, b, c) of the child-0 interpolation; false if the 1D operators
// do not have the expected symmetric structure.
bool q2_factors(double T[9], double lam[3], double pint[3]);

// Field evaluation on a batch of points: x [n][dim] in the unit cube,
// out [n][n_vars]; nonzero return = failure.
typedef int (*FieldFn)(const double *x, int64_t n, int dim, double *out, int n_vars, void *user);

struct Cell {
  uint32_t x[4];
  int lev;
};
void gaussian_points(int64_t n, int dim, int md, double mean, double sd, uint64_t seed, uint32_t *out);
std::vector<Cell> tree_from_points(const uint32_t *pts, int64_t n, int dim, int md, int64_t max_pts);
std::vector<Cell> moving_ball_tree(int md, int level, double R, double w, const double *c0, const double *c1);
std::vector<Cell> sphere_shell_tree(int dim, int md, int level, double R, double w, const double *ctr);
// Rotation tables of the harmonious Hilbert curve: per orientation, 2^dim
// Morton children in curve order then the curve rank of every Morton child
// (rot), and the orientation of every Morton child (ht).
void hilbert_tables(int dim, std::vector<int8_t> &rot, std::vector<int32_t> &ht, int &nrot);
// VTU file of a tree (dim 2 or 3), optionally with one value per cell.
void write_vtu(const char *path, int dim, int md, const uint32_t *coords, const uint8_t *levels, int64_t n,
               const double *cell_values, const char *cell_values_name);

}  // namespace dkt
