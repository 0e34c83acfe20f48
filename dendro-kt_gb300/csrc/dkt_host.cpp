// Host-side pieces of the product: reference-element operators and the mesh
// generators that produce the input trees (the callers of the matvec path).
//
//  * refel_1d: the 1D operators of RefElement (FEM/src/refel.cpp:75-220) from
//    the mathematics -- Lagrange basis on equispaced nodes, Gauss-Legendre
//    quadrature -- in the reference's storage convention A[k*M + j] = basis k
//    evaluated at point j.
//  * element matrices of the built-in operators, dense in lexicographic rank
//    order (x fastest).
//  * tree construction and 2:1 balancing with the semantics of
//    SFC_Tree::locTreeConstruction / propagateNeighbours / locTreeBalancing
//    (src/tsort.cpp:566-854), organised by level sets instead of recursive
//    bucketing.
//  * the moving-ball spacetime mesh (dim 4).
//  * VTU output of a tree (io::vtk::oct2vtu).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <stdexcept>
#include <unordered_set>
#include <vector>

#include "dkt_host.h"

namespace dkt {

static double lag(const std::vector<double> &u, int k, double x)
{
  double v = 1.0;
  for (int m = 0; m < (int) u.size(); m++) if (m != k) v *= (x - u[m]) / (u[k] - u[m]);
  return v;
}
static double lag_d(const std::vector<double> &u, int k, double x)
{
  double s = 0.0;
  for (int i = 0; i < (int) u.size(); i++) {
    if (i == k) continue;
    double t = 1.0 / (u[k] - u[i]);
    for (int m = 0; m < (int) u.size(); m++) if (m != k && m != i) t *= (x - u[m]) / (u[k] - u[m]);
    s += t;
  }
  return s;
}

RefEl1D refel_1d(int p)
{
  RefEl1D r;
  r.p = p;
  r.M = p + 1;
  const int M = r.M;
  std::vector<double> u(M), g(M), w(M);
  for (int k = 0; k < M; k++) u[k] = -1.0 + 2.0 * k / p;
  for (int i = 0; i < M; i++) {
    double x = -std::cos(M_PI * (i + 0.75) / (M + 0.5)), dp = 1.0;
    for (int it = 0; it < 60; it++) {
      double p0 = 1.0, p1 = x;
      for (int n = 2; n <= M; n++) { double p2 = ((2.0 * n - 1) * x * p1 - (n - 1.0) * p0) / n; p0 = p1; p1 = p2; }
      dp = M * (x * p1 - p0) / (x * x - 1.0);
      const double dx = p1 / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    double p0 = 1.0, p1 = x;
    for (int n = 2; n <= M; n++) { double p2 = ((2.0 * n - 1) * x * p1 - (n - 1.0) * p0) / n; p0 = p1; p1 = p2; }
    dp = M * (x * p1 - p0) / (x * x - 1.0);
    g[i] = x;
    w[i] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
  r.ip0.resize(M * M); r.ip1.resize(M * M); r.Q.resize(M * M); r.D.resize(M * M); r.W = w;
  for (int k = 0; k < M; k++)
    for (int j = 0; j < M; j++) {
      r.ip0[k * M + j] = lag(u, k, 0.5 * (u[j] - 1.0));
      r.ip1[k * M + j] = lag(u, k, 0.5 * (u[j] + 1.0));
      r.Q[k * M + j] = lag(u, k, g[j]);
      r.D[k * M + j] = lag_d(u, k, g[j]);
    }
  return r;
}

// Simultaneous diagonalisation of the order-2 1D mass M1 = Q^T W Q and
// stiffness K1 = D^T W D: a transform T with M1 = T^T T and K1 = T^T diag(lam) T.
// Both matrices are centrosymmetric (symmetric nodes and quadrature), so the
// pencil splits into an even 2x2 block on span{(1,0,1), (0,1,0)} and an odd
// 1x1 block on (1,0,-1).  The even block is reduced by the Cholesky factor of
// its mass and diagonalised by one Jacobi rotation.  Rows 0, 1 of T are even
// (t00, t01, t00), (t10, t11, t10) and row 2 is odd (t20, 0, -t20); T is
// returned row-major.  Computed in long double.
bool q2_factors(double T[9], double lam[3], double pint[3])
{
  const RefEl1D re = refel_1d(2);
  typedef long double R;
  R M1[9], K1[9];
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      R m = 0, k = 0;
      for (int g = 0; g < 3; g++) {
        m += (R) re.W[g] * re.Q[r * 3 + g] * re.Q[c * 3 + g];
        k += (R) re.W[g] * re.D[r * 3 + g] * re.D[c * 3 + g];
      }
      M1[r * 3 + c] = m;
      K1[r * 3 + c] = k;
    }
  const R s2 = std::sqrt((R) 0.5);
  const R me00 = (M1[0] + M1[2] + M1[6] + M1[8]) / 2, me01 = (M1[1] + M1[7]) * s2, me11 = M1[4];
  const R ke00 = (K1[0] + K1[2] + K1[6] + K1[8]) / 2, ke01 = (K1[1] + K1[7]) * s2, ke11 = K1[4];
  const R mo = (M1[0] - M1[2] - M1[6] + M1[8]) / 2, ko = (K1[0] - K1[2] - K1[6] + K1[8]) / 2;
  const R l11 = std::sqrt(me00), l21 = me01 / l11, l22 = std::sqrt(me11 - l21 * l21);
  // Li = L^-1, C = Li Ke Li^T
  const R i00 = 1 / l11, i10 = -l21 / (l11 * l22), i11 = 1 / l22;
  const R c00 = i00 * i00 * ke00;
  const R c01 = i00 * (i10 * ke00 + i11 * ke01);
  const R c11 = i10 * i10 * ke00 + 2 * i10 * i11 * ke01 + i11 * i11 * ke11;
  const R th = std::atan2(2 * c01, c00 - c11) / 2, c = std::cos(th), s = std::sin(th);
  const R lam0 = c00 * c * c + 2 * c01 * c * s + c11 * s * s;
  const R lam1 = c00 * s * s - 2 * c01 * c * s + c11 * c * c;
  // Se = Li^T V, V = [[c, -s], [s, c]]: generalised eigenvectors in the even basis
  const R se00 = i00 * c + i10 * s, se01 = -i00 * s + i10 * c;
  const R se10 = i11 * s, se11 = i11 * c;
  R S[9];   // columns: two even modes, one odd mode
  S[0] = se00 * s2; S[3] = se10; S[6] = se00 * s2;
  S[1] = se01 * s2; S[4] = se11; S[7] = se01 * s2;
  S[2] = s2 / std::sqrt(mo); S[5] = 0; S[8] = -s2 / std::sqrt(mo);
  // T = S^T M1 = S^-1 (S^T M1 S = I)
  R Tl[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      R v = 0;
      for (int k = 0; k < 3; k++) v += S[k * 3 + i] * M1[k * 3 + j];
      Tl[i * 3 + j] = v;
    }
  const R t00 = (Tl[0] + Tl[2]) / 2, t10 = (Tl[3] + Tl[5]) / 2, t20 = (Tl[6] - Tl[8]) / 2;
  const R Ts[9] = {t00, Tl[1], t00, t10, Tl[4], t10, t20, 0, -t20};
  for (int i = 0; i < 9; i++) T[i] = (double) Ts[i];
  lam[0] = (double) lam0;
  lam[1] = (double) lam1;
  lam[2] = (double) (ko / mo);
  // check M1 = T^T T and K1 = T^T diag(lam) T
  R err = 0, mx = 0;
  for (int r = 0; r < 3; r++)
    for (int cc = 0; cc < 3; cc++) {
      R m = 0, k = 0;
      for (int i = 0; i < 3; i++) {
        m += Ts[i * 3 + r] * Ts[i * 3 + cc];
        k += Ts[i * 3 + r] * (R) lam[i] * Ts[i * 3 + cc];
      }
      err = std::max(err, std::max(std::fabs(m - M1[r * 3 + cc]), std::fabs(k - K1[r * 3 + cc])));
      mx = std::max(mx, std::max(std::fabs(M1[r * 3 + cc]), std::fabs(K1[r * 3 + cc])));
    }
  // child interpolation: forward row j of child 0 is ip0[k*3 + j] over k;
  // rows 0 and 2 copy parent nodes 0 and 1, child 1 is the mirror image
  const std::vector<double> &a = re.ip0, &b = re.ip1;
  bool ok = err <= 1e-15L * mx;
  ok = ok && a[0] == 1 && a[3] == 0 && a[6] == 0 && a[2] == 0 && a[5] == 1 && a[8] == 0;
  for (int j = 0; j < 3; j++)
    for (int k = 0; k < 3; k++) ok = ok && b[k * 3 + j] == a[(2 - k) * 3 + (2 - j)];
  pint[0] = a[1];
  pint[1] = a[4];
  pint[2] = a[7];
  return ok;
}

// Dense element matrix sum_g w_g * (prod_d B_d[c_d][g_d]) * (prod_d B_d[r_d][g_d])
// over tensor Gauss points g, with B_d = D on axis `deriv` and Q elsewhere
// (deriv < 0: mass).  Only axes < nax carry the quadrature; further axes (the
// 3-axis HeatMat on more dimensions) are left out.
static void tensor_matrix(const RefEl1D &re, int dim, int deriv, std::vector<double> &Kout)
{
  const int M = re.M;
  int npe = 1;
  for (int d = 0; d < dim; d++) npe *= M;
  Kout.assign((size_t) npe * npe, 0.0);
  for (int r = 0; r < npe; r++)
    for (int c = 0; c < npe; c++) {
      double v = 1.0;
      int rr = r, cc = c;
      for (int d = 0; d < dim; d++) {
        const int rd = rr % M, cd = cc % M;
        rr /= M; cc /= M;
        const std::vector<double> &B = (d == deriv) ? re.D : re.Q;
        double s = 0.0;
        for (int g = 0; g < M; g++) s += re.W[g] * B[cd * M + g] * B[rd * M + g];
        v *= s;
      }
      Kout[(size_t) r * npe + c] = v;
    }
}

// Built-in operators: K_L = alpha[L] A + beta[L] B, L = 0..md, element side
// h_L = 2^-L on the unit domain, J = h/2.
void builtin_operator(int kind, int dim, int p, int md, std::vector<double> &A, std::vector<double> &B,
                      std::vector<double> &alpha, std::vector<double> &beta, bool &uses_scale)
{
  const RefEl1D re = refel_1d(p);
  int npe = 1;
  for (int d = 0; d < dim; d++) npe *= re.M;
  A.assign((size_t) npe * npe, 0.0);
  B.assign((size_t) npe * npe, 0.0);
  alpha.assign(md + 1, 0.0);
  beta.assign(md + 1, 0.0);
  uses_scale = true;
  if (kind == 0) {   // identity
    for (int r = 0; r < npe; r++) A[(size_t) r * npe + r] = 1.0;
    for (int l = 0; l <= md; l++) alpha[l] = 1.0;
    return;
  }
  std::vector<double> K;
  for (int t = 0; t < dim; t++) {
    tensor_matrix(re, dim, t, K);
    for (size_t i = 0; i < K.size(); i++) A[i] += K[i];
  }
  if (kind == 1) {   // HeatMat<3>: sum_t (prod_{d!=t} J / J) = J
    if (dim != 3) throw std::invalid_argument("the HeatMat operator is defined for dim 3");
    uses_scale = false;
    for (int l = 0; l <= md; l++) alpha[l] = 0.5 * std::ldexp(1.0, -l);
    return;
  }
  tensor_matrix(re, dim, -1, B);   // mass
  if (kind == 6) {   // HeatVec<3>: J_x J_y J_z (Q^T W Q)^(x)3, scale ignored
    if (dim != 3) throw std::invalid_argument("the HeatVec operator is defined for dim 3");
    uses_scale = false;
    for (int l = 0; l <= md; l++) beta[l] = std::pow(0.5 * std::ldexp(1.0, -l), 3);
    return;
  }
  for (int l = 0; l <= md; l++) {
    const double J = 0.5 * std::ldexp(1.0, -l);
    alpha[l] = (kind == 5) ? 0.0 : std::pow(J, dim - 2);   // 5: mass only
    beta[l] = (kind == 4) ? 0.0 : std::pow(J, dim);         // 4: Laplacian only
  }
}

// ---------------------------------------------------------------------------
// Mesh generation (input side).
// ---------------------------------------------------------------------------
static inline uint64_t splitmix64(uint64_t z)
{
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline double u01(uint64_t seed, uint64_t i)
{
  return (double) (splitmix64(seed * 0xD1B54A32D192ED03ull + i) >> 11) * (1.0 / 9007199254740992.0);
}

// n points, each coordinate N(mean, sd) clipped to the unit cube (Box-Muller
// on a counter-based uniform stream), quantised to level md.
void gaussian_points(int64_t n, int dim, int md, double mean, double sd, uint64_t seed, uint32_t *out)
{
  const double top = (double) (1u << md);
  for (int64_t i = 0; i < n; i++)
    for (int d = 0; d < dim; d++) {
      const uint64_t k = (uint64_t) (i * dim + d);
      double a = u01(seed, 2 * k), b = u01(seed, 2 * k + 1);
      if (a <= 0.0) a = 1e-300;
      double z = std::sqrt(-2.0 * std::log(a)) * std::cos(2.0 * M_PI * b);
      double v = mean + sd * z;
      v = std::min(std::max(v, 0.0), 1.0 - std::ldexp(1.0, -md));
      out[i * dim + d] = (uint32_t) std::floor(v * top);
    }
}

static inline uint64_t ckey(const Cell &c, int dim, int md)
{
  uint64_t k = (uint64_t) c.lev;
  for (int d = dim - 1; d >= 0; d--) k = (k << md) | c.x[d];
  return k;
}
static inline Cell cdecode(uint64_t k, int dim, int md)
{
  Cell c;
  const uint64_t m = (1ull << md) - 1;
  for (int d = 0; d < dim; d++) { c.x[d] = (uint32_t) (k & m); k >>= md; }
  c.lev = (int) k;
  return c;
}
static inline Cell cparent(const Cell &c, int md)
{
  Cell p = c;
  p.lev = c.lev - 1;
  const uint32_t mask = ~((1u << (md - p.lev)) - 1u);
  for (int d = 0; d < 4; d++) p.x[d] &= mask;
  return p;
}

// Complete tree in which every leaf above level md holds at most max_pts
// points (locTreeConstruction): recursive split of Morton-sorted points.
static void construct(const std::vector<uint64_t> &pk, size_t b, size_t e, const Cell &c, int dim, int md,
                      int64_t max_pts, std::vector<Cell> &leaves)
{
  const int nc = 1 << dim;
  // points are sorted by interleaved Morton key of full resolution
  for (int ch = 0; ch < nc; ch++) {
    Cell k = c;
    k.lev = c.lev + 1;
    const uint32_t cl = 1u << (md - k.lev);
    for (int d = 0; d < dim; d++) k.x[d] = c.x[d] | (((ch >> d) & 1) ? cl : 0u);
    // key range of the child: interleaved prefix
    uint64_t lo = 0;
    for (int bit = md - 1; bit >= 0; bit--)
      for (int d = dim - 1; d >= 0; d--) lo = (lo << 1) | ((k.x[d] >> bit) & 1u);
    const int shift = dim * (md - k.lev);
    const uint64_t hi = lo + (shift >= 64 ? ~0ull : ((1ull << shift) - 1ull));
    const size_t cb = std::lower_bound(pk.begin() + b, pk.begin() + e, lo) - pk.begin();
    const size_t ce = std::upper_bound(pk.begin() + cb, pk.begin() + e, hi) - pk.begin();
    if ((int64_t) (ce - cb) > max_pts && k.lev < md) construct(pk, cb, ce, k, dim, md, max_pts, leaves);
    else leaves.push_back(k);
  }
}

// 2:1 balancing with the semantics of propagateNeighbours + reconstruction
// (src/tsort.cpp:777-854): S = leaves closed under "parent and the parent's
// in-domain neighbours"; the balanced tree's leaves are the children of the
// parents of S-cells that are not themselves parents of S-cells.
static std::vector<Cell> balance(const std::vector<Cell> &leaves, int dim, int md)
{
  std::vector<std::unordered_set<uint64_t>> S(md + 1);
  for (const Cell &c : leaves) S[c.lev].insert(ckey(c, dim, md));
  int n3 = 1;
  for (int d = 0; d < dim; d++) n3 *= 3;
  const uint64_t top = 1ull << md;
  for (int l = md; l > 0; l--) {
    std::vector<uint64_t> cur(S[l].begin(), S[l].end());
    for (uint64_t k : cur) {
      const Cell p = cparent(cdecode(k, dim, md), md);
      const uint64_t len = 1ull << (md - p.lev);
      for (int idx = 0; idx < n3; idx++) {
        Cell nb = p;
        bool ok = true;
        int r = idx;
        for (int d = 0; d < dim && ok; d++) {
          const int delta = r % 3;
          r /= 3;
          if (delta == 1) { if (p.x[d] + len >= top) ok = false; else nb.x[d] = (uint32_t) (p.x[d] + len); }
          else if (delta == 2) { if (p.x[d] < len) ok = false; else nb.x[d] = (uint32_t) (p.x[d] - len); }
        }
        if (ok) S[p.lev].insert(ckey(nb, dim, md));
      }
    }
  }
  std::unordered_set<uint64_t> I;
  for (int l = 1; l <= md; l++)
    for (uint64_t k : S[l]) I.insert(ckey(cparent(cdecode(k, dim, md), md), dim, md));
  std::vector<Cell> out;
  const int nc = 1 << dim;
  for (uint64_t k : I) {
    const Cell c = cdecode(k, dim, md);
    const uint32_t cl = 1u << (md - c.lev - 1);
    for (int ch = 0; ch < nc; ch++) {
      Cell kc = c;
      kc.lev = c.lev + 1;
      for (int d = 0; d < dim; d++) kc.x[d] = c.x[d] | (((ch >> d) & 1) ? cl : 0u);
      if (!I.count(ckey(kc, dim, md))) out.push_back(kc);
    }
  }
  return out;
}

static uint64_t morton_full(const uint32_t *x, int dim, int md)
{
  uint64_t k = 0;
  for (int bit = md - 1; bit >= 0; bit--)
    for (int d = dim - 1; d >= 0; d--) k = (k << 1) | ((x[d] >> bit) & 1u);
  return k;
}

// Points -> 2:1-balanced complete tree (unsorted cells; the DA sorts them).
std::vector<Cell> tree_from_points(const uint32_t *pts, int64_t n, int dim, int md, int64_t max_pts)
{
  if (dim * md > 64) throw std::invalid_argument("dim*max_depth must be <= 64");
  std::vector<uint64_t> pk(n);
  for (int64_t i = 0; i < n; i++) pk[i] = morton_full(pts + i * dim, dim, md);
  std::sort(pk.begin(), pk.end());
  Cell root{};
  root.lev = 0;
  std::vector<Cell> leaves;
  if ((int64_t) pk.size() > max_pts) construct(pk, 0, pk.size(), root, dim, md, max_pts, leaves);
  else {
    const int nc = 1 << dim;
    for (int ch = 0; ch < nc; ch++) {
      Cell k{};
      k.lev = 1;
      for (int d = 0; d < dim; d++) k.x[d] = ((ch >> d) & 1) ? (1u << (md - 1)) : 0u;
      leaves.push_back(k);
    }
  }
  return balance(leaves, dim, md);
}

// Spacetime moving ball (dim 4: x, y, z, t): refine every cell whose box meets
// the shell | |(x,y,z) - c(t)| - R | <= w, c(t) = c0 + (c1 - c0) t, down to
// `level`, then 2:1 balance.  For a cell [lo,hi]^3 x [t0,t1] the distance from
// c(t) to the spatial box is convex in t (its square is a sum of squared
// clamped linear functions), so its minimum over [t0,t1] is found by golden
// section search; the largest distance to the box is convex too, so its
// maximum sits at t0 or t1.  The cell meets the shell iff
// min-distance <= R + w and max-distance >= R - w.
static double box_dist(const double *lo, const double *hi, const double *c)
{
  double s = 0.0;
  for (int d = 0; d < 3; d++) {
    const double g = c[d] < lo[d] ? lo[d] - c[d] : (c[d] > hi[d] ? c[d] - hi[d] : 0.0);
    s += g * g;
  }
  return std::sqrt(s);
}
static double box_far(const double *lo, const double *hi, const double *c)
{
  double s = 0.0;
  for (int d = 0; d < 3; d++) {
    const double f = std::max(std::fabs(c[d] - lo[d]), std::fabs(hi[d] - c[d]));
    s += f * f;
  }
  return std::sqrt(s);
}

static void ball_refine(const Cell &c, int md, int level, double R, double w, const double *c0, const double *c1,
                        std::vector<Cell> &leaves)
{
  const double s = std::ldexp(1.0, -md);
  const double h = std::ldexp(1.0, -c.lev);
  double lo[3], hi[3];
  for (int d = 0; d < 3; d++) { lo[d] = c.x[d] * s; hi[d] = lo[d] + h; }
  const double t0 = c.x[3] * s, t1 = t0 + h;
  auto centre = [&](double t, double *out) { for (int d = 0; d < 3; d++) out[d] = c0[d] + (c1[d] - c0[d]) * t; };
  double ca[3], cb[3];
  centre(t0, ca);
  centre(t1, cb);
  const double dmax = std::max(box_far(lo, hi, ca), box_far(lo, hi, cb));
  double a = t0, b = t1;
  const double gr = 0.5 * (std::sqrt(5.0) - 1.0);
  for (int it = 0; it < 80; it++) {
    const double m1 = b - gr * (b - a), m2 = a + gr * (b - a);
    double p1[3], p2[3];
    centre(m1, p1);
    centre(m2, p2);
    if (box_dist(lo, hi, p1) <= box_dist(lo, hi, p2)) b = m2; else a = m1;
  }
  double pm[3];
  centre(0.5 * (a + b), pm);
  const double dmin = std::min({box_dist(lo, hi, pm), box_dist(lo, hi, ca), box_dist(lo, hi, cb)});
  const bool meets = (dmin <= R + w) && (dmax >= R - w);
  if (meets && c.lev < level) {
    for (int ch = 0; ch < 16; ch++) {
      Cell k = c;
      k.lev = c.lev + 1;
      const uint32_t cl = 1u << (md - k.lev);
      for (int d = 0; d < 4; d++) k.x[d] = c.x[d] | (((ch >> d) & 1) ? cl : 0u);
      ball_refine(k, md, level, R, w, c0, c1, leaves);
    }
  } else {
    leaves.push_back(c);
  }
}

std::vector<Cell> moving_ball_tree(int md, int level, double R, double w, const double *c0, const double *c1)
{
  Cell root{};
  root.lev = 0;
  std::vector<Cell> leaves;
  ball_refine(root, md, level, R, w, c0, c1, leaves);
  return balance(leaves, 4, md);
}

// Static sphere shell in dim 2..4 (same arithmetic as the device test).
static void shell_refine(const Cell &c, int dim, int md, int level, double R, double w, const double *ctr,
                         std::vector<Cell> &leaves)
{
  const double sc = std::ldexp(1.0, -md), h = std::ldexp(1.0, -(int) c.lev);
  double s_near = 0.0, s_far = 0.0;
  for (int d = 0; d < dim; d++) {
    const double lo = (double) c.x[d] * sc, hi = lo + h;
    const double g = ctr[d] < lo ? lo - ctr[d] : (ctr[d] > hi ? ctr[d] - hi : 0.0);
    const double f = std::max(std::fabs(ctr[d] - lo), std::fabs(hi - ctr[d]));
    s_near = s_near + g * g;
    s_far = s_far + f * f;
  }
  const bool meets = (std::sqrt(s_near) <= R + w) && (std::sqrt(s_far) >= R - w);
  if (!meets || (int) c.lev >= level) { leaves.push_back(c); return; }
  const uint32_t cl = 1u << (md - c.lev - 1);
  for (int ch = 0; ch < (1 << dim); ch++) {
    Cell k = c;
    k.lev = c.lev + 1;
    for (int d = 0; d < dim; d++) k.x[d] = c.x[d] | (((ch >> d) & 1) ? cl : 0u);
    shell_refine(k, dim, md, level, R, w, ctr, leaves);
  }
}

// ---------------------------------------------------------------------------
// Harmonious Hilbert curve (H. Haverkort, "Harmonious Hilbert curves and other
// extradimensional space-filling curves", 2012; refinement rule of p. 23).
//
// A cell orientation is a symmetry of the cube: an axis permutation followed
// by a reflection.  Here it is held as its action on the 2^K child indices of
// a cell (Morton numbers), so composing two orientations is composing two
// index maps.  The refinement rule says, for the child with curve rank r of
// a cell in the canonical orientation, where it sits and how it is oriented:
//   position  g(r) = r xor (r >> 1)                      (reflected Gray code)
//   mirror    0 for r = 0, else g(r-1) with its last bit set to not(last bit of g(r))
//   axes      reading the bits of r from the most significant one, a bit that
//             differs from r's last bit sends its axis to the front block
//             (filled from the back), the others to the back block
// (Haverkort numbers bits from the left, so his index i is integer bit K-1-i.)
// The table for an orientation O then lists, for every rank r, the Morton
// child O(g(r)) and the orientation O composed with the child's.
// ---------------------------------------------------------------------------
namespace {
using ChildMap = std::array<uint8_t, 16>;   // action on child indices (K <= 4)

ChildMap haverkort_child(int K, unsigned r, unsigned &pos)
{
  pos = r ^ (r >> 1);
  unsigned mirror = 0;
  if (r > 0) {
    const unsigned g = (r - 1) ^ ((r - 1) >> 1);
    mirror = (g & ~1u) | (~pos & 1u);
  }
  // destination (Haverkort index, from the left) of every source axis
  int dest[4];
  const unsigned last = r & 1u;
  int front = 0;
  for (int i = 0; i < K; i++) front += (((r >> (K - 1 - i)) & 1u) != last);
  int fpos = front - 1, bpos = K - 1;
  for (int i = 0; i < K; i++) dest[i] = (((r >> (K - 1 - i)) & 1u) != last) ? fpos-- : bpos--;
  // action: output bit (from the left) i takes input bit dest[i], then the mirror
  ChildMap m{};
  for (unsigned x = 0; x < (1u << K); x++) {
    unsigned y = 0;
    for (int i = 0; i < K; i++) y = (y << 1) | ((x >> (K - 1 - dest[i])) & 1u);
    m[x] = (uint8_t) (y ^ mirror);
  }
  return m;
}
}  // namespace

void hilbert_tables(int K, std::vector<int8_t> &rot, std::vector<int32_t> &ht, int &nrot)
{
  if (K < 2 || K > 4) throw std::invalid_argument("Hilbert tables: dim must be 2..4");
  const unsigned nc = 1u << K;
  unsigned pos[16];
  ChildMap child[16];
  for (unsigned r = 0; r < nc; r++) child[r] = haverkort_child(K, r, pos[r]);
  ChildMap id{};
  for (unsigned x = 0; x < nc; x++) id[x] = (uint8_t) x;
  // every orientation reachable from the identity, numbered in discovery order
  std::vector<ChildMap> orients{id};
  auto index_of = [&](const ChildMap &m) -> int {
    for (size_t k = 0; k < orients.size(); k++)
      if (std::equal(m.begin(), m.begin() + nc, orients[k].begin())) return (int) k;
    orients.push_back(m);
    return (int) orients.size() - 1;
  };
  rot.clear();
  ht.clear();
  for (size_t o = 0; o < orients.size(); o++) {
    const ChildMap O = orients[o];
    std::vector<int8_t> row(2 * nc);
    std::vector<int32_t> hrow(nc);
    for (unsigned r = 0; r < nc; r++) {
      const unsigned morton = O[pos[r]];
      ChildMap c{};
      for (unsigned x = 0; x < nc; x++) c[x] = O[child[r][x]];
      row[r] = (int8_t) morton;
      row[nc + morton] = (int8_t) r;
      hrow[morton] = index_of(c);
    }
    rot.insert(rot.end(), row.begin(), row.end());
    ht.insert(ht.end(), hrow.begin(), hrow.end());
  }
  nrot = (int) orients.size();
}

std::vector<Cell> sphere_shell_tree(int dim, int md, int level, double R, double w, const double *ctr)
{
  Cell root{};
  root.lev = 0;
  std::vector<Cell> leaves;
  shell_refine(root, dim, md, level, R, w, ctr, leaves);
  return balance(leaves, dim, md);
}

// ---------------------------------------------------------------------------
// VTU output of an octree: io::vtk::oct2vtu (IO/vtk/include/oct2vtk.h:272-273,
// IO/vtk/src/oct2vtk.cpp:1530-1800).  The reference's arrays, names and types:
// one cell per octant with its own 2^dim corner points (integer lattice
// coordinates, UInt32, x fastest, z = 0 in 2D), UInt64 connectivity and
// offsets, UInt8 cell types (VTK hexahedra in 3D; quads in 2D, where the
// reference has no instantiation), and the cell data mpi_rank and cell_level
// (UInt32; rank 0: one process writes the whole tree); optionally one Float64
// value per cell after them.  Inline base64 "binary" data arrays with a
// UInt32 byte-count header (the reference's binary branch repeats the
// connectivity block once per cell, oct2vtk.cpp:1670-1690, so its ASCII
// branch is the one these arrays follow).
// ---------------------------------------------------------------------------
namespace {
std::string base64(const std::vector<uint8_t> &in)
{
  static const char *tab = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
  std::string out;
  out.reserve((in.size() + 2) / 3 * 4);
  size_t i = 0;
  for (; i + 2 < in.size(); i += 3) {
    const uint32_t v = (uint32_t) in[i] << 16 | (uint32_t) in[i + 1] << 8 | in[i + 2];
    out += tab[v >> 18]; out += tab[(v >> 12) & 63]; out += tab[(v >> 6) & 63]; out += tab[v & 63];
  }
  if (i < in.size()) {
    const uint32_t v = (uint32_t) in[i] << 16 | (i + 1 < in.size() ? (uint32_t) in[i + 1] << 8 : 0u);
    out += tab[v >> 18]; out += tab[(v >> 12) & 63];
    out += i + 1 < in.size() ? tab[(v >> 6) & 63] : '=';
    out += '=';
  }
  return out;
}
template <typename T>
std::string vtu_block(const std::vector<T> &v)
{
  const uint32_t nbytes = (uint32_t) (v.size() * sizeof(T));
  std::vector<uint8_t> raw(4 + (size_t) nbytes);
  for (int b = 0; b < 4; b++) raw[b] = (uint8_t) (nbytes >> (8 * b));   // little endian
  if (nbytes) std::memcpy(raw.data() + 4, v.data(), nbytes);
  return base64(raw);
}
}  // namespace

void write_vtu(const char *path, int dim, int md, const uint32_t *coords, const uint8_t *levels, int64_t n,
               const double *cell_values, const char *cell_values_name)
{
  if (dim != 2 && dim != 3) throw std::invalid_argument("VTU output is defined for dim 2 and 3");
  if (n < 0 || (uint64_t) n * (1u << dim) > 0xFFFFFFFFull / 12) throw std::invalid_argument("too many cells for one VTU piece");
  const int nv = 1 << dim;
  std::vector<uint32_t> pts((size_t) n * nv * 3);
  std::vector<uint64_t> conn((size_t) n * nv), offs(n);
  std::vector<uint32_t> rank(n, 0u), lev(n);
  std::vector<uint8_t> types(n, (uint8_t) (dim == 3 ? 12 : 9));   // VTK_HEXAHEDRON, VTK_QUAD
  // corner order of the VTK cell types: counter-clockwise in each z-layer
  static const int ci[8] = {0, 1, 3, 2, 4, 5, 7, 6};
  for (int64_t e = 0; e < n; e++) {
    if ((int) levels[e] > md) throw std::invalid_argument("cell level exceeds max_depth");
    const uint32_t len = 1u << (md - levels[e]);
    for (int k = 0; k < nv; k++)
      for (int d = 0; d < 3; d++)
        pts[((size_t) e * nv + k) * 3 + d] = d < dim ? coords[e * dim + d] + (((k >> d) & 1) ? len : 0u) : 0u;
    for (int k = 0; k < nv; k++) conn[(size_t) e * nv + k] = (uint64_t) (e * nv + ci[k]);
    offs[e] = (uint64_t) (e + 1) * nv;
    lev[e] = levels[e];
  }
  std::FILE *fp = std::fopen(path, "w");
  if (!fp) throw std::runtime_error(std::string("cannot open ") + path);
  std::fprintf(fp, "<?xml version=\"1.0\"?>\n");
  std::fprintf(fp, "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\" header_type=\"UInt32\">\n");
  std::fprintf(fp, "  <UnstructuredGrid>\n");
  std::fprintf(fp, "    <Piece NumberOfPoints=\"%lld\" NumberOfCells=\"%lld\">\n", (long long) n * nv, (long long) n);
  std::fprintf(fp, "      <Points>\n");
  std::fprintf(fp, "        <DataArray type=\"UInt32\" Name=\"Position\" NumberOfComponents=\"3\" format=\"binary\">\n");
  std::fprintf(fp, "          %s\n        </DataArray>\n      </Points>\n", vtu_block(pts).c_str());
  std::fprintf(fp, "      <Cells>\n");
  std::fprintf(fp, "        <DataArray type=\"UInt64\" Name=\"connectivity\" format=\"binary\">\n");
  std::fprintf(fp, "          %s\n        </DataArray>\n", vtu_block(conn).c_str());
  std::fprintf(fp, "        <DataArray type=\"UInt64\" Name=\"offsets\" format=\"binary\">\n");
  std::fprintf(fp, "          %s\n        </DataArray>\n", vtu_block(offs).c_str());
  std::fprintf(fp, "        <DataArray type=\"UInt8\" Name=\"types\" format=\"binary\">\n");
  std::fprintf(fp, "          %s\n        </DataArray>\n      </Cells>\n", vtu_block(types).c_str());
  if (cell_values)
    std::fprintf(fp, "      <CellData Scalars=\"%s\">\n", cell_values_name ? cell_values_name : "value");
  else
    std::fprintf(fp, "      <CellData>\n");
  std::fprintf(fp, "        <DataArray type=\"UInt32\" Name=\"mpi_rank\" format=\"binary\">\n");
  std::fprintf(fp, "          %s\n        </DataArray>\n", vtu_block(rank).c_str());
  std::fprintf(fp, "        <DataArray type=\"UInt32\" Name=\"cell_level\" format=\"binary\">\n");
  std::fprintf(fp, "          %s\n        </DataArray>\n", vtu_block(lev).c_str());
  if (cell_values) {
    std::vector<double> cv(cell_values, cell_values + n);
    std::fprintf(fp, "        <DataArray type=\"Float64\" Name=\"%s\" format=\"binary\">\n",
                 cell_values_name ? cell_values_name : "value");
    std::fprintf(fp, "          %s\n        </DataArray>\n", vtu_block(cv).c_str());
  }
  std::fprintf(fp, "      </CellData>\n");
  std::fprintf(fp, "    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n");
  const bool bad = std::ferror(fp) != 0;
  std::fclose(fp);
  if (bad) throw std::runtime_error(std::string("write error on ") + path);
}

}  // namespace dkt
