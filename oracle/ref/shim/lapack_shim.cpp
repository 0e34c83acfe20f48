// Minimal replacements for the two LAPACK routines the reference calls
// (FEM/include/lapac.h:22-23): dgesv_ (LU with partial pivoting) and dsyev_
// (symmetric eigensolver, here cyclic Jacobi rotations).  Written from the
// textbook algorithms; column-major Fortran calling convention.  Test
// infrastructure for building the reference as a CPU oracle only.
#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>

extern "C" void dgesv_(int *n_, int *nrhs_, double *a, int *lda_, int *ipiv, double *b, int *ldb_, int *info)
{
  const int n = *n_, nrhs = *nrhs_, lda = *lda_, ldb = *ldb_;
  *info = 0;
  for (int k = 0; k < n; k++) {
    int p = k;
    double best = std::fabs(a[k + k * lda]);
    for (int i = k + 1; i < n; i++)
      if (std::fabs(a[i + k * lda]) > best) { best = std::fabs(a[i + k * lda]); p = i; }
    ipiv[k] = p + 1;
    if (best == 0.0) { if (*info == 0) *info = k + 1; continue; }
    if (p != k) {
      for (int j = 0; j < n; j++) std::swap(a[k + j * lda], a[p + j * lda]);
      for (int j = 0; j < nrhs; j++) std::swap(b[k + j * ldb], b[p + j * ldb]);
    }
    for (int i = k + 1; i < n; i++) {
      double f = a[i + k * lda] / a[k + k * lda];
      a[i + k * lda] = f;
      for (int j = k + 1; j < n; j++) a[i + j * lda] -= f * a[k + j * lda];
      for (int j = 0; j < nrhs; j++) b[i + j * ldb] -= f * b[k + j * ldb];
    }
  }
  if (*info) return;
  for (int j = 0; j < nrhs; j++)
    for (int i = n - 1; i >= 0; i--) {
      double s = b[i + j * ldb];
      for (int c = i + 1; c < n; c++) s -= a[i + c * lda] * b[c + j * ldb];
      b[i + j * ldb] = s / a[i + i * lda];
    }
}

extern "C" void dsyev_(char *jobz, char *uplo, int *n_, double *a, int *lda_, double *w, double *work, int *lwork, int *info)
{
  const int n = *n_, lda = *lda_;
  *info = 0;
  if (*lwork == -1) { work[0] = 3.0 * n; return; }
  std::vector<double> A(n * n), V(n * n, 0.0);
  const bool upper = (uplo[0] == 'U' || uplo[0] == 'u');
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) {
      bool stored = upper ? (i <= j) : (i >= j);
      A[i + j * n] = stored ? a[i + j * lda] : a[j + i * lda];
    }
  for (int i = 0; i < n; i++) V[i + i * n] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0;
    for (int j = 0; j < n; j++) for (int i = 0; i < n; i++) if (i != j) off += A[i + j * n] * A[i + j * n];
    if (off < 1e-300) break;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) {
        double apq = A[p + q * n];
        if (apq == 0.0) continue;
        double theta = (A[q + q * n] - A[p + p * n]) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; k++) {
          double akp = A[k + p * n], akq = A[k + q * n];
          A[k + p * n] = c * akp - s * akq;
          A[k + q * n] = s * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {
          double apk = A[p + k * n], aqk = A[q + k * n];
          A[p + k * n] = c * apk - s * aqk;
          A[q + k * n] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; k++) {
          double vkp = V[k + p * n], vkq = V[k + q * n];
          V[k + p * n] = c * vkp - s * vkq;
          V[k + q * n] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> order(n);
  for (int i = 0; i < n; i++) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int x, int y) { return A[x + x * n] < A[y + y * n]; });
  for (int k = 0; k < n; k++) {
    int src = order[k];
    w[k] = A[src + src * n];
    if (jobz[0] == 'V' || jobz[0] == 'v')
      for (int i = 0; i < n; i++) a[i + k * lda] = V[i + src * n];
  }
}
