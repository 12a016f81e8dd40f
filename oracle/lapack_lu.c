/*
 * lapack_lu.c -- the two LAPACK routines the reference's determinant code
 * calls, written for this project (LAPACK is not installed here).
 *
 * TEST INFRASTRUCTURE ONLY: linked into the oracle builds of the reference's
 * full_determinant.c and tests/thirring_brute.c (oracle/make_ref.py), never
 * into the product.
 *
 * Same calling convention as LAPACK's dgetrf / dgetri: column-major storage
 * (element (i, j) at a[i + j*lda]), 1-based pivot indices, info = 0 on success
 * and info = k > 0 when U(k, k) is exactly zero.  The algorithm is the
 * textbook right-looking LU with partial pivoting (Golub & Van Loan,
 * "Matrix Computations", algorithm 3.4.1) and the inverse is formed column by
 * column from the factors, so results agree with LAPACK's to rounding, and a
 * determinant taken as the product of U's diagonal times the pivot signs is
 * the same number.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

void LAPACK_dgetrf(int* m, int* n, double* a, int* lda, int* ipiv, int* info) {
  const int M = *m, N = *n, ld = *lda;
  const int K = M < N ? M : N;
  *info = 0;
  for (int k = 0; k < K; k++) {
    int p = k;
    double best = fabs(a[k + k * ld]);
    for (int i = k + 1; i < M; i++) {
      const double v = fabs(a[i + k * ld]);
      if (v > best) {
        best = v;
        p = i;
      }
    }
    ipiv[k] = p + 1;
    if (a[p + k * ld] == 0.0) {
      if (*info == 0) *info = k + 1;
      continue;
    }
    if (p != k)
      for (int j = 0; j < N; j++) {
        const double t = a[k + j * ld];
        a[k + j * ld] = a[p + j * ld];
        a[p + j * ld] = t;
      }
    const double inv = 1.0 / a[k + k * ld];
    for (int i = k + 1; i < M; i++) a[i + k * ld] *= inv;
    for (int j = k + 1; j < N; j++) {
      const double u = a[k + j * ld];
      if (u == 0.0) continue;
      for (int i = k + 1; i < M; i++) a[i + j * ld] -= a[i + k * ld] * u;
    }
  }
}

/* A^-1 from the factors of LAPACK_dgetrf: solve L U X = P I column by column. */
void LAPACK_dgetri(int* n, double* a, int* lda, int* ipiv, double* work, int* lwork, int* info) {
  (void)work;
  (void)lwork;
  const int N = *n, ld = *lda;
  *info = 0;
  for (int k = 0; k < N; k++)
    if (a[k + k * ld] == 0.0) {
      *info = k + 1;
      return;
    }
  double* inv = malloc((size_t)N * N * sizeof(double));
  double* col = malloc((size_t)N * sizeof(double));
  for (int j = 0; j < N; j++) {
    memset(col, 0, (size_t)N * sizeof(double));
    col[j] = 1.0;
    for (int k = 0; k < N; k++) { /* row interchanges in factorisation order */
      const int p = ipiv[k] - 1;
      if (p != k) {
        const double t = col[k];
        col[k] = col[p];
        col[p] = t;
      }
    }
    for (int i = 0; i < N; i++) /* L y = b, unit diagonal */
      for (int k = 0; k < i; k++) col[i] -= a[i + k * ld] * col[k];
    for (int i = N - 1; i >= 0; i--) { /* U x = y */
      for (int k = i + 1; k < N; k++) col[i] -= a[i + k * ld] * col[k];
      col[i] /= a[i + i * ld];
    }
    for (int i = 0; i < N; i++) inv[i + j * N] = col[i];
  }
  for (int j = 0; j < N; j++)
    for (int i = 0; i < N; i++) a[i + j * ld] = inv[i + j * N];
  free(col);
  free(inv);
}
