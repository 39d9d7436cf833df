/*
 * LAPACKE_zgetrf / LAPACKE_zgetrs for the link test of the reference's driver --
 * TEST INFRASTRUCTURE ONLY: column-major, one square matrix, transposition 'N',
 * implemented with the oracle's unblocked LU (oracle/wmom_oracle.c), so that the
 * linked program needs no MKL.  Other layouts or shapes return -1.
 */
#include <stddef.h>

#include "mkl.h"

int oracle_zgetf2(int n, double* a, int lda, int* ipiv);
void oracle_zgetrs(int n, const double* lu, int lda, const int* ipiv, double* b);

lapack_int LAPACKE_zgetrf(int matrix_layout, lapack_int m, lapack_int n, MKL_Complex16* a, lapack_int lda,
                          lapack_int* ipiv) {
  if (matrix_layout != LAPACK_COL_MAJOR || m != n || lda < n) return -1;
  return oracle_zgetf2(n, (double*)a, lda, ipiv);
}

lapack_int LAPACKE_zgetrs(int matrix_layout, char trans, lapack_int n, lapack_int nrhs, const MKL_Complex16* a,
                          lapack_int lda, const lapack_int* ipiv, MKL_Complex16* b, lapack_int ldb) {
  if (matrix_layout != LAPACK_COL_MAJOR || (trans != 'n' && trans != 'N') || lda < n || ldb < n) return -1;
  for (lapack_int r = 0; r < nrhs; ++r) oracle_zgetrs(n, (const double*)a, lda, ipiv, (double*)(b + (size_t)r * ldb));
  return 0;
}
