/*
 * Stand-in for Intel MKL's mkl.h -- TEST INFRASTRUCTURE ONLY.  It declares just what
 * the reference's driver ("wersja referencyjna/Wire_MoM.cu") uses from MKL, so that
 * its unmodified source compiles here for the link test: the MKL_Complex16 type and
 * the LAPACKE pair it calls (Wire_MoM.cu:372,382).  oracle/shim/lapacke_oracle.c
 * implements the pair with the oracle's unblocked LU.
 */
#ifndef WMOM_ORACLE_SHIM_MKL_H
#define WMOM_ORACLE_SHIM_MKL_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  double real, imag;
} MKL_Complex16;
typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

lapack_int LAPACKE_zgetrf(int matrix_layout, lapack_int m, lapack_int n, MKL_Complex16* a, lapack_int lda,
                          lapack_int* ipiv);
lapack_int LAPACKE_zgetrs(int matrix_layout, char trans, lapack_int n, lapack_int nrhs, const MKL_Complex16* a,
                          lapack_int lda, const lapack_int* ipiv, MKL_Complex16* b, lapack_int ldb);

#ifdef __cplusplus
}
#endif

#endif
