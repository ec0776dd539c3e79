/*
 * lapack_shim.c -- the three BLAS/LAPACK routines the reference's matrix
 * class calls (matrix.cpp:528-636), forwarded to the OpenBLAS build that
 * ships with scipy (its symbols carry a scipy_ prefix).  TEST INFRASTRUCTURE ONLY.
 */
void scipy_dgemm_(char *, char *, int *, int *, int *, double *, const double *, int *, const double *, int *,
                  double *, double *, int *);
void scipy_dgetrf_(int *, int *, double *, int *, int *, int *);
void scipy_dgetri_(int *, double *, int *, int *, double *, int *, int *);

void dgemm_(char *ta, char *tb, int *m, int *n, int *k, double *alpha, const double *a, int *lda, const double *b,
            int *ldb, double *beta, double *c, int *ldc)
{
    scipy_dgemm_(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

void dgetrf_(int *m, int *n, double *a, int *lda, int *ipiv, int *info) { scipy_dgetrf_(m, n, a, lda, ipiv, info); }

void dgetri_(int *n, double *a, int *lda, int *ipiv, double *work, int *lwork, int *info)
{
    scipy_dgetri_(n, a, lda, ipiv, work, lwork, info);
}
