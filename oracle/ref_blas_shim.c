/* BLAS/LAPACK entry points the GCGE-1.0 sources call (src/gcge_ops.h:217-241),
 * forwarded to SciPy's bundled OpenBLAS, whose symbols carry a scipy_ prefix.
 * Used only by the oracle/_ref build (test infrastructure). */
extern void scipy_dsyevx_(char *, char *, char *, int *, double *, int *, double *, double *,
                          int *, int *, double *, int *, double *, double *, int *, double *,
                          int *, int *, int *, int *);
extern void scipy_dgemm_(char *, char *, int *, int *, int *, double *, double *, int *, double *,
                         int *, double *, double *, int *);
extern void scipy_dsymm_(char *, char *, int *, int *, double *, double *, int *, double *, int *,
                         double *, double *, int *);
extern void scipy_daxpy_(int *, double *, double *, int *, double *, int *);
extern double scipy_ddot_(int *, double *, int *, double *, int *);
extern double scipy_dnrm2_(int *, double *, int *);
extern void scipy_dscal_(int *, double *, double *, int *);
extern void scipy_dcopy_(int *, double *, int *, double *, int *);

void dsyevx_(char *jobz, char *range, char *uplo, int *n, double *a, int *lda, double *vl, double *vu,
             int *il, int *iu, double *abstol, int *m, double *w, double *z, int *ldz, double *work,
             int *lwork, int *iwork, int *ifail, int *info)
{ scipy_dsyevx_(jobz, range, uplo, n, a, lda, vl, vu, il, iu, abstol, m, w, z, ldz, work, lwork, iwork, ifail, info); }
void dgemm_(char *ta, char *tb, int *m, int *n, int *k, double *al, double *a, int *lda, double *b,
            int *ldb, double *be, double *c, int *ldc)
{ scipy_dgemm_(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc); }
void dsymm_(char *s, char *u, int *m, int *n, double *al, double *a, int *lda, double *b, int *ldb,
            double *be, double *c, int *ldc)
{ scipy_dsymm_(s, u, m, n, al, a, lda, b, ldb, be, c, ldc); }
void daxpy_(int *n, double *a, double *x, int *ix, double *y, int *iy) { scipy_daxpy_(n, a, x, ix, y, iy); }
double ddot_(int *n, double *x, int *ix, double *y, int *iy) { return scipy_ddot_(n, x, ix, y, iy); }
double dnrm2_(int *n, double *x, int *ix) { return scipy_dnrm2_(n, x, ix); }
void dscal_(int *n, double *a, double *x, int *ix) { scipy_dscal_(n, a, x, ix); }
void dcopy_(int *n, double *x, int *ix, double *y, int *iy) { scipy_dcopy_(n, x, ix, y, iy); }
