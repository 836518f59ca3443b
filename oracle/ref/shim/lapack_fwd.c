/*
 * LAPACK entry points the reference declares in lapack_we_use.h (without the
 * trailing underscore, except dpotrf_/dpotri_), forwarded to the
 * scipy_-prefixed Fortran-ABI routines of the OpenBLAS build that scipy
 * bundles in this image. Test infrastructure for oracle/_ref only.
 */


extern void scipy_dgeev_(char *, char *, int *, double *, int *, double *, double *, double *, int *, double *, int *, double *, int *, int *);
extern void scipy_dgetrf_(int *, int *, double *, int *, int *, int *);
extern void scipy_dgetri_(int *, double *, int *, int *, double *, int *, int *);
extern void scipy_dsyev_(char *, char *, int *, double *, int *, double *, double *, int *, int *);
extern void scipy_dpotrf_(char *, int *, double *, int *, int *);
extern void scipy_dpotri_(char *, int *, double *, int *, int *);
extern void scipy_dposv_(char *, int *, int *, double *, int *, double *, int *, int *);
extern void scipy_dgesv_(int *, int *, double *, int *, int *, double *, int *, int *);
extern void scipy_dgemv_(char *, int *, int *, double *, double *, int *, double *, int *, double *, double *, int *);
extern void scipy_dgemm_(char *, char *, int *, int *, int *, double *, double *, int *, double *, int *, double *, double *, int *);
extern void scipy_dsytrf_(char *, int *, double *, int *, int *, double *, int *, int *);
extern void scipy_dsytri_(char *, int *, double *, int *, int *, double *, int *);

void dgeev(char *jobvl, char *jobvr, int *n, double *a, int *lda, double *wr, double *wi, double *vl, int *ldvl,
           double *vr, int *ldvr, double *work, int *lwork, int *info)
{ scipy_dgeev_(jobvl, jobvr, n, a, lda, wr, wi, vl, ldvl, vr, ldvr, work, lwork, info); }
void dgetrf(int *m, int *n, double *a, int *lda, int *ipiv, int *info) { scipy_dgetrf_(m, n, a, lda, ipiv, info); }
void dgetri(int *n, double *a, int *lda, int *ipiv, double *work, int *lwork, int *info)
{ scipy_dgetri_(n, a, lda, ipiv, work, lwork, info); }
void dsyev(char *jobz, char *uplo, int *n, double *a, int *lda, double *w, double *work, int *lwork, int *info)
{ scipy_dsyev_(jobz, uplo, n, a, lda, w, work, lwork, info); }
void dpotrf_(char *uplo, int *n, double *a, int *lda, int *info) { scipy_dpotrf_(uplo, n, a, lda, info); }
void dpotri_(char *uplo, int *n, double *a, int *lda, int *info) { scipy_dpotri_(uplo, n, a, lda, info); }
void dposv(char *uplo, int *n, int *nrhs, double *a, int *lda, double *b, int *ldb, int *info)
{ scipy_dposv_(uplo, n, nrhs, a, lda, b, ldb, info); }
void dgesv(int *n, int *nrhs, double *a, int *lda, int *ipiv, double *b, int *ldb, int *info)
{ scipy_dgesv_(n, nrhs, a, lda, ipiv, b, ldb, info); }
void dgemv(char *t, int *m, int *n, double *al, double *a, int *lda, double *x, int *ix, double *be, double *y, int *iy)
{ scipy_dgemv_(t, m, n, al, a, lda, x, ix, be, y, iy); }
void dgemm(char *ta, char *tb, int *m, int *n, int *k, double *al, double *a, int *lda, double *b, int *ldb, double *be,
           double *c, int *ldc)
{ scipy_dgemm_(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc); }
void dsytrf(char *u, int *n, double *a, int *lda, int *ipiv, double *w, int *lw, int *info)
{ scipy_dsytrf_(u, n, a, lda, ipiv, w, lw, info); }
void dsytri(char *u, int *n, double *a, int *lda, int *ipiv, double *w, int *info)
{ scipy_dsytri_(u, n, a, lda, ipiv, w, info); }

/* The underscored names, for reference units compiled with LAPACK_UNDERSCORE. */
void dgemm_(char *ta, char *tb, int *m, int *n, int *k, double *al, double *a, int *lda, double *b, int *ldb,
            double *be, double *c, int *ldc)
{ scipy_dgemm_(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc); }
void dsyev_(char *jobz, char *uplo, int *n, double *a, int *lda, double *w, double *work, int *lwork, int *info)
{ scipy_dsyev_(jobz, uplo, n, a, lda, w, work, lwork, info); }
void dgetrf_(int *m, int *n, double *a, int *lda, int *ipiv, int *info) { scipy_dgetrf_(m, n, a, lda, ipiv, info); }
void dgetri_(int *n, double *a, int *lda, int *ipiv, double *work, int *lwork, int *info)
{ scipy_dgetri_(n, a, lda, ipiv, work, lwork, info); }
void dposv_(char *uplo, int *n, int *nrhs, double *a, int *lda, double *b, int *ldb, int *info)
{ scipy_dposv_(uplo, n, nrhs, a, lda, b, ldb, info); }
