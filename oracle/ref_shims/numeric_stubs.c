/* Link-only stubs for the LAPACK/BLAS/ARPACK routines the CIFlow reference
 * sources reference. The oracle harness never calls them: eigenpairs come
 * from scipy's ARPACK driving the reference's own SparseMatrix_CRS_Sym::mvprod.
 * Any call reports failure through its info argument (or does nothing). */
#include <stdio.h>

static void cigpu_stub_called(const char *name) {
    fprintf(stderr, "oracle reference build: stub %s called (not available)\n", name);
}

void dsaupd_(int *ido, char *bmat, int *n, char *which, int *nev, double *tol, double *resid,
             int *ncv, double *v, int *ldv, int *iparam, int *ipntr, double *workd, double *workl,
             int *lworkl, int *info) {
    cigpu_stub_called("dsaupd_");
    *ido = 99;
    *info = -9999;
}
void dseupd_(int *rvec, char *all, int *select, double *d, double *z, int *ldz, double *sigma,
             char *bmat, int *n, char *which, int *nev, double *tol, double *resid, int *ncv,
             double *v, int *ldv, int *iparam, int *ipntr, double *workd, double *workl,
             int *lworkl, int *info) {
    cigpu_stub_called("dseupd_");
    *info = -9999;
}
void dsyevd_(char *jobz, char *uplo, int *n, double *a, int *lda, double *w, double *work,
             int *lwork, int *iwork, int *liwork, int *info) { cigpu_stub_called("dsyevd_"); *info = -1; }
void dsyev_(char *jobz, char *uplo, int *n, double *a, int *lda, double *w, double *work,
            int *lwork, int *info) { cigpu_stub_called("dsyev_"); *info = -1; }
void dgesv_(int *n, int *nrhs, double *a, int *lda, int *ipiv, double *b, int *ldb, int *info) {
    cigpu_stub_called("dgesv_"); *info = -1;
}
void dgesvd_(char *ju, char *jvt, int *m, int *n, double *a, int *lda, double *s, double *u,
             int *ldu, double *vt, int *ldvt, double *work, int *lwork, int *info) {
    cigpu_stub_called("dgesvd_"); *info = -1;
}
void dgetrf_(int *m, int *n, double *a, int *lda, int *ipiv, int *info) { cigpu_stub_called("dgetrf_"); *info = -1; }
void dgetri_(int *n, double *a, int *lda, int *ipiv, double *work, int *lwork, int *info) {
    cigpu_stub_called("dgetri_"); *info = -1;
}
/* dgemm_ is not a stub: OrbitalTransform::fillHamCI and rotate_old_to_new
 * (OrbitalTransform.cpp:64-200) rotate the integrals with it, and the rotation
 * fixtures are made by running them. This is the plain triple loop of the BLAS
 * definition, column-major: C := alpha op(A) op(B) + beta C with op(X) = X or X^T
 * ('N' / 'T'); C is not read when beta == 0. */
void dgemm_(char *ta, char *tb, const int *m, const int *n, const int *k, double *alpha, double *a,
            const int *lda, double *b, const int *ldb, double *beta, double *c, const int *ldc) {
    const int M = *m, N = *n, K = *k, LA = *lda, LB = *ldb, LC = *ldc;
    const int tra = (*ta == 'T' || *ta == 't' || *ta == 'C' || *ta == 'c');
    const int trb = (*tb == 'T' || *tb == 't' || *tb == 'C' || *tb == 'c');
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < M; ++i) {
            double acc = 0.0;
            for (int l = 0; l < K; ++l) {
                const double av = tra ? a[l + (long)i * LA] : a[i + (long)l * LA];
                const double bv = trb ? b[j + (long)l * LB] : b[l + (long)j * LB];
                acc += av * bv;
            }
            double *cij = &c[i + (long)j * LC];
            *cij = (*beta == 0.0) ? *alpha * acc : *alpha * acc + *beta * *cij;
        }
}
void dsymv_(char *uplo, int *n, double *alpha, double *a, int *lda, double *x, int *incx,
            double *beta, double *y, int *incy) { cigpu_stub_called("dsymv_"); }
void dcopy_(int *n, double *x, int *incx, double *y, int *incy) { cigpu_stub_called("dcopy_"); }
