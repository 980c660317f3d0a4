/*
 * ORACLE TEST INFRASTRUCTURE -- not part of the product.
 *
 * LAPACK entry points for the reference's CPU core (lib/Crux/CxLapack.h:4-15
 * declares dgeev_, dgetrf_, dgetri_; the reference links its vendored Fortran
 * LAPACK, which cannot be compiled here for lack of a Fortran compiler).
 * Each symbol forwards to a function pointer installed at load time by
 * oracle/oracle.py from scipy.linalg.cython_lapack (scipy-openblas LAPACK,
 * same Fortran calling convention).
 */
#include <stddef.h>

typedef void (*geev_fn)(char *, char *, int *, double *, int *, double *,
                        double *, double *, int *, double *, int *, double *,
                        int *, int *);
typedef void (*getrf_fn)(int *, int *, double *, int *, int *, int *);
typedef void (*getri_fn)(int *, double *, int *, int *, double *, int *,
                         int *);

static geev_fn fwd_geev;
static getrf_fn fwd_getrf;
static getri_fn fwd_getri;

void oracle_set_lapack(void *geev, void *getrf, void *getri) {
    fwd_geev = (geev_fn)geev;
    fwd_getrf = (getrf_fn)getrf;
    fwd_getri = (getri_fn)getri;
}

void dgeev_(char *jobvl, char *jobvr, int *n, double *a, int *lda, double *wr,
            double *wi, double *vl, int *ldvl, double *vr, int *ldvr,
            double *work, int *lwork, int *info) {
    if (fwd_geev == NULL) { *info = -1000; return; }
    fwd_geev(jobvl, jobvr, n, a, lda, wr, wi, vl, ldvl, vr, ldvr, work, lwork,
             info);
}

void dgetrf_(int *m, int *n, double *a, int *lda, int *ipiv, int *info) {
    if (fwd_getrf == NULL) { *info = -1000; return; }
    fwd_getrf(m, n, a, lda, ipiv, info);
}

void dgetri_(int *n, double *a, int *lda, int *ipiv, double *work, int *lwork,
             int *info) {
    if (fwd_getri == NULL) { *info = -1000; return; }
    fwd_getri(n, a, lda, ipiv, work, lwork, info);
}
