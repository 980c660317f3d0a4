/*
 * ORACLE TEST INFRASTRUCTURE -- not part of the product.
 *
 * cxlik_port.c: a CPU restatement, in this repository's own code, of the
 * reference's pruning-likelihood core (canonware/crux lib/Crux/Tree/CxLik.c).
 * It is the FP64 checker for the GPU library wherever the reference's own
 * build (oracle/_ref) is unavailable, and the timed CPU baseline ("port") on
 * hosts without the reference tree.  It is pinned against the reference's
 * build by tests/test_oracle_pin.py and the fixtures in tests/golden/.
 *
 * Exported with the reference's names and struct ABI (include/cxlik_gpu.h):
 *   CxLikQDecomp  follows CxLik.c:59-141 (Q, qNorm) and CxLik.c:177-250
 *                 (eigen cube), but decomposes the symmetrised matrix
 *                 S = Pi^1/2 Q Pi^-1/2 with cyclic Jacobi rotations instead of
 *                 LAPACK dgeev/dgetrf/dgetri.  For a reversible Q the cube
 *                 V[i][k] Vinv[k][j] is the same matrix up to rounding.
 *   CxLikPt       follows CxLik.c:258-292.
 *   CxLikExecute  follows CxLik.c:294-633 (per-stripe step loop, scaler =
 *                 max over child messages, root aggregation) and
 *                 CxLik.c:914-968 (stripes fanned out to threads).
 *   port_set_threads(t)  number of worker threads (default 1).
 */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

#include "cxlik_gpu.h"

#define MAXDIM 32

static int port_threads = 1;

void port_set_threads(int t) { port_threads = t < 1 ? 1 : t; }
int port_get_threads(void) { return port_threads; }

/* Upper-triangle index of (x, y), x < y, in row order (CxLik.c:36-53). */
static unsigned tri_index(unsigned n, unsigned x, unsigned y) {
    return n * x + y - (((x + 3) * x) >> 1) - 1;
}

/* Eigen-decompose symmetric a (n x n, row-major) by cyclic Jacobi sweeps.
 * On return the diagonal of a holds the eigenvalues and u the eigenvectors
 * (columns).  Returns 0 on convergence. */
static int jacobi_eigen(int n, double *a, double *u) {
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) u[i * n + j] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; i++) {
            diag += a[i * n + i] * a[i * n + i];
            for (int j = i + 1; j < n; j++) off += a[i * n + j] * a[i * n + j];
        }
        if (off == 0.0 || off <= 1e-40 * diag) return 0;
        for (int p = 0; p < n - 1; p++) {
            for (int q = p + 1; q < n; q++) {
                double apq = a[p * n + q];
                if (apq == 0.0) continue;
                double app = a[p * n + p], aqq = a[q * n + q];
                /* Rotation angle that zeroes a[p][q] (Rutishauser form). */
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0.0 ? 1.0 : -1.0) /
                           (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = c * akp - s * akq;
                    a[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = c * apk - s * aqk;
                    a[q * n + k] = s * apk + c * aqk;
                }
                a[p * n + q] = a[q * n + p] = 0.0;
                for (int k = 0; k < n; k++) {
                    double ukp = u[k * n + p], ukq = u[k * n + q];
                    u[k * n + p] = c * ukp - s * ukq;
                    u[k * n + q] = s * ukp + c * ukq;
                }
            }
        }
    }
    return 1;
}

bool CxLikQDecomp(int n, double *RTri, double *PiDiag, double *PiDiagNorm,
                  double *qNorm, double *qEigVecCube, double *qEigVals) {
    if (n < 2 || n > MAXDIM) return true;
    double piSum = 0.0;
    for (int i = 0; i < n; i++) piSum += PiDiag[i];
    for (int i = 0; i < n; i++) {
        PiDiagNorm[i] = PiDiag[i] / piSum;
        if (!(PiDiagNorm[i] > 0.0)) return true;
    }
    /* Q_ij = R_ij pi_j off the diagonal; rows sum to zero. */
    double q[MAXDIM * MAXDIM], s[MAXDIM * MAXDIM], u[MAXDIM * MAXDIM];
    double sq[MAXDIM];
    double qScale = 0.0;
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < n; j++) {
            if (i == j) continue;
            double r = (i < j) ? RTri[tri_index(n, i, j)]
                               : RTri[tri_index(n, j, i)];
            q[i * n + j] = r * PiDiagNorm[j];
            if (j < i) qScale += q[i * n + j] * PiDiagNorm[i] * 2.0;
        }
    }
    for (int i = 0; i < n; i++) {
        double d = 0.0;
        for (int j = 0; j < n; j++)
            if (j != i) d -= q[i * n + j];
        q[i * n + i] = d;
    }
    *qNorm = 1.0 / qScale;
    for (int i = 0; i < n; i++) sq[i] = sqrt(PiDiagNorm[i]);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
            s[i * n + j] = (i == j) ? q[i * n + i]
                                    : q[i * n + j] * sq[i] / sq[j];
    /* Exact symmetry before rotating. */
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++) {
            double m = 0.5 * (s[i * n + j] + s[j * n + i]);
            s[i * n + j] = s[j * n + i] = m;
        }
    if (jacobi_eigen(n, s, u)) return true;
    for (int k = 0; k < n; k++) qEigVals[k] = s[k * n + k];
    /* V = Pi^-1/2 U, Vinv = U^T Pi^1/2; cube[i][j][k] = V[i][k] Vinv[k][j]. */
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
            for (int k = 0; k < n; k++)
                qEigVecCube[i * n * n + j * n + k] =
                    (u[i * n + k] / sq[i]) * (u[j * n + k] * sq[j]);
    return false;
}

void CxLikPt(int n, double *P, double *qEigVecCube, double *qEigVals,
             double v) {
    double ex[MAXDIM];
    for (int k = 0; k < n; k++) ex[k] = exp(qEigVals[k] * v);
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < n; j++) {
            double p = 0.0;
            for (int k = 0; k < n; k++)
                p += qEigVecCube[i * n * n + j * n + k] * ex[k];
            P[i * n + j] = p < 0.0 ? 0.0 : p;
        }
    }
}

/* 4-state messages of one component: m = P x, P row-major 4x4. */
static inline void msg4(const double *restrict pm, const double *restrict x,
                        double *restrict m) {
    const double x0 = x[0], x1 = x[1], x2 = x[2], x3 = x[3];
    m[0] = pm[0] * x0 + pm[1] * x1 + pm[2] * x2 + pm[3] * x3;
    m[1] = pm[4] * x0 + pm[5] * x1 + pm[6] * x2 + pm[7] * x3;
    m[2] = pm[8] * x0 + pm[9] * x1 + pm[10] * x2 + pm[11] * x3;
    m[3] = pm[12] * x0 + pm[13] * x1 + pm[14] * x2 + pm[15] * x3;
}

/* DNA stripe (CxLik.c:294-633): same arithmetic as run_stripe with the
 * 4x4 products unrolled and the active components listed once. */
static void run_stripe_dna(CxtLik *lik, unsigned stripe) {
    const unsigned ncomp = lik->compsLen, dn = 4 * ncomp;
    const unsigned c0 = lik->stripeWidth * stripe;
    const unsigned c1 = c0 + lik->stripeWidth;
    double *P = malloc(sizeof(double) * ncomp * 16);
    double *scale = calloc(lik->stripeWidth, sizeof(double));
    unsigned *act = malloc(sizeof(unsigned) * (ncomp ? ncomp : 1));
    unsigned nact = 0;
    for (unsigned mc = 0; mc < ncomp; mc++)
        if (lik->comps[mc].weightScaled != 0.0) act[nact++] = mc;

    for (unsigned s = 0; s < lik->stepsLen; s++) {
        const CxtLikStep *st = &lik->steps[s];
        double *restrict par = st->parentCL->cLMat;
        double *restrict parLn = st->parentCL->lnScale;
        const double *restrict ch = st->childCL->cLMat;
        const double *restrict chLn = st->childCL->lnScale;
        const int leaf = (st->variant == CxeLikStepComputeL ||
                          st->variant == CxeLikStepMergeL);
        const int merge = (st->variant == CxeLikStepMergeL ||
                           st->variant == CxeLikStepMergeI);
        for (unsigned a = 0; a < nact; a++) {
            const CxtLikComp *cp = &lik->comps[act[a]];
            CxLikPt(4, &P[act[a] * 16], cp->model->qEigVecCube,
                    cp->model->qEigVals,
                    st->edgeLen * cp->cmult * cp->model->rmult * lik->wNorm);
        }
        for (unsigned c = c0; c < c1; c++) {
            double sc = scale[c - c0];
            double m[4];
            for (unsigned a = 0; a < nact; a++) {
                const unsigned mc = act[a];
                msg4(&P[mc * 16], leaf ? &ch[c * 4] : &ch[c * dn + mc * 4], m);
                double *y = &par[c * dn + mc * 4];
                if (merge) {
                    y[0] *= m[0]; y[1] *= m[1]; y[2] *= m[2]; y[3] *= m[3];
                } else {
                    y[0] = m[0]; y[1] = m[1]; y[2] = m[2]; y[3] = m[3];
                }
                if (m[0] > sc) sc = m[0];
                if (m[1] > sc) sc = m[1];
                if (m[2] > sc) sc = m[2];
                if (m[3] > sc) sc = m[3];
            }
            scale[c - c0] = sc;
            parLn[c] = merge ? parLn[c] + chLn[c] : chLn[c];
        }
        if (st->ntrail == 0) {
            for (unsigned c = c0; c < c1; c++) {
                const double sc = scale[c - c0];
                if (sc != 1.0)
                    for (unsigned i = 0; i < dn; i++) par[c * dn + i] /= sc;
                parLn[c] += log(sc);
                scale[c - c0] = 0.0;
            }
        }
    }

    double sum = 0.0;
    const double *root = lik->rootCLC->cLMat;
    const double *rootLn = lik->rootCLC->lnScale;
    for (unsigned c = c0; c < c1; c++) {
        double L = 0.0;
        for (unsigned a = 0; a < nact; a++) {
            const CxtLikComp *cp = &lik->comps[act[a]];
            for (unsigned i = 0; i < 4; i++)
                L += (cp->model->piDiagNorm[i] * cp->weightScaled) *
                     root[c * dn + act[a] * 4 + i];
        }
        double v = (log(L) + rootLn[c]) *
                   (double)lik->charFreqs[lik->cbase + c];
        if (isnan(v)) v = -INFINITY;
        lik->siteLnL[lik->cbase + c] = v;
        sum += v;
    }
    lik->stripeLnL[stripe] = sum;
    free(P);
    free(scale);
    free(act);
}

/* One stripe of the plan (CxLik.c:294-633 restated for any dim). */
static void run_stripe(CxtLik *lik, unsigned stripe) {
    if (lik->dim == 4) {
        run_stripe_dna(lik, stripe);
        return;
    }
    const unsigned dim = lik->dim, ncomp = lik->compsLen;
    const unsigned dn = dim * ncomp;
    const unsigned c0 = lik->stripeWidth * stripe;
    const unsigned c1 = c0 + lik->stripeWidth;
    const unsigned w = lik->stripeWidth;
    double *P = malloc(sizeof(double) * ncomp * dim * dim);
    double *scale = calloc(w, sizeof(double));
    double msg[MAXDIM];

    for (unsigned s = 0; s < lik->stepsLen; s++) {
        const CxtLikStep *st = &lik->steps[s];
        double *par = st->parentCL->cLMat, *parLn = st->parentCL->lnScale;
        const double *ch = st->childCL->cLMat;
        const double *chLn = st->childCL->lnScale;
        const int leaf = (st->variant == CxeLikStepComputeL ||
                          st->variant == CxeLikStepMergeL);
        const int merge = (st->variant == CxeLikStepMergeL ||
                           st->variant == CxeLikStepMergeI);
        for (unsigned mc = 0; mc < ncomp; mc++) {
            const CxtLikComp *cp = &lik->comps[mc];
            if (cp->weightScaled != 0.0)
                CxLikPt(dim, &P[mc * dim * dim], cp->model->qEigVecCube,
                        cp->model->qEigVals,
                        st->edgeLen * cp->cmult * cp->model->rmult *
                            lik->wNorm);
        }
        for (unsigned c = c0; c < c1; c++) {
            double sc = scale[c - c0];
            for (unsigned mc = 0; mc < ncomp; mc++) {
                if (lik->comps[mc].weightScaled == 0.0) continue;
                const double *x = leaf ? &ch[c * dim] : &ch[c * dn + mc * dim];
                const double *pm = &P[mc * dim * dim];
                for (unsigned i = 0; i < dim; i++) {
                    double a = pm[i * dim] * x[0];
                    for (unsigned j = 1; j < dim; j++) a += pm[i * dim + j] * x[j];
                    msg[i] = a;
                    if (a > sc) sc = a;
                }
                double *y = &par[c * dn + mc * dim];
                if (merge)
                    for (unsigned i = 0; i < dim; i++) y[i] *= msg[i];
                else
                    for (unsigned i = 0; i < dim; i++) y[i] = msg[i];
            }
            scale[c - c0] = sc;
            parLn[c] = merge ? parLn[c] + chLn[c] : chLn[c];
        }
        if (st->ntrail == 0) {
            for (unsigned c = c0; c < c1; c++) {
                double sc = scale[c - c0];
                if (sc != 1.0)
                    for (unsigned i = 0; i < dn; i++) par[c * dn + i] /= sc;
                parLn[c] += log(sc);
                scale[c - c0] = 0.0;
            }
        }
    }

    /* Root aggregation (CxLik.c:598-632). */
    double sum = 0.0;
    const double *root = lik->rootCLC->cLMat;
    const double *rootLn = lik->rootCLC->lnScale;
    for (unsigned c = c0; c < c1; c++) {
        double L = 0.0;
        for (unsigned mc = 0; mc < ncomp; mc++) {
            const CxtLikComp *cp = &lik->comps[mc];
            if (cp->weightScaled == 0.0) continue;
            for (unsigned i = 0; i < dim; i++)
                L += (cp->model->piDiagNorm[i] * cp->weightScaled) *
                     root[c * dn + mc * dim + i];
        }
        double v = (log(L) + rootLn[c]) *
                   (double)lik->charFreqs[lik->cbase + c];
        if (isnan(v)) v = -INFINITY;
        lik->siteLnL[lik->cbase + c] = v;
        sum += v;
    }
    lik->stripeLnL[stripe] = sum;
    free(P);
    free(scale);
}

typedef struct {
    CxtLik *lik;
    atomic_uint next;
} pool_job;

static void *pool_worker(void *arg) {
    pool_job *job = arg;
    for (;;) {
        unsigned s = atomic_fetch_add(&job->next, 1u);
        if (s >= job->lik->nstripes) break;
        run_stripe(job->lik, s);
    }
    return NULL;
}

void CxLikExecute(CxtLik *lik) {
    if (lik->stepsLen == 0) return;
    int t = port_threads;
    if (t > (int)lik->nstripes) t = (int)lik->nstripes;
    if (t <= 1) {
        for (unsigned s = 0; s < lik->nstripes; s++) run_stripe(lik, s);
        return;
    }
    pool_job job;
    job.lik = lik;
    atomic_init(&job.next, 0u);
    pthread_t th[256];
    if (t > 256) t = 256;
    int started = 0;
    for (int i = 0; i < t; i++)
        if (pthread_create(&th[i], NULL, pool_worker, &job) == 0) started++;
    if (started == 0) pool_worker(&job);
    for (int i = 0; i < started; i++) pthread_join(th[i], NULL);
}
