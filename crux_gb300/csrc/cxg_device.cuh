// Device functions shared by the kernels of several translation units:
// the P matrix of one (child edge, component) written into its op record,
// and the FP64 eigensystem of a reversible 4-state Q.
#pragma once

#include <math.h>

#include "cxg_internal.h"

namespace cxg {

// P(t) = max(0, sum_k cube[i][j][k] exp(lambda_k t)) for child c and
// component k of idx = c * kact + k (CxLik.c:258-292), FP64, stored into
// the op record as the plan's precision.  A leaf child (tab >= 0) gets its
// message table instead: row mask = sum over the allowed states j of
// P[i][j], in j order (P times the reference's 0/1 row, CxLik.c:357-374
// with Lik.pyx:1466-1475), in the FP64 table for FP64 plans and in the
// record, rounded once to FP32, for FP32 plans.
//
// Four consecutive lanes (q = lane & 3, all four active) share one idx:
// lane q computes exp(lambda_q t) and row i = q, so each lane runs a
// quarter of the serial FP64 work.  Every entry's operations and their
// order are those of one lane doing it all.
__device__ inline void pmat_one(const PmatArgs &a, unsigned idx, unsigned q) {
    const unsigned c = idx / a.kact, k = idx % a.kact;
    const int m = a.model[k];
    // Same association as the reference: ((edgeLen*cmult)*rmult)*wNorm.
    const double wn = a.wnorm_dev ? *a.wnorm_dev : a.wnorm;
    const double t = __dmul_rn(__dmul_rn(__dmul_rn(a.edge_len[c], a.cmult[k]),
                                         a.rmult[k]), wn);
    const double *cube = a.cube + (size_t)m * 64;
    const double *ev = a.eig + (size_t)m * 4;
    const double exq = exp(__dmul_rn(ev[q], t));
    const unsigned gmask = 0xFu << ((threadIdx.x & 31u) & ~3u);
    double ex[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) ex[r] = __shfl_sync(gmask, exq, r, 4);
    const int i = (int)q;
    double P[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        double s = 0.0;
#pragma unroll
        for (int r = 0; r < 4; ++r) s = __dadd_rn(s, __dmul_rn(cube[i * 16 + j * 4 + r], ex[r]));
        P[j] = s < 0.0 ? 0.0 : s;
    }
    const int tb = a.tab[c];
    unsigned char *dst = a.rec + a.dst[c];
    if (tb >= 0) {
        // Message of a leaf with state mask m: the sum over allowed states j
        // of P[i][j], in j order -- exactly P times the reference's 0/1 row.
        // Built incrementally: entry m is entry (m without its highest
        // state h) plus P[i][h], which is the same sum in the same order.
        double T[16];
        T[0] = 0.0;
#pragma unroll
        for (int mk = 1; mk < 16; ++mk) {
            const int h = mk >= 8 ? 3 : mk >= 4 ? 2 : mk >= 2 ? 1 : 0;
            T[mk] = __dadd_rn(T[mk ^ (1 << h)], P[h]);
        }
        if (a.precision == CXG_FP32) {
            float *o = reinterpret_cast<float *>(dst) + (size_t)k * 4 + i;
#pragma unroll
            for (int mk = 0; mk < 16; ++mk) o[(size_t)mk * a.kact * 4] = (float)T[mk];
            return;
        }
        double *tt = a.ltab + ((size_t)tb * 16 * a.kact + k) * 4 + i;
#pragma unroll
        for (int mk = 0; mk < 16; ++mk) tt[(size_t)mk * a.kact * 4] = T[mk];
    }
    if (a.precision == CXG_FP32) {
        float *o = reinterpret_cast<float *>(dst) + (size_t)k * 16 + i * 4;
#pragma unroll
        for (int j = 0; j < 4; ++j) o[j] = (float)P[j];
    } else {
        double *o = reinterpret_cast<double *>(dst) + (size_t)k * 16 + i * 4;
#pragma unroll
        for (int j = 0; j < 4; ++j) o[j] = P[j];
    }
}


// ---------------------------------------------------------------------------
// FP64 eigensystem of Q = R Pi (reversible, 4 states).
// out: [0..3] piNorm, [4] qNorm, [5..68] cube, [69..72] eigenvalues,
// [73] status (0 ok, 1 bad input, 2 no convergence).
// ---------------------------------------------------------------------------
__device__ inline void qdecomp4(const double *rtri, const double *pi, double *out) {
    // Every fixed-size loop is unrolled so that the 4 x 4 matrices live in
    // registers; the arithmetic and its order are those of the loops.
    double pn[4], sq[4], q[16], s[16], u[16];
    double psum = 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) psum += pi[i];
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        pn[i] = pi[i] / psum;
        ok = ok && (pn[i] > 0.0);
    }
    if (!ok) {
        out[73] = 1.0;
        return;
    }
    // Upper-triangle order of rtri: (0,1) (0,2) (0,3) (1,2) (1,3) (2,3).
    const int tri[4][4] = {{-1, 0, 1, 2}, {0, -1, 3, 4}, {1, 3, -1, 5},
                           {2, 4, 5, -1}};
    double rt[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) rt[i] = rtri[i];
    double qscale = 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (i == j) continue;
            q[i * 4 + j] = rt[tri[i][j]] * pn[j];
            if (j < i) qscale += q[i * 4 + j] * pn[i] * 2.0;
        }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        double d = 0.0;
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (j != i) d -= q[i * 4 + j];
        q[i * 4 + i] = d;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) sq[i] = sqrt(pn[i]);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
            s[i * 4 + j] = (i == j) ? q[i * 4 + i] : rt[tri[i][j]] * sq[i] * sq[j];
#pragma unroll
    for (int i = 0; i < 16; ++i) u[i] = (i % 5 == 0) ? 1.0 : 0.0;
    int conv = 0;
    for (int sweep = 0; sweep < 64 && !conv; ++sweep) {
        double off = 0.0, dg = 0.0;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            dg += s[i * 4 + i] * s[i * 4 + i];
#pragma unroll
            for (int j = i + 1; j < 4; ++j) off += s[i * 4 + j] * s[i * 4 + j];
        }
        if (off == 0.0 || off <= 1e-40 * dg) {
            conv = 1;
            break;
        }
#pragma unroll
        for (int pp = 0; pp < 3; ++pp)
#pragma unroll
            for (int qq = pp + 1; qq < 4; ++qq) {
                const double apq = s[pp * 4 + qq];
                if (apq != 0.0) {
                    const double app = s[pp * 4 + pp], aqq = s[qq * 4 + qq];
                    const double th = (aqq - app) / (2.0 * apq);
                    const double t = (th >= 0.0 ? 1.0 : -1.0) /
                                     (fabs(th) + sqrt(th * th + 1.0));
                    const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const double akp = s[k * 4 + pp], akq = s[k * 4 + qq];
                        s[k * 4 + pp] = c * akp - sn * akq;
                        s[k * 4 + qq] = sn * akp + c * akq;
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const double apk = s[pp * 4 + k], aqk = s[qq * 4 + k];
                        s[pp * 4 + k] = c * apk - sn * aqk;
                        s[qq * 4 + k] = sn * apk + c * aqk;
                    }
                    s[pp * 4 + qq] = s[qq * 4 + pp] = 0.0;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const double ukp = u[k * 4 + pp], ukq = u[k * 4 + qq];
                        u[k * 4 + pp] = c * ukp - sn * ukq;
                        u[k * 4 + qq] = sn * ukp + c * ukq;
                    }
                }
            }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) out[i] = pn[i];
    out[4] = 1.0 / qscale;
    // V = Pi^-1/2 U and V^-1 = U^T Pi^1/2: cube[i][j][k] = V[i][k] V^-1[k][j].
    // Four reciprocals instead of 64 divisions (FP64 division is a long
    // instruction sequence on this part); V[i][k] moves by at most an ulp.
    double isq[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) isq[i] = 1.0 / sq[i];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k)
                out[5 + i * 16 + j * 4 + k] =
                    (u[i * 4 + k] * isq[i]) * (u[j * 4 + k] * sq[j]);
#pragma unroll
    for (int k = 0; k < 4; ++k) out[69 + k] = s[k * 4 + k];
    out[73] = conv ? 0.0 : 2.0;
}


}  // namespace cxg
