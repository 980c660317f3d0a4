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
// with Lik.pyx:1466-1475), in the FP64 table for FP64 plans ([16 masks]
// [kact][4]) and in the record, rounded once to FP32, for FP32 plans
// ([kact][16 masks][4]).
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
            // Component-major, [kact][16 masks][4 states]: the walker's
            // threads read one component's rows at once, so rows of
            // different masks sit in different shared-memory banks.
            float *o = reinterpret_cast<float *>(dst) + (size_t)k * 64 + i;
#pragma unroll
            for (int mk = 0; mk < 16; ++mk) o[(size_t)mk * 4] = (float)T[mk];
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
// FP64 eigensystem of Q = R Pi (reversible, 4 states): Q is similar to the
// symmetric S = Pi^1/2 Q Pi^-1/2, diagonalised by Jacobi rotations
// (Rutishauser's form), then V = Pi^-1/2 U and V^-1 = U^T Pi^1/2.
// out: [0..3] piNorm, [4] qNorm, [5..68] cube, [69..72] eigenvalues,
// [73] status (0 ok, 1 bad input, 2 no convergence).
// ---------------------------------------------------------------------------

// Pick entry r (0..3) without indexing a register array by a run-time value.
__device__ __forceinline__ double sel4(int r, double a, double b, double c, double d) {
    return r == 0 ? a : r == 1 ? b : r == 2 ? c : d;
}

// The eigensystem of qdecomp4 on four lanes of a warp (lanes base .. base+3,
// all four calling; out in memory those lanes can all reach, as for
// qdecomp4).  Lane base+r holds row r of S = Pi^1/2 Q Pi^-1/2 and of the
// rotations U.  Jacobi by rounds: each round applies two disjoint rotations,
// (0,1)(2,3), then (0,2)(1,3), then (0,3)(1,2).  Disjoint rotations commute
// and neither changes the entries the other's angle is computed from, so
// taking both angles from the round's starting matrix is the same as
// applying them one after the other.  Both lanes of a pair use the lower
// lane's off-diagonal entry, so they compute the same rotation.  Each FP64
// instruction of a warp costs the same with one lane active or four, so the
// four lanes do in one instruction stream what qdecomp4 does in four.
__device__ inline void qdecomp4_warp(const double *rtri, const double *pi, double *out,
                                     unsigned base) {
    const unsigned lane = threadIdx.x & 31u;
    const int r = (int)(lane - base);
    const unsigned mask = 0xFu << base;
    double pn[4];
    double psum = 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) psum += pi[i];
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        pn[i] = pi[i] / psum;
        ok = ok && (pn[i] > 0.0);
    }
    if (!ok) {  // the same on the four lanes
        if (r == 0) out[73] = 1.0;
        return;
    }
    double rt[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) rt[i] = rtri[i];
    // Upper-triangle order of rtri: (0,1) (0,2) (0,3) (1,2) (1,3) (2,3).
    const int tri[4][4] = {{-1, 0, 1, 2}, {0, -1, 3, 4}, {1, 3, -1, 5},
                           {2, 4, 5, -1}};
    double q[16];
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
    const double sqr = sqrt(sel4(r, pn[0], pn[1], pn[2], pn[3]));
    double sq[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) sq[j] = __shfl_sync(mask, sqr, base + j);
    // Row r of S and of U.
    double s[4], u[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        double e[4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
            e[i] = (i == j) ? q[i * 4 + i] : rt[tri[i][j]] * sq[i] * sq[j];
        s[j] = sel4(r, e[0], e[1], e[2], e[3]);
        u[j] = (j == r) ? 1.0 : 0.0;
    }
    int conv = 0;
    for (int sweep = 0; sweep < 64 && !conv; ++sweep) {
        double offr = 0.0, dgr = 0.0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (j == r) dgr = s[j] * s[j];
            if (j > r) offr += s[j] * s[j];
        }
        // Butterfly sums: every lane adds the same pairs, so all agree.
        offr += __shfl_xor_sync(mask, offr, 1);
        offr += __shfl_xor_sync(mask, offr, 2);
        dgr += __shfl_xor_sync(mask, dgr, 1);
        dgr += __shfl_xor_sync(mask, dgr, 2);
        if (offr == 0.0 || offr <= 1e-40 * dgr) {
            conv = 1;
            break;
        }
#pragma unroll
        for (int X = 1; X <= 3; ++X) {  // partner of row r: r ^ X
            const int pr = r ^ X;
            const int lo = r < pr ? r : pr;
            // The pair's entries: the diagonals from their own lanes, the
            // off-diagonal from the lower lane.
            const double dr = sel4(r, s[0], s[1], s[2], s[3]);
            const double dp = __shfl_sync(mask, dr, base + pr);
            const double opr = sel4(pr, s[0], s[1], s[2], s[3]);
            const double apq = __shfl_sync(mask, opr, base + lo);
            const double app = r == lo ? dr : dp, aqq = r == lo ? dp : dr;
            double c = 1.0, sn = 0.0;
            if (apq != 0.0) {
                const double th = (aqq - app) / (2.0 * apq);
                const double t = (th >= 0.0 ? 1.0 : -1.0) /
                                 (fabs(th) + sqrt(th * th + 1.0));
                c = 1.0 / sqrt(t * t + 1.0);
                sn = t * c;
            }
            // The other pair's rotation, from one of its lanes.
            const int ol = r ^ (X == 1 ? 2 : 1);
            const double co = __shfl_sync(mask, c, base + ol);
            const double so = __shfl_sync(mask, sn, base + ol);
            // Columns: row r of S J and of U J.  Column j pairs with j ^ X.
            double ns[4], nu[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int jp = j ^ X;
                const bool mine = (j == r) || (j == pr);
                const double cj = mine ? c : co, sj = mine ? sn : so;
                if (j < jp) {
                    ns[j] = cj * s[j] - sj * s[jp];
                    nu[j] = cj * u[j] - sj * u[jp];
                } else {
                    ns[j] = sj * s[jp] + cj * s[j];
                    nu[j] = sj * u[jp] + cj * u[j];
                }
            }
            // Rows: row r of J^T (S J) mixes with the partner's row.
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const double o = __shfl_sync(mask, ns[j], base + pr);
                s[j] = (r == lo) ? c * ns[j] - sn * o : sn * o + c * ns[j];
                u[j] = nu[j];
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (j == pr) s[j] = 0.0;
        }
    }
    out[r] = sel4(r, pn[0], pn[1], pn[2], pn[3]);
    if (r == 0) out[4] = 1.0 / qscale;
    // cube[r][j][k] = V[r][k] V^-1[k][j] with V = Pi^-1/2 U, V^-1 = U^T Pi^1/2.
    const double isq = 1.0 / sel4(r, sq[0], sq[1], sq[2], sq[3]);
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double ujk = __shfl_sync(mask, u[k], base + j);
            out[5 + r * 16 + j * 4 + k] = (u[k] * isq) * (ujk * sq[j]);
        }
    out[69 + r] = sel4(r, s[0], s[1], s[2], s[3]);
    if (r == 0) out[73] = conv ? 0.0 : 2.0;
}

}  // namespace cxg
