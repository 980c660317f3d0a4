// Device kernels of the pruning likelihood on sm_103a.
//
// Layout in HBM: a CL buffer of K active components over ppad patterns is
// state-planar, [K][4][ppad], so that the threads of a warp, one pattern
// each, read and write 32 consecutive elements of a plane per instruction.
// Leaves are one uint8 state mask per pattern.  Scalers are one FP64 log
// scale (plain form) or one int32 power-of-two exponent (FP32 form) per
// pattern.
//
// Kernels:
//   pmat_kernel     P(t) = V diag(exp(lambda r t)) V^-1 per (child edge,
//                   component), FP64, clipped at 0 (CxLik.c:258-292), plus
//                   the 16-entry message table of every leaf child.
//   plan_kernel<T>  walks the whole node-update list for one pattern per
//                   thread (patterns are independent through the entire
//                   post-order, CxLik.c:314-596, so no grid-wide sync is
//                   needed), then aggregates the root (CxLik.c:598-632) and
//                   reduces the weighted site lnLs with a compensated sum.
//   qdecomp_kernel  FP64 eigensystem of a reversible 4x4 Q by Jacobi
//                   rotations of the symmetrised matrix (CxLik.c:59-250).
#include <math.h>

#include "cxg_internal.h"

namespace cxg {

// ---------------------------------------------------------------------------
// P matrices and leaf message tables.
// ---------------------------------------------------------------------------
__global__ void pmat_kernel(PmatArgs a) {
    const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= a.nchild * a.kact) return;
    const unsigned c = idx / a.kact, k = idx % a.kact;
    const int m = a.model[k];
    // Same association as the reference: ((edgeLen*cmult)*rmult)*wNorm.
    const double t = __dmul_rn(__dmul_rn(__dmul_rn(a.edge_len[c], a.cmult[k]),
                                         a.rmult[k]), a.wnorm);
    const double *cube = a.cube + (size_t)m * 64;
    const double *ev = a.eig + (size_t)m * 4;
    double ex[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) ex[q] = exp(__dmul_rn(ev[q], t));
    double P[16];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            double s = 0.0;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                s = __dadd_rn(s, __dmul_rn(cube[i * 16 + j * 4 + q], ex[q]));
            P[i * 4 + j] = s < 0.0 ? 0.0 : s;
        }
    }
    double *o64 = a.pm64 + ((size_t)c * a.kact + k) * 16;
    float *o32 = a.pm32 + ((size_t)c * a.kact + k) * 16;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        o64[q] = P[q];
        o32[q] = (float)P[q];
    }
    if (a.leafflag[c]) {
        // Message of a leaf with state mask m: sum over allowed states j of
        // P[i][j], in j order -- exactly the reference's P * (0/1 vector).
        for (int mask = 0; mask < 16; ++mask) {
            double *t64 = a.ltab64 + (((size_t)c * 16 + mask) * a.kact + k) * 4;
            float *t32 = a.ltab32 + (((size_t)c * 16 + mask) * a.kact + k) * 4;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                double s = 0.0;
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (mask & (1 << j)) s = __dadd_rn(s, P[i * 4 + j]);
                t64[i] = s;
                t32[i] = (float)s;
            }
        }
    }
}

cudaError_t launch_pmat(const PmatArgs &a, cudaStream_t s) {
    const unsigned n = a.nchild * a.kact;
    if (n == 0) return cudaSuccess;
    pmat_kernel<<<(n + 127) / 128, 128, 0, s>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Compensated (Neumaier two-sum) reduction helpers.
// ---------------------------------------------------------------------------
struct Comp {
    double s, c;
};

__device__ __forceinline__ Comp comp_add(Comp a, Comp b) {
    const double s = a.s + b.s;
    const double bb = s - a.s;
    const double err = (a.s - (s - bb)) + (b.s - bb);
    return Comp{s, a.c + b.c + err};
}

__device__ __forceinline__ Comp warp_comp(Comp v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        Comp o;
        o.s = __shfl_down_sync(0xffffffffu, v.s, off);
        o.c = __shfl_down_sync(0xffffffffu, v.c, off);
        v = comp_add(v, o);
    }
    return v;
}

// Block sum of `v` (finite values; -inf sites are counted separately), then
// the last block to finish folds all block partials into a.total.
__device__ void reduce_sites(const PlanArgs &a, double v, bool neg_inf) {
    __shared__ Comp warp_part[kBlock / 32];
    __shared__ unsigned ninf_block;
    __shared__ bool last;
    if (threadIdx.x == 0) ninf_block = 0;
    __syncthreads();
    if (neg_inf) atomicAdd(&ninf_block, 1u);
    Comp c = warp_comp(Comp{v, 0.0});
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_part[warp] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        Comp b = warp_part[0];
        for (unsigned w = 1; w < kBlock / 32; ++w) b = comp_add(b, warp_part[w]);
        a.partial[2 * blockIdx.x] = b.s;
        a.partial[2 * blockIdx.x + 1] = b.c;
        if (ninf_block) atomicAdd(a.ninf, ninf_block);
        __threadfence();
        const unsigned t = atomicAdd(a.ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    Comp acc{0.0, 0.0};
    for (unsigned b = threadIdx.x; b < gridDim.x; b += kBlock) {
        const volatile double *pp = a.partial;
        acc = comp_add(acc, Comp{pp[2 * b], pp[2 * b + 1]});
    }
    acc = warp_comp(acc);
    if (lane == 0) warp_part[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        Comp b = warp_part[0];
        for (unsigned w = 1; w < kBlock / 32; ++w) b = comp_add(b, warp_part[w]);
        a.total[0] = b.s;
        a.total[1] = b.c;
        *a.ticket = 0;  // ready for the next launch
    }
}

// ---------------------------------------------------------------------------
// Plan walkers.  T = double: plain form, the reference's scaler (max over
// child messages, CxLik.c:390-403 and 577-588).  T = float: FP32 form, scale
// by the power of two that puts the largest parent entry in [0.5, 1); the
// exponent is an exact integer.
// ---------------------------------------------------------------------------
template <typename T>
struct Prec;

template <>
struct Prec<double> {
    typedef double S;  // scaler type
};

template <>
struct Prec<float> {
    typedef int S;
};

__device__ __forceinline__ float pow2f(int n) {  // n in [-126, 127]
    return __int_as_float((n + 127) << 23);
}

template <typename T, int KT>
__global__ void __launch_bounds__(kBlock) plan_kernel(PlanArgs a) {
    typedef typename Prec<T>::S S;
    const unsigned p = blockIdx.x * kBlock + threadIdx.x;
    const size_t ppad = a.ppad;
    const T *pm = static_cast<const T *>(a.pm);
    const T *lt = static_cast<const T *>(a.ltab);

    for (unsigned o = 0; o < a.nops; ++o) {
        const DevOp op = a.ops[o];
        T acc[KT * 4];
        T sc = T(0);       // plain form: max over child messages
        S lns = S(0);      // log scale (double) or exponent (int)
        for (unsigned ci = 0; ci < op.nchild; ++ci) {
            const DevChild ch = a.children[op.child0 + ci];
            T msg[KT * 4];
            if (ch.leaf) {
                const unsigned m = static_cast<const uint8_t *>(ch.data)[p];
                const T *t = lt + ((size_t)ch.pm * 16 + m) * (KT * 4);
#pragma unroll
                for (int q = 0; q < KT * 4; ++q) msg[q] = t[q];
            } else {
                const T *x = static_cast<const T *>(ch.data);
                const T *P = pm + (size_t)ch.pm * (KT * 16);
#pragma unroll
                for (int k = 0; k < KT; ++k) {
                    const T x0 = x[(k * 4 + 0) * ppad + p];
                    const T x1 = x[(k * 4 + 1) * ppad + p];
                    const T x2 = x[(k * 4 + 2) * ppad + p];
                    const T x3 = x[(k * 4 + 3) * ppad + p];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const T *r = P + k * 16 + i * 4;
                        T v = r[0] * x0;
                        v = fma(r[1], x1, v);
                        v = fma(r[2], x2, v);
                        v = fma(r[3], x3, v);
                        msg[k * 4 + i] = v;
                    }
                }
                const S l = static_cast<const S *>(ch.scaler)[p];
                lns = (ci == 0) ? l : lns + l;
            }
            if (ci == 0) {
#pragma unroll
                for (int q = 0; q < KT * 4; ++q) acc[q] = msg[q];
            } else {
#pragma unroll
                for (int q = 0; q < KT * 4; ++q) acc[q] *= msg[q];
            }
            if (sizeof(T) == 8) {
#pragma unroll
                for (int q = 0; q < KT * 4; ++q) sc = fmax(sc, msg[q]);
            }
        }
        if (sizeof(T) == 8) {
            // Reference rescale: divide by the scaler unless it is 1, add
            // its log (a zero scaler gives NaN rows and a -inf site, as in
            // the reference).
            if (sc != T(1)) {
                const T r = T(1) / sc;
#pragma unroll
                for (int q = 0; q < KT * 4; ++q) acc[q] *= r;
            }
            lns = lns + (S)log((double)sc);
        } else {
            T mx = T(0);
#pragma unroll
            for (int q = 0; q < KT * 4; ++q) mx = fmax(mx, acc[q]);
            if (mx > T(0) && mx <= (T)3.0e38) {
                int e;
                frexpf((float)mx, &e);
                const int n = -e;
                if (n >= -126 && n <= 127) {
                    const float s = pow2f(n);
#pragma unroll
                    for (int q = 0; q < KT * 4; ++q) acc[q] *= (T)s;
                } else {
                    const int n1 = n / 2, n2 = n - n1;
                    const float s1 = pow2f(n1), s2 = pow2f(n2);
#pragma unroll
                    for (int q = 0; q < KT * 4; ++q) acc[q] = (acc[q] * (T)s1) * (T)s2;
                }
                lns = lns + (S)e;
            }
        }
        T *y = static_cast<T *>(op.data);
#pragma unroll
        for (int q = 0; q < KT * 4; ++q) y[q * ppad + p] = acc[q];
        static_cast<S *>(op.scaler)[p] = lns;
    }

    // Root aggregation (CxLik.c:598-632): L = sum_k sum_i pn[k][i] root.
    const T *root = static_cast<const T *>(a.root);
    double L = 0.0;
#pragma unroll
    for (int k = 0; k < KT; ++k)
#pragma unroll
        for (int i = 0; i < 4; ++i)
            L = fma(a.pn[k * 4 + i], (double)root[(k * 4 + i) * ppad + p], L);
    const S rs = static_cast<const S *>(a.rootsc)[p];
    double v = 0.0;
    bool ninf = false;
    if (p < a.npat) {
        const double lsc = (sizeof(T) == 8) ? (double)rs
                                           : (double)rs * 0.69314718055994530942;
        v = (log(L) + lsc) * (double)a.freqs[p];
        if (isnan(v)) v = -INFINITY;
        if (a.site) a.site[p] = v;
        if (isinf(v)) {
            ninf = (v < 0.0);
            v = 0.0;
        }
    }
    reduce_sites(a, v, ninf);
}

unsigned plan_blocks(unsigned ppad) { return ppad / kBlock; }

template <typename T>
static cudaError_t launch_plan_t(const PlanArgs &a, cudaStream_t s) {
    const unsigned nb = plan_blocks(a.ppad);
    switch (a.kact) {
#define CXG_K(K) \
    case K: plan_kernel<T, K><<<nb, kBlock, 0, s>>>(a); break;
        CXG_K(1) CXG_K(2) CXG_K(3) CXG_K(4) CXG_K(5) CXG_K(6) CXG_K(7) CXG_K(8)
#undef CXG_K
        default:
            return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_plan(int precision, const PlanArgs &a, cudaStream_t s) {
    return precision == CXG_FP32 ? launch_plan_t<float>(a, s)
                                 : launch_plan_t<double>(a, s);
}

// ---------------------------------------------------------------------------
// FP64 eigensystem of Q = R Pi (reversible, 4 states).
// out: [0..3] piNorm, [4] qNorm, [5..68] cube, [69..72] eigenvalues,
// [73] status (0 ok, 1 bad input, 2 no convergence).
// ---------------------------------------------------------------------------
__device__ void qdecomp4(const double *rtri, const double *pi, double *out) {
    double pn[4], sq[4], q[16], s[16], u[16];
    double psum = 0.0;
    for (int i = 0; i < 4; ++i) psum += pi[i];
    bool ok = true;
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
    double qscale = 0.0;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            if (i == j) continue;
            q[i * 4 + j] = rtri[tri[i][j]] * pn[j];
            if (j < i) qscale += q[i * 4 + j] * pn[i] * 2.0;
        }
    for (int i = 0; i < 4; ++i) {
        double d = 0.0;
        for (int j = 0; j < 4; ++j)
            if (j != i) d -= q[i * 4 + j];
        q[i * 4 + i] = d;
    }
    for (int i = 0; i < 4; ++i) sq[i] = sqrt(pn[i]);
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            s[i * 4 + j] = (i == j) ? q[i * 4 + i] : rtri[tri[i][j]] * sq[i] * sq[j];
    for (int i = 0; i < 16; ++i) u[i] = (i % 5 == 0) ? 1.0 : 0.0;
    int conv = 0;
    for (int sweep = 0; sweep < 64 && !conv; ++sweep) {
        double off = 0.0, dg = 0.0;
        for (int i = 0; i < 4; ++i) {
            dg += s[i * 4 + i] * s[i * 4 + i];
            for (int j = i + 1; j < 4; ++j) off += s[i * 4 + j] * s[i * 4 + j];
        }
        if (off == 0.0 || off <= 1e-40 * dg) {
            conv = 1;
            break;
        }
        for (int pp = 0; pp < 3; ++pp)
            for (int qq = pp + 1; qq < 4; ++qq) {
                const double apq = s[pp * 4 + qq];
                if (apq == 0.0) continue;
                const double app = s[pp * 4 + pp], aqq = s[qq * 4 + qq];
                const double th = (aqq - app) / (2.0 * apq);
                const double t = (th >= 0.0 ? 1.0 : -1.0) /
                                 (fabs(th) + sqrt(th * th + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < 4; ++k) {
                    const double akp = s[k * 4 + pp], akq = s[k * 4 + qq];
                    s[k * 4 + pp] = c * akp - sn * akq;
                    s[k * 4 + qq] = sn * akp + c * akq;
                }
                for (int k = 0; k < 4; ++k) {
                    const double apk = s[pp * 4 + k], aqk = s[qq * 4 + k];
                    s[pp * 4 + k] = c * apk - sn * aqk;
                    s[qq * 4 + k] = sn * apk + c * aqk;
                }
                s[pp * 4 + qq] = s[qq * 4 + pp] = 0.0;
                for (int k = 0; k < 4; ++k) {
                    const double ukp = u[k * 4 + pp], ukq = u[k * 4 + qq];
                    u[k * 4 + pp] = c * ukp - sn * ukq;
                    u[k * 4 + qq] = sn * ukp + c * ukq;
                }
            }
    }
    for (int i = 0; i < 4; ++i) out[i] = pn[i];
    out[4] = 1.0 / qscale;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            for (int k = 0; k < 4; ++k)
                out[5 + i * 16 + j * 4 + k] =
                    (u[i * 4 + k] / sq[i]) * (u[j * 4 + k] * sq[j]);
    for (int k = 0; k < 4; ++k) out[69 + k] = s[k * 4 + k];
    out[73] = conv ? 0.0 : 2.0;
}

__global__ void qdecomp_kernel(const double *rtri, const double *pi,
                               double *out) {
    if (blockIdx.x == 0 && threadIdx.x == 0) qdecomp4(rtri, pi, out);
}

cudaError_t launch_qdecomp(const double *rtri, const double *pi, double *out,
                           cudaStream_t s) {
    qdecomp_kernel<<<1, 32, 0, s>>>(rtri, pi, out);
    return cudaGetLastError();
}

}  // namespace cxg
