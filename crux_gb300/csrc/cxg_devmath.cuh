// Device FP64 helpers for on-device MC3: a counter-based RNG, the discrete
// Gamma rate categories and Gamma/Dirichlet variates.
#pragma once

#include <math.h>
#include <stdint.h>

namespace cxg {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw 2011, "Parallel random numbers:
// as easy as 1, 2, 3"): ten rounds of two 32x32->64 multiplies with the
// published multipliers and Weyl key increments.
// ---------------------------------------------------------------------------
struct Philox {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t out[4];
    int used;
};

__device__ __forceinline__ void philox_round(uint32_t c[4], const uint32_t k[2]) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t hi0 = __umulhi(M0, c[0]), lo0 = M0 * c[0];
    const uint32_t hi1 = __umulhi(M1, c[2]), lo1 = M1 * c[2];
    const uint32_t n0 = hi1 ^ c[1] ^ k[0];
    const uint32_t n1 = lo1;
    const uint32_t n2 = hi0 ^ c[3] ^ k[1];
    const uint32_t n3 = lo0;
    c[0] = n0;
    c[1] = n1;
    c[2] = n2;
    c[3] = n3;
}

__device__ __forceinline__ void philox_block(const uint32_t ctr[4],
                                             const uint32_t key[2],
                                             uint32_t out[4]) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    uint32_t k[2] = {key[0], key[1]};
    for (int r = 0; r < 10; ++r) {
        philox_round(c, k);
        k[0] += 0x9E3779B9u;
        k[1] += 0xBB67AE85u;
    }
    out[0] = c[0];
    out[1] = c[1];
    out[2] = c[2];
    out[3] = c[3];
}

// Stream for (seed, stream id, generation): counter = (gen lo, gen hi,
// stream, draw block).
__device__ __forceinline__ void philox_init(Philox &r, uint64_t seed,
                                            uint32_t stream, uint64_t gen) {
    r.key[0] = (uint32_t)seed;
    r.key[1] = (uint32_t)(seed >> 32);
    r.ctr[0] = (uint32_t)gen;
    r.ctr[1] = (uint32_t)(gen >> 32);
    r.ctr[2] = stream;
    r.ctr[3] = 0;
    r.used = 4;
}

__device__ __forceinline__ uint32_t philox_u32(Philox &r) {
    if (r.used == 4) {
        philox_block(r.ctr, r.key, r.out);
        r.ctr[3]++;
        r.used = 0;
    }
    return r.out[r.used++];
}

// Uniform in [0, 1) with 53 random bits.
__device__ __forceinline__ double philox_u01(Philox &r) {
    const uint32_t a = philox_u32(r) >> 5, b = philox_u32(r) >> 6;
    return (a * 67108864.0 + b) * (1.0 / 9007199254740992.0);
}

// Uniform integer in [0, n).
__device__ __forceinline__ uint32_t philox_below(Philox &r, uint32_t n) {
    return (uint32_t)(philox_u01(r) * n) % n;
}

// Standard normal by Box-Muller.
__device__ __forceinline__ double philox_normal(Philox &r) {
    double u1 = philox_u01(r);
    if (u1 < 1e-300) u1 = 1e-300;
    const double u2 = philox_u01(r);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586476925 * u2);
}

// Gamma(shape, 1) by Marsaglia and Tsang (2000); shape < 1 via the
// u^(1/shape) boost.
__device__ inline double philox_gamma(Philox &r, double shape) {
    double boost = 1.0;
    if (shape < 1.0) {
        boost = pow(philox_u01(r), 1.0 / shape);
        shape += 1.0;
    }
    const double d = shape - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * d);
    for (int it = 0; it < 1000; ++it) {
        double x, v;
        do {
            x = philox_normal(r);
            v = 1.0 + c * x;
        } while (v <= 0.0);
        v = v * v * v;
        const double u = philox_u01(r);
        if (u < 1.0 - 0.0331 * x * x * x * x) return boost * d * v;
        if (log(u) < 0.5 * x * x + d * (1.0 - v + log(v))) return boost * d * v;
    }
    return boost * d;  // not reached in practice
}

// ---------------------------------------------------------------------------
// Discrete Gamma rates (the restated AS 32 / AS 91+R85 / AS 241 / ACM 291
// routines of crux_gb300/cxmath.py, FP64 on the device).
// ---------------------------------------------------------------------------
__device__ inline double d_ln_gamma(double x) {
    double shift = 0.0;
    if (x < 7.0) {
        double prod = 1.0, z = x;
        while (z < 7.0) {
            prod *= z;
            z += 1.0;
        }
        x = z;
        shift = -log(prod);
    }
    const double z = 1.0 / (x * x);
    const double series = (((-0.000595238095238 * z + 0.000793650793651) * z -
                            0.002777777777778) * z + 0.083333333333333) / x;
    return shift + (x - 0.5) * log(x) - x + 0.918938533204673 + series;
}

__device__ inline double d_gamma_inc(double x, double p, double lgp) {
    if (x == 0.0) return 0.0;
    const double acu = 1.0e-10, big = 1.0e30;
    const double factor = exp(p * log(x) - x - lgp);
    if (x <= 1.0 || x < p) {
        double total = 1.0, term = 1.0, rn = p;
        for (int it = 0; it < 100000; ++it) {
            rn += 1.0;
            term *= x / rn;
            total += term;
            if (term <= acu) break;
        }
        return total * factor / p;
    }
    double a = 1.0 - p, b = a + x + 1.0, cnt = 0.0;
    double p0 = 1.0, p1 = x, p2 = x + 1.0, p3 = x * b;
    double cur = p2 / p3;
    for (int it = 0; it < 100000; ++it) {
        a += 1.0;
        b += 2.0;
        cnt += 1.0;
        const double an = a * cnt;
        const double p4 = b * p2 - an * p0, p5 = b * p3 - an * p1;
        if (p5 != 0.0) {
            const double rn = p4 / p5, dif = fabs(cur - rn);
            if (dif <= acu && dif <= acu * rn) return 1.0 - factor * cur;
            cur = rn;
        }
        p0 = p2;
        p1 = p3;
        p2 = p4;
        p3 = p5;
        if (fabs(p4) >= big) {
            p0 /= big;
            p1 /= big;
            p2 /= big;
            p3 /= big;
        }
    }
    return 1.0 - factor * cur;
}

__device__ inline double d_poly(const double *c, int n, double r) {
    double acc = 0.0;
    for (int i = 0; i < n; ++i) acc = acc * r + c[i];
    return acc;
}

__device__ inline double d_norm_quantile(double p) {
    const double A[8] = {2.5090809287301226727e3, 3.3430575583588128105e4,
                         6.7265770927008700853e4, 4.5921953931549871457e4,
                         1.3731693765509461125e4, 1.9715909503065514427e3,
                         1.3314166789178437745e2, 3.3871328727963666080e0};
    const double B[8] = {5.2264952788528545610e3, 2.8729085735721942674e4,
                         3.9307895800092710610e4, 2.1213794301586595867e4,
                         5.3941960214247511077e3, 6.8718700749205790830e2,
                         4.2313330701600911252e1, 1.0};
    const double C[8] = {7.74545014278341407640e-4, 2.27238449892691845833e-2,
                         2.41780725177450611770e-1, 1.27045825245236838258e0,
                         3.64784832476320460504e0, 5.76949722146069140550e0,
                         4.63033784615654529590e0, 1.42343711074968357734e0};
    const double D[8] = {1.05075007164441684324e-9, 5.47593808499534494600e-4,
                         1.51986665636164571966e-2, 1.48103976427480074590e-1,
                         6.89767334985100004550e-1, 1.67638483018380384940e0,
                         2.05319162663775882187e0, 1.0};
    const double E[8] = {2.01033439929228813265e-7, 2.71155556874348757815e-5,
                         1.24266094738807843860e-3, 2.65321895265761230930e-2,
                         2.96560571828504891230e-1, 1.78482653991729133580e0,
                         5.46378491116411436990e0, 6.65790464350110377720e0};
    const double F[8] = {2.04426310338993978564e-15, 1.42151175831644588870e-7,
                         1.84631831751005468180e-5, 7.86869131145613259100e-4,
                         1.48753612908506148525e-2, 1.36929880922735805310e-1,
                         5.99832206555887937690e-1, 1.0};
    const double q = p - 0.5;
    if (fabs(q) <= 0.425) {
        const double r = 0.180625 - q * q;
        return q * d_poly(A, 8, r) / d_poly(B, 8, r);
    }
    double r = (q < 0.0) ? p : 1.0 - p;
    r = sqrt(-log(r));
    double v;
    if (r <= 5.0) {
        r -= 1.6;
        v = d_poly(C, 8, r) / d_poly(D, 8, r);
    } else {
        r -= 5.0;
        v = d_poly(E, 8, r) / d_poly(F, 8, r);
    }
    return q < 0.0 ? -v : v;
}

__device__ inline double d_chi2_quantile(double p, double v, double lg) {
    const double e = 5.0e-7, ln2 = 0.6931471805;
    const double xx = 0.5 * v, c = xx - 1.0;
    double ch;
    if (v < -1.24 * log(p)) {
        ch = pow(p * xx * exp(lg + xx * ln2), 1.0 / xx);
        if (ch - e < 0.0) return ch;
    } else if (v > 0.32) {
        const double x = d_norm_quantile(p);
        const double p1 = 0.222222 / v;
        ch = v * pow(x * sqrt(p1) + 1.0 - p1, 3.0);
        if (ch > 2.2 * v + 6.0)
            ch = -2.0 * (log(1.0 - p) - c * log(0.5 * ch) + lg);
    } else {
        ch = 0.4;
        const double a = log(1.0 - p);
        for (int it = 0; it < 1000; ++it) {
            const double q = ch;
            const double p1 = 1.0 + ch * (4.67 + ch);
            const double p2 = ch * (6.73 + ch * (6.66 + ch));
            const double t = -0.5 + (4.67 + 2.0 * ch) / p1 -
                             (6.73 + ch * (13.32 + 3.0 * ch)) / p2;
            ch -= (1.0 - exp(a + lg + 0.5 * ch + c * ln2) * p2 / p1) / t;
            if (fabs(q / ch - 1.0) - 0.01 <= 0.0) break;
        }
    }
    for (int it = 0; it < 20; ++it) {
        const double q = ch, p1 = 0.5 * ch;
        if (p1 < 0.0) return -1.0;
        const double p2 = p - d_gamma_inc(p1, xx, lg);
        const double t = p2 * exp(xx * ln2 + lg + p1 - c * log(ch));
        const double b = t / ch, a = 0.5 * t - b * c;
        const double s1 = (210.0 + a * (140.0 + a * (105.0 + a * (84.0 + a * (70.0 + 60.0 * a))))) / 420.0;
        const double s2 = (420.0 + a * (735.0 + a * (966.0 + a * (1141.0 + 1278.0 * a)))) / 2520.0;
        const double s3 = (210.0 + a * (462.0 + a * (707.0 + 932.0 * a))) / 2520.0;
        const double s4 = (252.0 + a * (672.0 + 1182.0 * a) + c * (294.0 + a * (889.0 + 1740.0 * a))) / 5040.0;
        const double s5 = (84.0 + 264.0 * a + c * (175.0 + 606.0 * a)) / 2520.0;
        const double s6 = (120.0 + c * (346.0 + 127.0 * c)) / 5040.0;
        ch += t * (1.0 + 0.5 * t * s1 - b * c * (s1 - b * (s2 - b * (s3 - b * (s4 - b * (s5 - b * s6))))));
        if (fabs(q / ch - 1.0) <= e) break;
    }
    return ch;
}

// Category means (median = false) of ncat equal-probability Gamma(alpha)
// categories, mean 1 (Lik.pyx:1222-1242), in two steps.  d_gamma_cut: the
// cumulative share of the mean below the i-th category boundary (i <
// ncat - 1); -1 if the quantile fails.  Categories are independent, so a
// warp computes them in parallel.
__device__ inline double d_gamma_cut(double alpha, int ncat, int i) {
    const double lga = d_ln_gamma(alpha), lga1 = d_ln_gamma(alpha + 1.0);
    const double pt = d_chi2_quantile((i + 1.0) / ncat, alpha * 2.0, lga);
    if (pt == -1.0) return -1.0;
    return d_gamma_inc(pt / 2.0, alpha + 1.0, lga1);
}

// Category mean rates from the cuts (rates[0..ncat-2] hold the cuts).
__device__ inline void d_gamma_rates_from_cuts(int ncat, double *rates) {
    rates[ncat - 1] = 1.0;
    for (int i = ncat - 1; i > 0; --i) {
        rates[i] -= rates[i - 1];
        rates[i] *= ncat;
    }
    rates[0] *= ncat;
}

}  // namespace cxg
