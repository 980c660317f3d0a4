"""Discrete-Gamma rate categories, FP64 host math.

Restates, from the published algorithms, the four routines that
``Lik.setAlpha`` (pkg/Crux/Tree/Lik.pyx:1196-1278) uses via
lib/Crux/CxMath.pxd:125-368:

* ``ln_gamma``   log Gamma(x): Pike & Hill (1966), CACM Algorithm 291
                 (shift x up to >= 7, then the Stirling series).
* ``gamma_inc``  regularised lower incomplete Gamma ratio: Bhattacharjee
                 (1970), Applied Statistics AS 32 (series for x <= max(1, p),
                 else a continued fraction), accuracy 1e-10.
* ``norm_quantile``  standard-normal quantile: Wichura (1988), AS 241
                 (PPND16, rational approximations in three regions).
* ``chi2_quantile``  chi-square quantile: Best & Roberts (1975), AS 91, with
                 Shea's (1991) AS R85 remark (starting value, then a
                 seven-term Taylor refinement), tolerance 5e-7.

``gamma_rates(alpha, ncat, median)`` returns the category multipliers that
``setAlpha`` stores in ``cmult``: category means (the default) or medians,
each scaled to mean 1.
"""
import math

_LN_SQRT_2PI = 0.918938533204673


def ln_gamma(x):
    assert x > 0.0
    shift = 0.0
    if x < 7.0:
        prod = 1.0
        z = x
        while z < 7.0:
            prod *= z
            z += 1.0
        x = z
        shift = -math.log(prod)
    z = 1.0 / (x * x)
    series = (((-0.000595238095238 * z + 0.000793650793651) * z
               - 0.002777777777778) * z + 0.083333333333333) / x
    return shift + (x - 0.5) * math.log(x) - x + _LN_SQRT_2PI + series


def gamma_inc(x, p, ln_gamma_p):
    """P(p, x) = (1/Gamma(p)) int_0^x t^(p-1) e^-t dt."""
    assert p > 0.0 and x >= 0.0
    if x == 0.0:
        return 0.0
    acu = 1.0e-10
    big = 1.0e30
    factor = math.exp(p * math.log(x) - x - ln_gamma_p)
    if x <= 1.0 or x < p:
        total = 1.0
        term = 1.0
        rn = p
        while True:
            rn += 1.0
            term *= x / rn
            total += term
            if term <= acu:
                return total * factor / p
    a = 1.0 - p
    b = a + x + 1.0
    cnt = 0.0
    p0, p1, p2, p3 = 1.0, x, x + 1.0, x * b
    cur = p2 / p3
    while True:
        a += 1.0
        b += 2.0
        cnt += 1.0
        an = a * cnt
        p4 = b * p2 - an * p0
        p5 = b * p3 - an * p1
        if p5 != 0.0:
            rn = p4 / p5
            dif = abs(cur - rn)
            if dif <= acu and dif <= acu * rn:
                return 1.0 - factor * cur
            cur = rn
        p0, p1, p2, p3 = p2, p3, p4, p5
        if abs(p4) >= big:
            p0 /= big
            p1 /= big
            p2 /= big
            p3 /= big


def _poly(coefs, r):
    """Horner evaluation, highest-order coefficient first."""
    acc = 0.0
    for c in coefs:
        acc = acc * r + c
    return acc


# AS 241 (PPND16) coefficient sets, highest order first.
_A = (2.5090809287301226727e3, 3.3430575583588128105e4,
      6.7265770927008700853e4, 4.5921953931549871457e4,
      1.3731693765509461125e4, 1.9715909503065514427e3,
      1.3314166789178437745e2, 3.3871328727963666080e0)
_B = (5.2264952788528545610e3, 2.8729085735721942674e4,
      3.9307895800092710610e4, 2.1213794301586595867e4,
      5.3941960214247511077e3, 6.8718700749205790830e2,
      4.2313330701600911252e1, 1.0)
_C = (7.74545014278341407640e-4, 2.27238449892691845833e-2,
      2.41780725177450611770e-1, 1.27045825245236838258e0,
      3.64784832476320460504e0, 5.76949722146069140550e0,
      4.63033784615654529590e0, 1.42343711074968357734e0)
_D = (1.05075007164441684324e-9, 5.47593808499534494600e-4,
      1.51986665636164571966e-2, 1.48103976427480074590e-1,
      6.89767334985100004550e-1, 1.67638483018380384940e0,
      2.05319162663775882187e0, 1.0)
_E = (2.01033439929228813265e-7, 2.71155556874348757815e-5,
      1.24266094738807843860e-3, 2.65321895265761230930e-2,
      2.96560571828504891230e-1, 1.78482653991729133580e0,
      5.46378491116411436990e0, 6.65790464350110377720e0)
_F = (2.04426310338993978564e-15, 1.42151175831644588870e-7,
      1.84631831751005468180e-5, 7.86869131145613259100e-4,
      1.48753612908506148525e-2, 1.36929880922735805310e-1,
      5.99832206555887937690e-1, 1.0)


def norm_quantile(p):
    assert 0.0 < p < 1.0
    q = p - 0.5
    if abs(q) <= 0.425:
        r = 0.180625 - q * q
        return q * _poly(_A, r) / _poly(_B, r)
    r = p if q < 0.0 else 1.0 - p
    r = math.sqrt(-math.log(r))
    if r <= 5.0:
        r -= 1.6
        val = _poly(_C, r) / _poly(_D, r)
    else:
        r -= 5.0
        val = _poly(_E, r) / _poly(_F, r)
    return -val if q < 0.0 else val


def chi2_quantile(p, v, ln_gamma_half_v):
    """Point z with P(chi2_v <= z) = p; -1.0 on failure (AS 91 ifault)."""
    assert 0.0 <= p < 1.0 and v > 0.0
    e = 5.0e-7
    ln2 = 0.6931471805
    xx = 0.5 * v
    c = xx - 1.0
    if v < -1.24 * math.log(p):
        ch = math.pow(p * xx * math.exp(ln_gamma_half_v + xx * ln2), 1.0 / xx)
        if ch - e < 0.0:
            return ch
    elif v > 0.32:
        x = norm_quantile(p)
        p1 = 0.222222 / v
        ch = v * math.pow(x * math.sqrt(p1) + 1.0 - p1, 3.0)
        if ch > 2.2 * v + 6.0:
            ch = -2.0 * (math.log(1.0 - p) - c * math.log(0.5 * ch)
                         + ln_gamma_half_v)
    else:
        ch = 0.4
        a = math.log(1.0 - p)
        while True:
            q = ch
            p1 = 1.0 + ch * (4.67 + ch)
            p2 = ch * (6.73 + ch * (6.66 + ch))
            t = -0.5 + (4.67 + 2.0 * ch) / p1 \
                - (6.73 + ch * (13.32 + 3.0 * ch)) / p2
            ch -= (1.0 - math.exp(a + ln_gamma_half_v + 0.5 * ch + c * ln2)
                   * p2 / p1) / t
            if abs(q / ch - 1.0) - 0.01 <= 0.0:
                break
    for _ in range(20):
        q = ch
        p1 = 0.5 * ch
        if p1 < 0.0:
            return -1.0
        p2 = p - gamma_inc(p1, xx, ln_gamma_half_v)
        t = p2 * math.exp(xx * ln2 + ln_gamma_half_v + p1 - c * math.log(ch))
        b = t / ch
        a = 0.5 * t - b * c
        s1 = (210.0 + a * (140.0 + a * (105.0 + a * (84.0 + a * (70.0
              + 60.0 * a))))) / 420.0
        s2 = (420.0 + a * (735.0 + a * (966.0 + a * (1141.0
              + 1278.0 * a)))) / 2520.0
        s3 = (210.0 + a * (462.0 + a * (707.0 + 932.0 * a))) / 2520.0
        s4 = (252.0 + a * (672.0 + 1182.0 * a) + c * (294.0 + a * (889.0
              + 1740.0 * a))) / 5040.0
        s5 = (84.0 + 264.0 * a + c * (175.0 + 606.0 * a)) / 2520.0
        s6 = (120.0 + c * (346.0 + 127.0 * c)) / 5040.0
        ch += t * (1.0 + 0.5 * t * s1 - b * c * (s1 - b * (s2 - b * (s3
                   - b * (s4 - b * (s5 - b * s6))))))
        if abs(q / ch - 1.0) <= e:
            break
    return ch


def gamma_rates(alpha, ncat, median=False):
    """Rate multipliers of ncat equal-probability Gamma(alpha) categories.

    Means (Lik.pyx:1222-1242): category boundaries from chi2 quantiles at
    i/ncat with 2*alpha degrees of freedom, then differences of
    P(alpha+1, boundary/2) times ncat.  Medians (Lik.pyx:1243-1260): chi2
    quantiles at (2i+1)/(2 ncat) divided by 2 alpha, rescaled to mean 1.
    Raises OverflowError when the quantile routine fails.
    """
    lga = ln_gamma(alpha)
    rates = [0.0] * ncat
    if not median:
        lga1 = ln_gamma(alpha + 1.0)
        for i in range(ncat - 1):
            pt = chi2_quantile((i + 1.0) / ncat, alpha * 2.0, lga)
            if pt == -1.0:
                raise OverflowError("Error discretizing gamma (ncat=%d, "
                                    "alpha=%e)" % (ncat, alpha))
            rates[i] = gamma_inc(pt / 2.0, alpha + 1.0, lga1)
        rates[ncat - 1] = 1.0
        for i in range(ncat - 1, 0, -1):
            rates[i] -= rates[i - 1]
            rates[i] *= ncat
        rates[0] *= ncat
    else:
        total = 0.0
        for i in range(ncat):
            pt = chi2_quantile((i * 2 + 1.0) / (ncat * 2), alpha * 2.0, lga)
            if pt == -1.0:
                raise OverflowError("Error discretizing gamma (ncat=%d, "
                                    "alpha=%e)" % (ncat, alpha))
            pt /= alpha * 2.0
            total += pt
            rates[i] = pt
        for i in range(ncat):
            rates[i] *= ncat / total
    return rates
