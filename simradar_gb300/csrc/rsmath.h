/*
 * rsmath.h -- portable single-precision elementary functions.
 *
 * The OpenCL kernels of SimRadar call log1p, log, acos, atan2, sincos, cos and
 * pow (rs.cl:151, rs.cl:212-215, rs.cl:268-280, rs.cl:282-359, rs.cl:590-648,
 * rs.cl:744-907, rs.cl:1050-1110).  OpenCL only bounds their error (several
 * ulp), so every device and every libm gives slightly different bits.  This
 * header evaluates each of them with a fixed sequence of IEEE single-precision
 * operations (add, sub, mul, div, sqrt, floor, rint, copysign: all correctly
 * rounded), so the CUDA kernels and the CPU oracle produce identical bits on
 * x86-64 and aarch64 hosts and on sm_103a.  That is what makes the respawn RNG
 * state, the positions and the scatterer-to-gate indices bit-exact between the
 * GPU and the oracle even on the stretched LES grid, where log1p feeds the
 * wind lookup every pulse.
 *
 * Methods (textbook mathematics; coefficients from the Taylor series or from
 * least-squares fits made for this file, as noted):
 *   - sin/cos: Cody-Waite reduction by pi/2 split in three floats, applied
 *     with fmaf (the first step is exact for |x| < 2^22 * pi/2), then the
 *     Taylor polynomials of sin (to x^9) and cos (to x^10) on [-pi/4, pi/4].
 *   - log: x = m 2^e with m in [sqrt(1/2), sqrt(2)), log(m) = f - f^2/2 +
 *     f^3 P(f), f = m - 1, P a degree-7 least-squares fit made for this file
 *     (relative error 7.7e-9); e*ln2 added as a 16-bit head + tail.  No
 *     division.
 *   - log1p: the same polynomial on x inside sqrt(1/2) - 1 < x < sqrt(2) - 1;
 *     outside, log(u) + e / u with u = 1 + x rounded and e = (1 + x) - u
 *     formed exactly (the correction is below an ulp, so 1/u comes from the
 *     exponent and one Newton step, again without a division).
 *   - asin/acos: asin(s) = s + s^3 P(s^2) on |s| <= 1/2, P a degree-4
 *     least-squares fit made for this file (0.62 ulp in exact arithmetic),
 *     and the half-angle identity acos(x) = 2 asin(sqrt((1-x)/2)) above.
 *   - atan/atan2: reduction to [0, 1], then to |u| <= tan(pi/8) by
 *     atan(t) = pi/4 + atan((t-1)/(t+1)), atan(u) = u + u^3 Q(u^2) with Q a
 *     degree-5 least-squares fit made for this file (0.59 ulp).
 *   - exp: k = rint(x/ln2), r = x - k ln2 (two-part), Taylor to r^7, 2^k by
 *     exponent construction.  pow(b, e) = exp(e log b) with the rounding error
 *     of the product carried by fmaf.
 *
 * Polynomials are evaluated with fmaf (one correctly rounded operation on both
 * the CPU and the GPU).  The CUDA translation unit that includes this header
 * is compiled with -fmad=false and the oracle with -ffp-contract=off, so any
 * "a * b + c" not written as fmaf is two rounded operations on both sides.
 * Measured accuracy against float64 references is checked by the CPU tests.
 */
#ifndef SIMRADAR_GB300_RSMATH_H
#define SIMRADAR_GB300_RSMATH_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define RSM_FN static __host__ __device__ __forceinline__
#else
#define RSM_FN static inline
#endif

/* pi/2 in three floats; pi and pi/2 as head + tail */
#define RSM_PIO2_1   0x1.921fb6p+0f
#define RSM_PIO2_2  (-0x1.777a5cp-25f)
#define RSM_PIO2_3  (-0x1.ee59dap-50f)
#define RSM_PI_HI    0x1.921fb6p+1f
#define RSM_PI_LO   (-0x1.777a5cp-24f)
#define RSM_PIO2_HI  0x1.921fb6p+0f
#define RSM_PIO2_LO (-0x1.777a5cp-25f)
#define RSM_PIO4_HI  0x1.921fb6p-1f
#define RSM_PIO4_LO (-0x1.777a5cp-26f)
#define RSM_LN2_HI   0x1.62e400p-1f
#define RSM_LN2_LO   0x1.7f7d1cp-20f
#define RSM_TWO_OVER_PI 0x1.45f306p-1f
#define RSM_INV_LN2  0x1.715476p+0f
#define RSM_SQRT2    0x1.6a09e6p+0f
#define RSM_TAN_PIO8 0x1.a8279ap-2f

RSM_FN uint32_t rsm_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, sizeof(u));
    return u;
#endif
}

RSM_FN float rsm_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, sizeof(f));
    return f;
#endif
}

RSM_FN int rsm_isnan(float x) { return x != x; }

/* 2^k for k in [-149, 127] (exact) */
RSM_FN float rsm_exp2i(int k) {
    if (k >= -126) {
        return rsm_u2f((uint32_t)(k + 127) << 23);
    }
    return rsm_u2f(1u << (uint32_t)(k + 149));
}

/* x - q pi/2 for q = rint(x 2/pi); the first step is exact for |x| < 2^22 pi/2 */
RSM_FN float rsm_reduce_pio2(float x, float *q_out) {
    float q = rintf(x * RSM_TWO_OVER_PI);
    float r = fmaf(-q, RSM_PIO2_1, x);
    r = fmaf(-q, RSM_PIO2_2, r);
    r = fmaf(-q, RSM_PIO2_3, r);
    *q_out = q;
    return r;
}

/* sin and cos of (r + q pi/2) for a reduced argument |r| <~ pi/4 and an
 * integer-valued float q */
RSM_FN void rsm_sincos_reduced(float r, float q, float *s_out, float *c_out) {
    float z = r * r;
    /* sin(r) = r + r z (-1/6 + z (1/120 + z (-1/5040 + z / 362880))) */
    float ps = 0x1.71de3ap-19f;              /*  1/362880 */
    ps = fmaf(ps, z, (-0x1.a01a02p-13f));        /* -1/5040   */
    ps = fmaf(ps, z, 0x1.111112p-7f);            /*  1/120    */
    ps = fmaf(ps, z, (-0x1.555556p-3f));         /* -1/6      */
    float sn = fmaf(r * z, ps, r);
    /* cos(r) = 1 + z (-1/2 + z (1/24 + z (-1/720 + z (1/40320 - z / 3628800)))) */
    float pc = -0x1.27e4fcp-22f;             /* -1/3628800 */
    pc = fmaf(pc, z, 0x1.a01a02p-16f);           /*  1/40320   */
    pc = fmaf(pc, z, (-0x1.6c16c2p-10f));        /* -1/720     */
    pc = fmaf(pc, z, 0x1.555556p-5f);            /*  1/24      */
    pc = fmaf(pc, z, (-0.5f));
    float cs = fmaf(z, pc, 1.0f);
    /* quadrant from the low two bits of q (an integer-valued float, |q| <
     * 2^23, so the conversion is exact; two's complement gives q mod 4 for
     * negative q too): (sin, cos) of r + quad pi/2 = (sn, cs), (cs, -sn),
     * (-sn, -cs), (-cs, sn) */
    const int quad = (int)q & 3;
    const int swap = quad & 1;
    float s = swap ? cs : sn;
    float c = swap ? sn : cs;
    *s_out = (quad & 2) ? -s : s;
    *c_out = ((quad + 1) & 2) ? -c : c;
}

/* sin and cos of x.  Accurate for |x| < 6.7e6; beyond that the reduction
 * loses bits (the kernels never pass such phases: k*r at 30 km is 3.8e6). */
RSM_FN void rsm_sincosf(float x, float *s_out, float *c_out) {
    if (!(fabsf(x) < INFINITY)) {
        float n = x - x;
        *s_out = n;
        *c_out = n;
        return;
    }
    float q;
    float r = rsm_reduce_pio2(x, &q);
    rsm_sincos_reduced(r, q, s_out, c_out);
}

RSM_FN float rsm_sinf(float x) {
    float s, c;
    rsm_sincosf(x, &s, &c);
    return s;
}

RSM_FN float rsm_cosf(float x) {
    float s, c;
    rsm_sincosf(x, &s, &c);
    return c;
}

/* log(1 + f) for f in [sqrt(1/2) - 1, sqrt(2) - 1]: f - f^2 / 2 + f^3 P(f)
 * with P of degree 7, a weighted least-squares fit of the relative error
 * (7.7e-9 with these single-precision coefficients); no division. */
RSM_FN float rsm_log1p_core(float f) {
    float p = -0x1.38b4a6p-4f;
    p = fmaf(p, f, 0x1.055b42p-3f);
    p = fmaf(p, f, -0x1.0d8558p-3f);
    p = fmaf(p, f, 0x1.22da24p-3f);
    p = fmaf(p, f, -0x1.547242p-3f);
    p = fmaf(p, f, 0x1.99a008p-3f);
    p = fmaf(p, f, -0x1.000228p-2f);
    p = fmaf(p, f, 0x1.555554p-2f);
    float z = f * f;
    float t = fmaf(f * z, p, -0.5f * z);
    return f + t;
}

/* natural logarithm */
RSM_FN float rsm_logf(float x) {
    if (rsm_isnan(x) || x < 0.0f) {
        return (x - x) / (x - x);            /* NaN */
    }
    if (x == 0.0f) {
        return -INFINITY;
    }
    if (x == INFINITY) {
        return x;
    }
    int e = 0;
    if (x < 0x1p-126f) {                      /* subnormal: scale up (exact) */
        x = x * 0x1p23f;
        e = -23;
    }
    uint32_t u = rsm_f2u(x);
    e += (int)((u >> 23) & 0xff) - 127;
    float m = rsm_u2f((u & 0x007fffffu) | 0x3f800000u);   /* [1, 2) */
    if (m > RSM_SQRT2) {
        m = m * 0.5f;                         /* exact */
        e += 1;
    }
    float f = m - 1.0f;                       /* exact (Sterbenz) */
    float lm = rsm_log1p_core(f);
    float fe = (float)e;
    return fe * RSM_LN2_HI + fmaf(fe, RSM_LN2_LO, lm);
}

/* log(1 + x) */
RSM_FN float rsm_log1pf(float x) {
    if (x > -0x1.2bec34p-2f && x < 0x1.a8279ap-2f) {
        /* 1 + x in [sqrt(1/2), sqrt(2)): the polynomial on x directly,
         * without rounding 1 + x */
        return rsm_log1p_core(x);
    }
    const float u = 1.0f + x;
    if (rsm_isnan(x) || !(u > 0.0f) || u == INFINITY) {
        return rsm_logf(u);
    }
    /* u = m 2^k is normal here (u >= 2^-24).  log(1 + x) = log(u) +
     * log(1 + e / u) with e = (1 + x) - u, exact (u - 1 is exact below 2^24,
     * and above it e / u is far below an ulp of the result); e / u < 2^-24,
     * so log(1 + e / u) = e / u and 1 / u needs only a few correct bits:
     * 2^-k (1.5 - m / 2) for m in [1, 2), refined once by Newton's step.  The
     * correction joins the polynomial's small part before the k ln 2 head. */
    const float e = x - (u - 1.0f);
    const uint32_t b = rsm_f2u(u);
    int k = (int)(b >> 23) - 127;
    const float m1 = rsm_u2f((b & 0x007fffffu) | 0x3f800000u);
    float y = 1.5f - 0.5f * m1;
    y = y * (2.0f - m1 * y);
    const float inv = y * rsm_u2f((uint32_t)(127 - k) << 23);
    float m = m1;
    if (m > RSM_SQRT2) {
        m = m * 0.5f;                         /* exact */
        k += 1;
    }
    const float fk = (float)k;
    return fk * RSM_LN2_HI + fmaf(fk, RSM_LN2_LO, rsm_log1p_core(m - 1.0f) + e * inv);
}

/* the degree-4 fit P of asin(s) = s + s z P(z), z = s^2, |s| <= 1/2 */
RSM_FN float rsm_asin_poly(float z) {
    float p = 0x1.5625d6p-5f;
    p = fmaf(p, z, 0x1.8ff98cp-6f);
    p = fmaf(p, z, 0x1.741a60p-5f);
    p = fmaf(p, z, 0x1.330612p-4f);
    return fmaf(p, z, 0x1.5555bap-3f);
}

/* asin on |s| <= 1/2 : s + s z P(z) */
RSM_FN float rsm_asin_core(float s, float z) {
    return fmaf(s * z, rsm_asin_poly(z), s);
}

/* Every acos of the kernels takes a cosine formed from unit vectors or a unit
 * quaternion (rs.cl:210, 327, 330, 485, 488, 855, 1066, 1451); rounding can
 * carry it just past +-1, where the OpenCL builtin returns NaN and the NaN
 * then reaches the scatterer's state and every range gate.  An argument
 * within 16 ulp beyond +-1 is taken as +-1 here (a leaf whose relative wind
 * lies along its body axis has beta = 0); inside [-1, 1], further out and
 * for NaN nothing changes. */
RSM_FN float rsm_acosf(float x) {
    float ax = fabsf(x);
    if (ax > 1.0f && ax <= 0x1.00002p+0f) {
        x = x > 0.0f ? 1.0f : -1.0f;
        ax = 1.0f;
    }
    if (rsm_isnan(x) || ax > 1.0f) {
        return (x - x) / (x - x);
    }
    if (ax <= 0.5f) {
        float a = rsm_asin_core(x, x * x);
        return RSM_PIO2_HI - (a - RSM_PIO2_LO);
    }
    float z = (1.0f - ax) * 0.5f;             /* exact */
    float s = sqrtf(z);
    float a = 2.0f * rsm_asin_core(s, z);
    if (x > 0.0f) {
        return a;
    }
    return RSM_PI_HI - (a - RSM_PI_LO);
}

/* atan on |u| <= tan(pi/8) : u + u z Q(z), Q the degree-5 fit */
RSM_FN float rsm_atan_core(float u) {
    float z = u * u;
    float q = 0x1.889eccp-5f;
    q = fmaf(q, z, -0x1.5c2c30p-4f);
    q = fmaf(q, z, 0x1.c49292p-4f);
    q = fmaf(q, z, -0x1.2480d4p-3f);
    q = fmaf(q, z, 0x1.99992cp-3f);
    q = fmaf(q, z, -0x1.555554p-2f);
    return fmaf(u * z, q, u);
}

/* atan of t in [0, 1] */
RSM_FN float rsm_atan01(float t) {
    if (t > RSM_TAN_PIO8) {
        float u = (t - 1.0f) / (t + 1.0f);
        return RSM_PIO4_HI + (rsm_atan_core(u) + RSM_PIO4_LO);
    }
    return rsm_atan_core(t);
}

RSM_FN float rsm_atan2f(float y, float x) {
    if (rsm_isnan(x) || rsm_isnan(y)) {
        return x + y;
    }
    float ax = fabsf(x);
    float ay = fabsf(y);
    float a;
    if (ay == 0.0f) {
        /* atan2(+-0, x) = +-0 for x > 0 or x = +0, +-pi for x < 0 or x = -0 */
        a = (x < 0.0f || (x == 0.0f && (rsm_f2u(x) >> 31))) ? RSM_PI_HI : 0.0f;
        return copysignf(a, y);
    }
    if (ax == INFINITY || ay == INFINITY) {
        if (ax == INFINITY && ay == INFINITY) {
            a = x > 0.0f ? RSM_PIO4_HI : 3.0f * RSM_PIO4_HI;
        } else if (ax == INFINITY) {
            a = x > 0.0f ? 0.0f : RSM_PI_HI;
        } else {
            a = RSM_PIO2_HI;
        }
        return copysignf(a, y);
    }
    if (ay > ax) {
        a = rsm_atan01(ax / ay);
        a = RSM_PIO2_HI - (a - RSM_PIO2_LO);
    } else {
        a = rsm_atan01(ay / ax);
    }
    if (x < 0.0f) {
        a = RSM_PI_HI - (a - RSM_PI_LO);
    }
    return copysignf(a, y);
}

/* e^x */
RSM_FN float rsm_expf(float x) {
    if (rsm_isnan(x)) {
        return x;
    }
    if (x > 88.7228394f) {
        return INFINITY;
    }
    if (x < -103.972076f) {
        return 0.0f;
    }
    float k = rintf(x * RSM_INV_LN2);
    float r = fmaf(-k, RSM_LN2_LO, x - k * RSM_LN2_HI);
    /* e^r, |r| <= ln2/2, Taylor series to r^7 */
    float p = 0x1.a01a02p-13f;                /* 1/5040 */
    p = fmaf(p, r, 0x1.6c16c2p-10f);              /* 1/720  */
    p = fmaf(p, r, 0x1.111112p-7f);               /* 1/120  */
    p = fmaf(p, r, 0x1.555556p-5f);               /* 1/24   */
    p = fmaf(p, r, 0x1.555556p-3f);               /* 1/6    */
    p = fmaf(p, r, 0.5f);
    float er = 1.0f + fmaf(r * r, p, r);
    int ki = (int)k;
    if (ki > 127) {
        return (er * 2.0f) * rsm_exp2i(ki - 1);
    }
    if (ki < -125) {
        return (er * rsm_exp2i(ki + 64)) * 0x1p-64f;
    }
    return er * rsm_exp2i(ki);
}

/* b^e for b >= 0 (the kernels raise 10 and the stretch ratios) */
RSM_FN float rsm_powf(float b, float e) {
    if (e == 0.0f || b == 1.0f) {
        return 1.0f;
    }
    if (rsm_isnan(b) || rsm_isnan(e)) {
        return b + e;
    }
    if (b < 0.0f) {
        return (b - b) / (b - b);
    }
    if (b == 0.0f) {
        return e > 0.0f ? 0.0f : INFINITY;
    }
    float l = rsm_logf(b);
    float p = e * l;
    float perr = fmaf(e, l, -p);             /* rounding error of e * l */
    float r = rsm_expf(p);
    return fmaf(r, perr, r);
}

#endif /* SIMRADAR_GB300_RSMATH_H */
