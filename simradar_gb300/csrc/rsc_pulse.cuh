/*
 * rsc_pulse.cuh -- pulse formation on sm_103a: scat_sig_aux, make_pulse_pass_1
 * and make_pulse_pass_2 (rs.cl:1050-1441) as one kernel.
 *
 * Each thread forms its scatterer's signal in registers and adds it only to the
 * gates the range weight can reach (the weights are the pass-1 weights, bit for
 * bit).  Sums go into per-warp gate bins in shared memory; each block adds its
 * sum per gate into an FP64 accumulator in global memory (one atomic per gate
 * and lane) and the last block to finish converts it, so the pulse comes out
 * of a single launch with no serial tail.
 *
 *   RSC_PULSE_PLAIN        FP32 throughout, as the reference; per-warp bins
 *                          updated with shared-memory atomics.
 *   RSC_PULSE_COMPENSATED  every factor of a term as a double-float (range,
 *                          beam angle, table lerps, split range phase and its
 *                          sine and cosine, 1 / r^2, rotation), FP64 gate
 *                          origins; the warp sums each gate with an error-free
 *                          butterfly into double-float bins, the block sums
 *                          double-float and the grid FP64.
 *   RSC_PULSE_F64          FP64 reference of the same FP32 state: per-warp
 *                          FP64 bins, lanes on the same gate serialised.
 *
 * Bins of FP32 sums are 5 floats apart per gate so that lanes on different
 * gates rarely meet in one shared-memory bank (5 is prime to the 32 banks).
 */
#ifndef SIMRADAR_GB300_RSC_PULSE_CUH
#define SIMRADAR_GB300_RSC_PULSE_CUH

#include "rsc_kernels.cuh"
#include "rsc_sincos_table.h"

namespace rsc {

constexpr unsigned kBinStride32 = 5;   /* floats per gate in an FP32 bin row */

/* Table lerp at index (a_hi + a_lo) * desc[0] + desc[1], clamped to
 * [0, desc[2]], with the rounding error of the index computation carried into
 * the interpolation fraction (compensated form). */
__device__ __forceinline__ float weight_comp(const float *W, const float *desc, float a_hi, float a_lo) {
    const float s = desc[0], o = desc[1], m = desc[2];
    float p = a_hi * s;
    float pe = fmaf(a_hi, s, -p) + a_lo * s;
    float f, fe;
    two_sum(p, o, f, fe);
    fe = fe + pe;
    const float fsum = f + fe;
    if (!(fsum > 0.0f)) return __ldg(W);
    if (fsum >= m) return __ldg(W + (int)m);
    const float fl = floorf(fsum);
    float frac = fminf(fmaxf((f - fl) + fe, 0.0f), 1.0f);
    const int i0 = (int)fl;
    const int i1 = min(i0 + 1, (int)m);
    const float w0 = __ldg(W + i0), w1 = __ldg(W + i1);
    return fmaf(w1 - w0, frac, w0);
}

/* The compensated range weight.  On the triangle {0, 1, 0} with origin 1 and
 * max 2 the weight is 1 - |t| for t = index - 1 = p + pe, with p + pe the
 * double-float (a_hi + a_lo) s: no addition of the origin.  With sg the
 * sign of t, 1 - |t| = (1 - sg p) - sg pe, where 1 - sg p is exact for the
 * |p| within a factor 2 of 1 where the weight is small, and the tail joins
 * in one rounding: the weight keeps its relative accuracy up to the edges of
 * the support (1.2e-7 against 3e-5 for weight_comp, whose 1 - frac cancels
 * there).  Other tables go through weight_comp. */
__device__ __forceinline__ float range_weight_comp(const float *W, const float *desc, int tri, float a_hi,
                                                   float a_lo) {
    if (!tri) return weight_comp(W, desc, a_hi, a_lo);
    const float s = desc[0];
    const float p = a_hi * s;
    const float pe = fmaf(a_hi, s, -p) + a_lo * s;
    const float sg = (p + pe) < 0.0f ? -1.0f : 1.0f;
    return fmaxf((1.0f - sg * p) - sg * pe, 0.0f);
}

/* weight_comp as a double-float (wh + wl): the fraction (f - fl) + fe kept
 * as a pair (f - fl is exact), the table difference w1 - w0 exact
 * (two_sum), their product and the sum with w0 error-free but for the
 * product of the tails -- the lerp of the FP32 table at the double-float
 * index, to ~1e-14 of the weight. */
__device__ __forceinline__ void weight_comp_df(const float *W, const float *desc, float a_hi, float a_lo, float &wh,
                                               float &wl) {
    const float s = desc[0], o = desc[1], m = desc[2];
    float p = a_hi * s;
    float pe = fmaf(a_hi, s, -p) + a_lo * s;
    float f, fe;
    two_sum(p, o, f, fe);
    fe = fe + pe;
    const float fsum = f + fe;
    wl = 0.0f;
    if (!(fsum > 0.0f)) {
        wh = __ldg(W);
        return;
    }
    if (fsum >= m) {
        wh = __ldg(W + (int)m);
        return;
    }
    const float fl = floorf(fsum);
    float fh = f - fl, fr = fe;
    const float ft = fh + fr;
    if (ft <= 0.0f) {
        fh = 0.0f;
        fr = 0.0f;
    } else if (ft >= 1.0f) {
        fh = 1.0f;
        fr = 0.0f;
    }
    const int i0 = (int)fl;
    const int i1 = min(i0 + 1, (int)m);
    const float w0 = __ldg(W + i0), w1 = __ldg(W + i1);
    float dh, dl;
    two_sum(w1, -w0, dh, dl);
    float ph, pl;
    df_mul_pair(dh, dl, fh, fr, ph, pl);
    float sh, se;
    two_sum(w0, ph, sh, se);
    fast_two_sum(sh, se + pl, wh, wl);
}

/* range_weight_comp as a double-float: on the triangle 1 - |t| with the
 * head 1 - sg p formed error-free. */
__device__ __forceinline__ void range_weight_comp_df(const float *W, const float *desc, int tri, float a_hi, float a_lo,
                                                     float &wh, float &wl) {
    if (!tri) {
        weight_comp_df(W, desc, a_hi, a_lo, wh, wl);
        return;
    }
    const float s = desc[0];
    const float p = a_hi * s;
    const float pe = fmaf(a_hi, s, -p) + a_lo * s;
    const float sg = (p + pe) < 0.0f ? -1.0f : 1.0f;
    float h, e;
    two_sum(1.0f, -sg * p, h, e);
    const float l = e - sg * pe;
    const bool pos = (h + l) > 0.0f;
    wh = pos ? h : 0.0f;
    wl = pos ? l : 0.0f;
}

/* double-float helpers: (hi, lo) with |lo| <= ulp(hi) / 2 */
__device__ __forceinline__ void df_add(float ah, float al, float bh, float bl, float &h, float &l) {
    float s, e;
    two_sum(ah, bh, s, e);
    e = e + (al + bl);
    h = s + e;
    l = e - (h - s);
}
/* In both the correction c is a few ulps of the head, so an approximate
 * quotient for it (__fdividef, 2 ulp) leaves the pair accurate to ~1e-14;
 * the head of the quotient is corrected the same way. */
__device__ __forceinline__ void df_sqrt(float ah, float al, float &h, float &l) {
    float r = sqrtf(ah);
    float c = __fdividef(fmaf(-r, r, ah) + al, 2.0f * r);
    h = r + c;
    l = c - (h - r);
}
__device__ __forceinline__ void df_div(float ah, float al, float bh, float bl, float &h, float &l) {
    float q = __fdividef(ah, bh);
    float c = __fdividef(fmaf(-q, bh, ah) + al - q * bl, bh);
    h = q + c;
    l = c - (h - q);
}
/* a * b exactly as a double-float, minus c * d exactly as a double-float */
__device__ __forceinline__ void df_prod_diff(float a, float b, float c, float d, float &h, float &l) {
    float p, pe, q, qe;
    two_prod(a, b, p, pe);
    two_prod(c, d, q, qe);
    df_add(p, pe, -q, -qe, h, l);
}
/* sum of squares of three double-floats (the squares of the tails dropped) */
__device__ __forceinline__ void df_norm2(const float *h3, const float *l3, float &h, float &l) {
    float sh, sl;
    two_prod(h3[0], h3[0], sh, sl);
    sl = fmaf(2.0f * h3[0], l3[0], sl);
#pragma unroll
    for (int i = 1; i < 3; i++) {
        float p, pe;
        two_prod(h3[i], h3[i], p, pe);
        pe = fmaf(2.0f * h3[i], l3[i], pe);
        df_add(sh, sl, p, pe, sh, sl);
    }
    h = sh;
    l = sl;
}

/* sum of squares of three floats as a double-float (df_norm2 with zero
 * tails: the first square starts the sum) */
__device__ __forceinline__ void df_norm2_f(const float *h3, float &h, float &l) {
    float sh, sl;
    two_prod(h3[0], h3[0], sh, sl);
#pragma unroll
    for (int i = 1; i < 3; i++) {
        float p, pe;
        two_prod(h3[i], h3[i], p, pe);
        df_add(sh, sl, p, pe, sh, sl);
    }
    h = sh;
    l = sl;
}

/* x - q pi/2 as a double-float for x = xh + xsh + xsl, with xh an FP32
 * value and xsh + xsl a small double-float (|xsh| < 1: the tails of a
 * split product), q the integer nearest to x 2/pi.  q is found from x 2/pi
 * formed as a double-float (2/pi in two parts, the head product exact): a
 * single FP32 product rounds to a quarter near 4e6 rad (the phase at 30 km)
 * and 2/pi in one float is off by 4e-8 of it, which together can leave q
 * one off.  xh - q RSM_PIO2_1 is exact (xh is a multiple of the ulp of
 * RSM_PIO2_1, or q is 0 or 1, and the difference is below 1 in magnitude,
 * for |xh| < 2^22); q RSM_PIO2_2 is subtracted as an exact product and xsh
 * added error-free, so only the terms below 1e-7 (the product errors, the
 * third part of pi/2 and xsl) are rounded: the result is within ~1e-15 rad
 * of x - q pi/2 whatever the size of x. */
__device__ __forceinline__ void reduce_pio2_df(float xh, float xsh, float xsl, float &q, float &rh, float &rl) {
    float ph, pl;
    two_prod(xh, RSM_TWO_OVER_PI, ph, pl);
    pl = fmaf(xh, 0x1.b93910p-26f, pl) + xsh * RSM_TWO_OVER_PI;   /* 2/pi - RSM_TWO_OVER_PI */
    const float q0 = rintf(ph);
    const float fr = (ph - q0) + pl;
    q = fr > 0.5f ? q0 + 1.0f : (fr < -0.5f ? q0 - 1.0f : q0);
    const float r1 = fmaf(-q, RSM_PIO2_1, xh);
    float th, tl;
    two_prod(q, RSM_PIO2_2, th, tl);
    float s, e, s2, e2;
    two_sum(r1, -th, s, e);
    two_sum(s, xsh, s2, e2);
    const float tail = e2 + ((e - tl) + fmaf(-q, RSM_PIO2_3, xsl));
    two_sum(s2, tail, rh, rl);
}

/* sine and cosine of the double-float r = rh + rl (|r| <= pi/4 + 1e-6)
 * plus q pi/2, as double-floats accurate to ~1e-14.  With t = j/64 the
 * nearest node and d = r - t (|d| <= 1/128; rh - t is exact):
 *   sin(t + d) = S + (S m + C sd),  cos(t + d) = C + (C m - S sd),
 *   sd = sin d = d - d^3/6 + d^5/120,  m = cos d - 1 = -d^2/2 + d^4/24,
 * S, C the node's sine and cosine as double-floats (kSinCosNode, exact to
 * 2^-48).  Past their first terms the series are below 8e-8 (sd) and
 * 1.6e-10 (m) and are formed in FP32; d^2 is split exactly.  The terms
 * dropped (d^7/5040, d^6/720) are below 1e-18. */
__device__ __forceinline__ void sincos_df(float rh, float rl, float q, float &sh, float &sl, float &ch, float &cl) {
    const float jf = rintf(rh * kSinCosStep);
    const float dh = fmaf(-jf, 1.0f / kSinCosStep, rh);
    const int j = (int)jf;
    const float4 T = __ldg(&kSinCosNode[min(abs(j), kSinCosNodes - 1)]);
    const float Sh = j < 0 ? -T.x : T.x, Sl = j < 0 ? -T.y : T.y;
    const float Ch = T.z, Cl = T.w;
    /* d^2 = p + pe (exact head product, tail with 2 dh rl) */
    float p, pe;
    two_prod(dh, dh, p, pe);
    pe = fmaf(2.0f * dh, rl, pe);
    const float mh = -0.5f * p;
    const float ml = fmaf(0x1.555556p-5f * p, p, -0.5f * pe);   /* d^4/24 - pe/2 */
    /* sd = dh + (rl + c3), c3 = -dh^3/6 + dh^5/120 - dh^2 rl/2 */
    const float c3 = fmaf(dh * p, fmaf(p, 0x1.111112p-7f, -0x1.555556p-3f), -0.5f * p * rl);
    const float sdl = rl + c3;
    float Ah, Al, Bh, Bl, Dh, Dl, Eh, El;
    df_mul_pair(Sh, Sl, mh, ml, Ah, Al);    /* S m */
    df_mul_pair(Ch, Cl, dh, sdl, Bh, Bl);   /* C sd */
    df_mul_pair(Ch, Cl, mh, ml, Dh, Dl);    /* C m */
    df_mul_pair(Sh, Sl, dh, sdl, Eh, El);   /* S sd */
    float u, ue, v, ve;
    two_sum(Ah, Bh, u, ue);
    two_sum(Sh, u, v, ve);
    float s0h, s0l, c0h, c0l;
    fast_two_sum(v, ve + (ue + Al + Bl + Sl), s0h, s0l);
    two_sum(Dh, -Eh, u, ue);
    two_sum(Ch, u, v, ve);
    fast_two_sum(v, ve + (ue + Dl - El + Cl), c0h, c0l);
    /* quadrant (as rsm_sincos_reduced): (s, c), (c, -s), (-s, -c), (-c, s) */
    const int quad = (int)q & 3;
    const bool swap = (quad & 1) != 0;
    const float a_h = swap ? c0h : s0h, a_l = swap ? c0l : s0l;
    const float b_h = swap ? s0h : c0h, b_l = swap ? s0l : c0l;
    const bool ns = (quad & 2) != 0, nc = ((quad + 1) & 2) != 0;
    sh = ns ? -a_h : a_h;
    sl = ns ? -a_l : a_l;
    ch = nc ? -b_h : b_h;
    cl = nc ? -b_l : b_l;
}

/* Diagnostics of the two-way phase's sine and cosine, against double: the
 * compensated form's (fn 9 sine, 10 cosine: the exact k r of range a[i] and
 * wave number b[i], reduced by reduce_pio2_df, sincos_df's double-float
 * values) and the plain form's
 * (fn 11, 12: rsm_sincosf of the rounded k r).  out[i] = error. */
__global__ void k_eval_phase(int fn, const float *a, const float *b, float *out, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float r = a[i], k = b[i];
    double ref_s, ref_c;
    sincos((double)k * (double)r, &ref_s, &ref_c);
    double ss, cc;
    if (fn == 9 || fn == 10) {
        float phh, phl, q, rh, rl, sh, sl, ch, cl;
        two_prod(k, r, phh, phl);
        reduce_pio2_df(phh, phl, 0.0f, q, rh, rl);
        sincos_df(rh, rl, q, sh, sl, ch, cl);
        ss = (double)sh + (double)sl;
        cc = (double)ch + (double)cl;
    } else {
        float s32, c32;
        rsm_sincosf(k * r, &s32, &c32);
        ss = s32;
        cc = c32;
    }
    out[i] = (fn == 9 || fn == 11) ? (float)(ss - ref_s) : (float)(cc - ref_c);
}

/* The beam angle theta between b = sim[0..2] and p as a double-float, from
 * s = |b x p| / (|b| |p|) (sh + sl) and the FP32 dot product: an FP32 first
 * guess (asin(s) = s + s z P(z) below 30 degrees, atan2 beyond and behind
 * the radar), then -- unless the antenna table clamps there anyway -- one
 * Newton step with the guess's sine and cosine as double-floats
 * (sincos_df): on sin theta = s where |cos theta| >= 0.7 (below 45 and
 * above 135 degrees), where it is well conditioned, and on
 * cos theta = b.p / (|b| |p|) (the dot product split exactly) between.
 * The guess is good to ~1e-7 of theta, so the step leaves ~1e-15 rad, which
 * the steep flanks of the antenna table's sidelobes need: an FP32 angle
 * there moves a small weight by 1e-6 of itself.  Below 5.7 degrees the
 * asin series in double-float does the same for a fraction of the cost. */
__device__ __forceinline__ void beam_angle_df(const PulseArgs &P, float4 p, float sh, float sl, float dot, float cnh,
                                              float dph, float dpl, float &ang_h, float &ang_l) {
    const float *sd = P.sim;
    float th0;
    if (dot > 0.0f && sh < 0.5f) {
        const float z = sh * sh;
        th0 = fmaf(sh * z, rsm_asin_poly(z), sh);
    } else {
        th0 = rsm_atan2f(cnh, dot);
    }
    ang_h = th0;
    ang_l = 0.0f;
    const float fs = fmaf(th0, P.awd[0], P.awd[1]);
    if (!(fs > -1.0f && fs < P.awd[2] + 1.0f)) return;   /* the table clamps: its edge entry */
    if (dot > 0.0f && sh < 0.1f) {
        /* below 5.7 degrees the series converges fast: asin s = s + s^3/6 +
         * s^5 Q(s^2), Q the next Taylor terms (3/40, 15/336, 105/3456,
         * 945/42240; the rest below 1e-9 of Q), with s^3/6 a double-float
         * and s^5 Q below 8e-7 of s in FP32: within 1e-14 rad */
        float zh, zl, ch3, cl3;
        two_prod(sh, sh, zh, zl);
        zl = fmaf(2.0f * sh, sl, zl);
        df_mul_pair(sh, sl, zh, zl, ch3, cl3);                              /* s^3 */
        float th, tl;
        df_mul_pair(ch3, cl3, 0x1.555556p-3f, -0x1.555556p-28f, th, tl);  /* / 6 */
        float q = fmaf(zh, 0x1.6e8ba2p-6f, 0x1.f1c71cp-6f);
        q = fmaf(zh, q, 0x1.6db6dcp-5f);
        q = fmaf(zh, q, 0x1.333334p-4f);
        const float t5 = (ch3 * zh) * q;
        float a, e;
        two_sum(sh, th, a, e);
        fast_two_sum(a, e + (sl + tl + t5), ang_h, ang_l);
        return;
    }
    float q = 0.0f, rh = th0, rl = 0.0f;
    if (th0 > 0.78f) reduce_pio2_df(th0, 0.0f, 0.0f, q, rh, rl);
    float s0h, s0l, c0h, c0l;
    sincos_df(rh, rl, q, s0h, s0l, c0h, c0l);
    float d;
    if (fabsf(c0h) >= 0.7f) {
        d = __fdividef((sh - s0h) + (sl - s0l), c0h);
    } else {
        /* c = b.p / (|b| |p|) as a double-float */
        float a0, e0, a1, e1, a2, e2, th, tl;
        two_prod(sd[0], p.x, a0, e0);
        two_prod(sd[1], p.y, a1, e1);
        two_prod(sd[2], p.z, a2, e2);
        df_add(a0, e0, a1, e1, th, tl);
        df_add(th, tl, a2, e2, th, tl);
        float ch, cl;
        df_div(th, tl, dph, dpl, ch, cl);
        d = -__fdividef((ch - c0h) + (cl - c0l), s0h);
    }
    two_sum(th0, d, ang_h, ang_l);
}

/* compensated signal, every factor a double-float.  Range r = |p| from the
 * exact squares of the FP32 position; the beam angle from
 * |b x p| / (|b| |p|) with the cross product formed exactly, refined to a
 * double-float by beam_angle_df; the antenna weight as
 * the lerp of its table at that angle (weight_comp_df); the phase k r split
 * exactly, reduced by pi/2 as a double-float (reduce_pio2_df) and its sine
 * and cosine as double-floats (sincos_df); 1 / r^2 from the double-float
 * r^2 with one Newton correction; the rotation a cc + b ss with both
 * products split exactly.  The term (rotation x attenuation x antenna
 * weight) leaves as head s and tail s_lo: the FP32 rounding of its factors,
 * some 1e-7 of it each, is carried instead of dropped, so a gate sum of
 * such terms reaches the FP64 pulse of the same state to the double-float's
 * own precision. */
__device__ __forceinline__ void signal_comp(const PulseArgs &P, float4 p, float4 x, Sig32 &o) {
    const float *sd = P.sim;
    /* range */
    const float ph3[3] = {p.x, p.y, p.z};
    float r2h, r2l, rh, rl;
    df_norm2_f(ph3, r2h, r2l);
    df_sqrt(r2h, r2l, rh, rl);
    /* sin of the beam angle */
    const float bx = sd[0], by = sd[1], bz = sd[2];
    float ch[3], cl[3];
    df_prod_diff(by, p.z, bz, p.y, ch[0], cl[0]);
    df_prod_diff(bz, p.x, bx, p.z, ch[1], cl[1]);
    df_prod_diff(bx, p.y, by, p.x, ch[2], cl[2]);
    float c2h, c2l, cnh, cnl;
    df_norm2(ch, cl, c2h, c2l);
    df_sqrt(c2h, c2l, cnh, cnl);
    const float bnh = P.bn_hi, bnl = P.bn_lo;   /* |b|, once per pulse */
    float dph, dpl;                      /* |b| |p| */
    two_prod(bnh, rh, dph, dpl);
    dpl = fmaf(bnh, rl, fmaf(bnl, rh, dpl));
    float sh, sl;
    df_div(cnh, cnl, dph, dpl, sh, sl);
    const float dot = fmaf(bx, p.x, fmaf(by, p.y, bz * p.z));
    float ang_h, ang_l;
    beam_angle_df(P, p, sh, sl, dot, cnh, dph, dpl, ang_h, ang_l);
    float wah, wal;
    weight_comp_df(P.aw, P.awd, ang_h, ang_l, wah, wal);
    o.wang = wah;
    /* phase k r = k rh + k rl, both products split exactly: the head of
     * k rh is reduced by pi/2 and the three small parts (up to 0.25 rad at
     * 30 km) join after the reduction, where a double-float holds them to
     * 1e-15 rad; then its sine and cosine */
    float phh, phl, pa, pb, xsh, xse;
    two_prod(sd[4], rh, phh, phl);
    two_prod(sd[4], rl, pa, pb);
    two_sum(phl, pa, xsh, xse);
    float q, red_h, red_l;
    reduce_pio2_df(phh, xsh, xse + pb, q, red_h, red_l);
    float ssh, ssl, cch, ccl;
    sincos_df(red_h, red_l, q, ssh, ssl, cch, ccl);
    /* attenuation 1 / r^2: y = 1 / r2h corrected by its residual */
    const float y = 1.0f / r2h;
    const float res = fmaf(-r2h, y, 1.0f) - r2l * y;
    float ath, atl;
    fast_two_sum(y, y * res, ath, atl);
    /* k = attenuation x antenna weight */
    float kh, kl;
    df_mul_pair(ath, atl, wah, wal, kh, kl);
    const float xa[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
    for (int l = 0; l < 4; l++) {
        /* (x.x, x.y) -> x.x cc + x.y ss, x.y cc - x.x ss */
        const float a = xa[l], b = (l & 1) ? -xa[l - 1] : xa[l + 1];
        float p1, e1, p2, e2, rot_h, e;
        two_prod(a, cch, p1, e1);
        two_prod(b, ssh, p2, e2);
        two_sum(p1, p2, rot_h, e);
        const float rot_l = e + fmaf(a, ccl, fmaf(b, ssl, e1 + e2));
        o.sig[l] = rot_h * ath;
        df_mul_pair(rot_h, rot_l, kh, kl, o.s.v[l], o.s_lo[l]);
    }
    o.r = rh;
    o.r_lo = rl;
}

template <int MODE>  /* RSC_PULSE_PLAIN, RSC_PULSE_COMPENSATED, RSC_PULSE_F64 */
struct PulseTraits;
template <> struct PulseTraits<0> { typedef AccF32 Acc; static constexpr unsigned kMain = kBinStride32; };
template <> struct PulseTraits<1> { typedef AccDF Acc; static constexpr unsigned kMain = 8; };
template <> struct PulseTraits<2> { typedef AccF64 Acc; static constexpr unsigned kMain = 4; };

/* The block's flags (bit l for lane l) that a non-finite value met the
 * moment form: that lane of every gate of the pulse is then NaN, as
 * 0 x NaN is in pass 1. */
__device__ __forceinline__ int &pulse_poison() {
    __shared__ int flag;
    return flag;
}

/* Largest triangle support, in gate spacings, of the compensated form's
 * interval moments (PulseArgs::mom_n). */
constexpr int kMomMaxN = 4;

/* shared memory per warp of k_pulse<MODE>, in bytes, for G gates (the
 * compensated form: double-float bins of G gates, or of G + 2 kMomMaxN - 1
 * range intervals with two moments each, and FP32 mini bins) */
__host__ __device__ constexpr size_t pulse_warp_bytes(int mode, unsigned G) {
    return mode == 0 ? (size_t)G * kBinStride32 * 4
                     : (mode == 1 ? (size_t)(G + 2 * kMomMaxN - 1) * 64 + (size_t)G * kBinStride32 * 4
                                  : (size_t)G * 32);
}

/* block blk of the nblk blocks that form one pulse */
/* Largest number of gates a warp visits together on the coherent path; a
 * wider spread goes through per-lane atomics. */
/* The warp's candidate gates [w_lo, w_hi] over the lanes that have any; true
 * when the span is at most `span` gates (the coherent path).  The host sets
 * span to G when the state is in spatial order (neighbouring lanes share
 * gates, and per-lane atomics would collide) and to 0 otherwise (random
 * ranges: a warp spans most gates, and per-lane atomics rarely collide). */
__device__ __forceinline__ bool warp_coherent(bool has, int k_lo, int k_hi, int span, int &w_lo, int &w_hi) {
    if (span <= 0) return false;
    const bool any = has && k_hi >= k_lo;
    w_lo = (int)__reduce_min_sync(0xffffffffu, any ? (unsigned)k_lo : 0xffffffffu);
    w_hi = (int)__reduce_max_sync(0xffffffffu, any ? (unsigned)k_hi : 0u);
    if (w_lo == -1) {       /* no lane has a candidate */
        w_hi = -2;
        return true;
    }
    return w_hi - w_lo < span;
}

/* x = fma(w, a, x) and y = fma(w, b, y), each rounded once as fmaf rounds
 * it: one packed FP32 instruction (fma.rn.f32x2) for the two */
__device__ __forceinline__ void fma_pair(float w, float a, float b, float &x, float &y) {
    unsigned long long wp, ab, xy;
    asm("mov.b64 %0, {%1, %1};" : "=l"(wp) : "f"(w));
    asm("mov.b64 %0, {%1, %2};" : "=l"(ab) : "f"(a), "f"(b));
    asm("mov.b64 %0, {%1, %2};" : "=l"(xy) : "f"(x), "f"(y));
    asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(xy) : "l"(wp), "l"(ab));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(xy));
}

/* Add the warp's sum of four values into bin[0..3]: a transposed butterfly
 * (6 shuffles instead of 20) leaves the sum of value c in lanes 8c..8c+7,
 * and lanes 0, 8, 16, 24 add them to the warp's own bins (no other warp
 * writes them, and one lane per address, so no atomic is needed). */
__device__ __forceinline__ void warp_reduce4_add(float *bin, unsigned lane, float v0, float v1, float v2, float v3) {
    const bool h16 = (lane & 16u) != 0;
    float k0 = h16 ? v2 : v0, k1 = h16 ? v3 : v1;
    const float s0 = h16 ? v0 : v2, s1 = h16 ? v1 : v3;
    k0 = k0 + __shfl_xor_sync(0xffffffffu, s0, 16);
    k1 = k1 + __shfl_xor_sync(0xffffffffu, s1, 16);
    const bool h8 = (lane & 8u) != 0;
    float k = h8 ? k1 : k0;
    const float s = h8 ? k0 : k1;
    k = k + __shfl_xor_sync(0xffffffffu, s, 8);
    k = k + __shfl_xor_sync(0xffffffffu, k, 4);
    k = k + __shfl_xor_sync(0xffffffffu, k, 2);
    k = k + __shfl_xor_sync(0xffffffffu, k, 1);
    if ((lane & 7u) == 0u && k != 0.0f) bin[lane >> 3] += k;
}

/* One block's share of a pulse: per-warp bins in shared memory, filled one
 * scatterer per lane (add), then summed over the block into the grid's FP64
 * accumulator, the last block converting (finish).  Used by the pulse kernel
 * (scatterers loaded from memory) and by the fused step kernel (scatterers
 * just advanced, in registers). */
/* The warp's sum of four double-float values (heads v, tails u) added into
 * a double-float bin row (hi[0..3], lo[0..3]): the transposed butterfly of
 * warp_reduce4_add with an error-free addition of the heads at every level,
 * their rounding errors joining the tails, which are summed alongside in
 * FP32 (they are some 1e-7 of the heads: their own rounding is below
 * 1e-14 of the sum).  The compensated form's path for a state in spatial
 * order. */
__device__ __forceinline__ void warp_reduce4_add_df(float *df, unsigned lane, const float *v, const float *u) {
    const bool h16 = (lane & 16u) != 0;
    float k0 = h16 ? v[2] : v[0], k1 = h16 ? v[3] : v[1];
    float t0 = h16 ? u[2] : u[0], t1 = h16 ? u[3] : u[1];
    const float s0 = h16 ? v[0] : v[2], s1 = h16 ? v[1] : v[3];
    const float z0 = h16 ? u[0] : u[2], z1 = h16 ? u[1] : u[3];
    float a, e;
    two_sum(k0, __shfl_xor_sync(0xffffffffu, s0, 16), a, e);
    k0 = a;
    t0 = t0 + (__shfl_xor_sync(0xffffffffu, z0, 16) + e);
    two_sum(k1, __shfl_xor_sync(0xffffffffu, s1, 16), a, e);
    k1 = a;
    t1 = t1 + (__shfl_xor_sync(0xffffffffu, z1, 16) + e);
    const bool h8 = (lane & 8u) != 0;
    float k = h8 ? k1 : k0, t = h8 ? t1 : t0;
    const float s = h8 ? k0 : k1, z = h8 ? t0 : t1;
    two_sum(k, __shfl_xor_sync(0xffffffffu, s, 8), a, e);
    k = a;
    t = t + (__shfl_xor_sync(0xffffffffu, z, 8) + e);
#pragma unroll
    for (int off = 4; off > 0; off >>= 1) {
        two_sum(k, __shfl_xor_sync(0xffffffffu, k, off), a, e);
        k = a;
        t = t + (__shfl_xor_sync(0xffffffffu, t, off) + e);
    }
    if ((lane & 7u) == 0u && (k != 0.0f || t != 0.0f)) {
        const unsigned c = lane >> 3;
        float hi;
        two_sum(df[c], k, hi, e);
        df[c] = hi;
        df[4 + c] = df[4 + c] + (e + t);
    }
}

/* PATH: 0 sparse gates with per-lane atomics (state in the caller's order),
 * 1 sparse gates, summed across the warp where its lanes share a few gates
 * (state in spatial order), per-lane atomics elsewhere, 2 every gate (a range
 * weight with non-zero edges), -1 chosen at run time from the arguments (the
 * batched and fused kernels).  A kernel compiled for one path holds only that
 * path's code. */
template <int MODE, int PATH = -1>
struct PulseBins {
    typedef PulseTraits<MODE> Tr;
    typedef typename Tr::Acc Acc;
    typedef typename Acc::bin_t bin_t;
    static constexpr unsigned kMain = Tr::kMain;   /* bin_t per gate in the main bins */
    bin_t *bins, *wbins;
    float *mini, *fbins;
    unsigned G, words, nwarps, warp, lane;
    int mom;

    __device__ __forceinline__ void init(const PulseArgs &P) {
        extern __shared__ __align__(16) unsigned char smem_raw[];
        G = P.G;
        mom = (MODE == 1) ? P.mom_n : 0;
        /* interval moments: rows of 16 floats (S0 hi, lo, S1 hi, lo) for the
         * intervals -mom .. G + mom - 2 */
        words = mom ? (G + 2 * mom - 1) * 16 : G * kMain;
        if (threadIdx.x == 0) pulse_poison() = 0;
        nwarps = blockDim.x >> 5;
        warp = threadIdx.x >> 5;
        lane = threadIdx.x & 31u;
        bins = reinterpret_cast<bin_t *>(smem_raw);
        float *mini_all = reinterpret_cast<float *>(bins + (size_t)nwarps * words);   /* compensated: FP32 mini bins */
        for (unsigned t = threadIdx.x; t < nwarps * words; t += blockDim.x) bins[t] = (bin_t)0;
        if (MODE == 1) {
            for (unsigned t = threadIdx.x; t < nwarps * G * kBinStride32; t += blockDim.x) mini_all[t] = 0.0f;
        }
        __syncthreads();
        wbins = bins + (size_t)warp * words;
        mini = mini_all + (size_t)warp * G * kBinStride32;
        fbins = (MODE == 1) ? mini : reinterpret_cast<float *>(wbins);   /* where FP32 atomics go */
    }

    /* Scatterer i (position p, backscatter x) of this lane, if `in`.  Every
     * lane of the warp calls it together (warp collectives inside). */
    __device__ __forceinline__ void add(const PulseArgs &P, bool in, unsigned long long i, float4 p, float4 x) {
        bool mini_used = false;   /* FP32 mini bins written this iteration (compensated form) */
        Acc c;
        c.set(0, 0, 0, 0);
        float r = 0.0f, r_lo = 0.0f;
        double r64 = 0.0;
        bool finite = false;
        if (in) {
            if constexpr (MODE == 2) {
                double px = p.x, py = p.y, pz = p.z;
                r64 = sqrt(px * px + py * py + pz * pz);
                double bx = P.sim[0], by = P.sim[1], bz = P.sim[2];
                double cx = by * pz - bz * py, cy = bz * px - bx * pz, cz = bx * py - by * px;
                double ang = atan2(sqrt(cx * cx + cy * cy + cz * cz), bx * px + by * py + bz * pz);
                double wa = lerp64(P.aw, P.awd, ang);
                double atten = 1.0 / (r64 * r64);
                double ss, cc;
                sincos((double)P.sim[4] * r64, &ss, &cc);
                double k = atten * wa;
                c.v[0] = ((double)x.x * cc + (double)x.y * ss) * k;
                c.v[1] = ((double)x.y * cc - (double)x.x * ss) * k;
                c.v[2] = ((double)x.z * cc + (double)x.w * ss) * k;
                c.v[3] = ((double)x.w * cc - (double)x.z * ss) * k;
                r = (float)r64;
                finite = isfinite(r64) && isfinite(c.v[0]) && isfinite(c.v[1]) && isfinite(c.v[2]) &&
                         isfinite(c.v[3]);
            } else {
                Sig32 sg;
                if constexpr (MODE == 0) {
                    signal_plain(P, p, x, sg);
                } else {
                    signal_comp(P, p, x, sg);
                }
                c.set(sg.s.v[0], sg.s.v[1], sg.s.v[2], sg.s.v[3]);
                if constexpr (MODE == 1) c.set_lo(sg.s_lo);
                r = sg.r;
                r_lo = sg.r_lo;
                finite = fabsf(r) < INFINITY && finite4(sg.s.v);
                if (MODE == 0 && P.materialize) {
                    float4 ax = P.aux[i];
                    ax.x = r;
                    ax.y = ax.y + P.sim[15];
                    ax.w = sg.wang;
                    P.aux[i] = ax;
                    P.sig[i] = make_float4(sg.sig[0], sg.sig[1], sg.sig[2], sg.sig[3]);
                }
            }
        }
        if (PATH == 2 ? false : (PATH >= 0 ? true : !P.dense)) {
            /* candidate gates: only those the range weight can reach */
            int k_lo = 0, k_hi = -1;
            if (in && finite) {
                float g = (r - P.rs) * P.inv_delta;
                k_lo = max(0, (int)ceilf(fminf(fmaxf(g - P.win_hi, -1.0f), (float)G)));
                k_hi = min((int)G - 1, (int)floorf(fminf(g - P.win_lo, (float)G)));
            }
            const int maxc = min(kMaxCandidates, (int)__reduce_max_sync(0xffffffffu, (unsigned)max(k_hi - k_lo + 1, 0)));
            int w_lo = 0, w_hi = -1;
            bool coherent = false;
            if constexpr (MODE == 2) {
                for (int j = 0; j < maxc; j++) {
                    const int gate = k_lo + j;
                    Acc cw;
                    bool nz = false;
                    if (gate <= k_hi) {
                        double w = lerp64(P.rw, P.rwd, r64 - P.rk64[gate]);
                        c.scale(w, cw);
                        nz = (w != 0.0);
                    }
                    bin_add<Acc>(wbins, 0xffffffffu, nz, gate, cw);
                }
            } else if (PATH != 0 && (coherent = warp_coherent(in && finite, k_lo, k_hi, P.coherent_span, w_lo, w_hi))) {
                /* the warp's candidates fall in a few gates (a state kept in
                 * spatial order): visit them together and reduce each gate
                 * across the warp, no atomics.  The gate origin is advanced
                 * from w_lo by the reference's running-sum additions, so every
                 * lane's origin is the same bit pattern as in the branch below */
                float rkj = 0.0f;
                if (MODE == 0) rkj = __ldg(P.rk + w_lo);
                for (int gate = w_lo; gate <= w_hi; gate++) {
                    float w = 0.0f;
                    if constexpr (MODE == 1) {
                        float wl = 0.0f;
                        if (gate >= k_lo && gate <= k_hi) {
                            range_weight_comp_df(P.rw, P.rwd, P.rw_tri, r - __ldg(P.rk + gate),
                                                 r_lo - __ldg(P.rk_lo + gate), w, wl);
                        }
                        Acc cw;
                        c.scale_df(w, wl, cw);
                        warp_reduce4_add_df(reinterpret_cast<float *>(wbins) + (size_t)gate * 8, lane, cw.v, cw.u);
                    } else {
                        if (gate >= k_lo && gate <= k_hi) w = range_weight_reg(P, r - rkj);
                        warp_reduce4_add(fbins + (size_t)gate * kBinStride32, lane, w * c.v[0], w * c.v[1],
                                         w * c.v[2], w * c.v[3]);
                    }
                    rkj = rkj + P.rdelta;
                }
            } else {
                /* plain: one gate origin is loaded and advanced by the same
                 * FP32 additions the reference's running sum makes
                 * (rs.cl:1214), so every candidate's origin is bit-identical */
                float rkj = 0.0f;
                if (MODE == 0 && k_hi >= k_lo) rkj = __ldg(P.rk + k_lo);
                for (int j = 0; j < maxc; j++) {
                    const int gate = k_lo + j;
                    if (gate <= k_hi) {
                        float w;
                        if constexpr (MODE == 1) {
                            w = range_weight_comp(P.rw, P.rwd, P.rw_tri, r - __ldg(P.rk + gate),
                                                  r_lo - __ldg(P.rk_lo + gate));
                        } else {
                            w = range_weight_reg(P, r - rkj);
                        }
                        if (w != 0.0f) {
                            float *b = fbins + (size_t)gate * kBinStride32;
                            float t[4] = {w * c.v[0], w * c.v[1], w * c.v[2], w * c.v[3]};
                            if constexpr (MODE == 1) {
                                /* unordered state: each term rounded once into
                                 * the FP32 mini bins (its tail included first) */
#pragma unroll
                                for (int l = 0; l < 4; l++) t[l] = fmaf(w, c.v[l], w * c.u[l]);
                            }
                            atomicAdd(b + 0, t[0]);
                            atomicAdd(b + 1, t[1]);
                            atomicAdd(b + 2, t[2]);
                            atomicAdd(b + 3, t[3]);
                        }
                    }
                    rkj = rkj + P.rdelta;
                }
            }
            /* a non-finite signal meets every gate (0 * inf = NaN in pass 1) */
            mini_used = !coherent;
            if (__any_sync(0xffffffffu, in && !finite)) {
                mini_used = true;
                for (unsigned k = 0; k < G; k++) {
                    bool valid = in && !finite;
                    Acc cw;
                    cw.set(0, 0, 0, 0);
                    if (valid) {
                        if constexpr (MODE == 2) {
                            c.scale(lerp64(P.rw, P.rwd, r64 - P.rk64[k]), cw);
                        } else {
                            c.scale(range_weight(P, r - __ldg(P.rk + k)), cw);
                        }
                    }
                    if constexpr (MODE == 2) {
                        bin_add<Acc>(wbins, 0xffffffffu, valid, (int)k, cw);
                    } else if (valid) {
                        float *b = fbins + (size_t)k * kBinStride32;
                        atomicAdd(b + 0, cw.v[0]);
                        atomicAdd(b + 1, cw.v[1]);
                        atomicAdd(b + 2, cw.v[2]);
                        atomicAdd(b + 3, cw.v[3]);
                    }
                }
            }
        } else {
            /* dense: every gate, as pass 1 does; the warp sums each gate with a
             * fixed shuffle tree and lane 0 adds it to the warp's bin */
            for (unsigned k = 0; k < G; k++) {
                Acc cw;
                cw.set(0, 0, 0, 0);
                if (in) {
                    if constexpr (MODE == 2) {
                        c.scale(lerp64(P.rw, P.rwd, r64 - P.rk64[k]), cw);
                    } else if constexpr (MODE == 1) {
                        float wh, wl;
                        weight_comp_df(P.rw, P.rwd, r - __ldg(P.rk + k), r_lo - __ldg(P.rk_lo + k), wh, wl);
                        c.scale_df(wh, wl, cw);
                    } else {
                        c.scale(range_weight(P, r - __ldg(P.rk + k)), cw);
                    }
                }
                warp_sum_into<Acc>(wbins + (size_t)k * kMain, cw);
            }
        }
        if (MODE == 1 && mini_used) {
            /* fold the FP32 mini bins into the warp's double-float bins */
            __syncwarp();
            float *df = reinterpret_cast<float *>(wbins);
            for (unsigned o = lane; o < G * 4; o += 32) {
                const unsigned k = o >> 2, l = o & 3u;
                const float v = mini[k * kBinStride32 + l];
                if (v != 0.0f) {
                    float s, e;
                    two_sum(df[k * 8 + l], v, s, e);
                    df[k * 8 + l] = s;
                    df[k * 8 + 4 + l] = df[k * 8 + 4 + l] + e;
                    mini[k * kBinStride32 + l] = 0.0f;
                }
            }
            __syncwarp();
        }
    }

    /* The compensated form's terms on the triangle whose support is mom
     * gate spacings: within the range interval [rho_j, rho_j+1) between two
     * gate origins every gate's weight is linear in r, 1 - |j - k| delta s
     * -+ s u with u = r - rho_j (the sign by the side of gate k, s the
     * table's scale), so a scatterer adds its term x to S0_j and u x to S1_j
     * of its one interval, and finish forms each gate from the 2 mom
     * intervals of its support.  A warp of sorted neighbours meets one or
     * two intervals instead of the 4-5 gates their triangles reach, each
     * with two error-free reductions.  rho_j = r_0 + j delta as a
     * double-float; j from FP32, which can put a scatterer within 1e-4 m of
     * an origin on the other side of it (its weight then off by 1e-5 of
     * itself, for 1 in 1e5 scatterers). */
    template <int K>
    __device__ __forceinline__ void add_moments(const PulseArgs &P, const bool *in, const float *rr, const float *rl,
                                                const float (*c)[4], const float (*cu)[4]) {
        const int n = mom;
        const float r0h = __ldg(P.rk), r0l = __ldg(P.rk_lo);
        int bq[K];
        float uh[K], ul[K];
        unsigned lo = 0xffffffffu, hi = 0u;
#pragma unroll
        for (int q = 0; q < K; q++) {
            bq[q] = -1;
            uh[q] = 0.0f;
            ul[q] = 0.0f;
            if (in[q]) {
                const float jf = floorf((rr[q] - r0h) * P.inv_delta);
                if (jf >= (float)(-n - 1) && jf <= (float)((int)G + n - 1)) {
                    int j = (int)jf;
                    float ph, pl, rho_h, rho_l;
                    two_prod((float)j, P.rdelta, ph, pl);
                    df_add(r0h, r0l, ph, pl, rho_h, rho_l);
                    float u0 = rr[q] - rho_h, u1 = rl[q] - rho_l;
                    /* j from the head in FP32 can be one off within 1e-3 m of
                     * an origin (the range's tail is up to that): the
                     * double-float offset puts the scatterer on its side */
                    const float ut = u0 + u1;
                    if (ut < 0.0f || ut >= P.rdelta) {
                        const float sh = ut < 0.0f ? P.rdelta : -P.rdelta;
                        float a, e;
                        two_sum(u0, sh, a, e);
                        u0 = a;
                        u1 = u1 + e;
                        j += ut < 0.0f ? -1 : 1;
                    }
                    if (j >= -n && j <= (int)G + n - 2) {
                        uh[q] = u0;
                        ul[q] = u1;
                        bq[q] = j + n;
                        lo = min(lo, (unsigned)bq[q]);
                        hi = max(hi, (unsigned)bq[q]);
                    }
                }
            }
        }
        const unsigned b_lo = __reduce_min_sync(0xffffffffu, lo);
        const unsigned b_hi = __reduce_max_sync(0xffffffffu, hi);
        if (b_lo == 0xffffffffu) return;   /* no lane's scatterer reaches a gate */
        float *rows = reinterpret_cast<float *>(wbins);
        for (unsigned b = b_lo; b <= b_hi; b++) {
            /* S0 then S1 (fewer live registers than both at once) */
#pragma unroll
            for (int m = 0; m < 2; m++) {
                float sh[4] = {0.0f, 0.0f, 0.0f, 0.0f}, sl[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
                for (int q = 0; q < K; q++) {
                    if (bq[q] == (int)b) {
#pragma unroll
                        for (int l = 0; l < 4; l++) {
                            float th = c[q][l], tl = cu[q][l], a, e;
                            if (m == 1) df_mul_pair(c[q][l], cu[q][l], uh[q], ul[q], th, tl);
                            two_sum(sh[l], th, a, e);
                            sh[l] = a;
                            sl[l] = sl[l] + (tl + e);
                        }
                    }
                }
                warp_reduce4_add_df(rows + (size_t)b * 16 + 8 * m, lane, sh, sl);
            }
        }
    }

    /* K scatterers per lane (plain or compensated form, state in spatial
     * order): lane l
     * holds scatterers l, l + 32, ... of a run of 32 K neighbours, the warp
     * visits the gates of all of them together and each lane adds its K
     * weighted signals before the one warp reduction per gate (1 / K of the
     * reductions of K add calls).  The weights are those of add, bit for bit
     * (the same running-sum gate origin from the warp's first gate).  A warp
     * with a non-finite signal takes its scatterers one at a time through
     * add. */
    template <int K, int TRI = -1>   /* TRI 1: the range table is the triangle (known at compile time) */
    __device__ __forceinline__ void add_k(const PulseArgs &P, const bool *in, const unsigned long long *idx,
                                          const float4 *pp, const float4 *xx) {
        static_assert(MODE == 0 || MODE == 1, "the grouped form is the plain or compensated one");
        float c[K][4], cu[K][4], rr[K], rl[K];
        int klo[K], khi[K];
        bool bad = false;
        unsigned lo = 0xffffffffu, hi = 0u;
#pragma unroll
        for (int q = 0; q < K; q++) {
            Sig32 sg;
            sg.r = 0.0f;
            sg.r_lo = 0.0f;
            sg.s.set(0.0f, 0.0f, 0.0f, 0.0f);
            klo[q] = 0;
            khi[q] = -1;
            if (in[q]) {
                if constexpr (MODE == 0) {
                    signal_plain(P, pp[q], xx[q], sg);
                } else {
                    signal_comp(P, pp[q], xx[q], sg);
                }
                const bool fin = fabsf(sg.r) < INFINITY && finite4(sg.s.v);
                bad = bad || !fin;
                const float g = (sg.r - P.rs) * P.inv_delta;
                klo[q] = max(0, (int)ceilf(fminf(fmaxf(g - P.win_hi, -1.0f), (float)G)));
                khi[q] = min((int)G - 1, (int)floorf(fminf(g - P.win_lo, (float)G)));
                if (khi[q] >= klo[q]) {
                    lo = min(lo, (unsigned)klo[q]);
                    hi = max(hi, (unsigned)khi[q]);
                }
            }
            rr[q] = sg.r;
            rl[q] = sg.r_lo;
            c[q][0] = sg.s.v[0];
            c[q][1] = sg.s.v[1];
            c[q][2] = sg.s.v[2];
            c[q][3] = sg.s.v[3];
            if constexpr (MODE == 1) {
                if (!in[q]) sg.s_lo[0] = sg.s_lo[1] = sg.s_lo[2] = sg.s_lo[3] = 0.0f;
#pragma unroll
                for (int l = 0; l < 4; l++) cu[q][l] = sg.s_lo[l];
            }
        }
        if constexpr (MODE == 1) {
            if (mom) {
                /* a non-finite value reaches its lane of every gate (0 x NaN
                 * in pass 1): its lane is flagged NaN for the pulse and the
                 * finite lanes are summed; a non-finite range flags all four */
                bool use[K];
#pragma unroll
                for (int q = 0; q < K; q++) use[q] = in[q];
                if (__any_sync(0xffffffffu, bad)) {
#pragma unroll
                    for (int q = 0; q < K; q++) {
                        if (!in[q]) continue;
                        unsigned bits = 0u;
                        if (!(fabsf(rr[q]) < INFINITY)) {
                            bits = 15u;
                            use[q] = false;
                        } else {
#pragma unroll
                            for (int l = 0; l < 4; l++) {
                                if (!(fabsf(c[q][l]) < INFINITY) || !(fabsf(cu[q][l]) < INFINITY)) {
                                    bits |= 1u << l;
                                    c[q][l] = 0.0f;
                                    cu[q][l] = 0.0f;
                                }
                            }
                        }
                        if (bits) atomicOr(&pulse_poison(), (int)bits);
                    }
                }
                add_moments<K>(P, use, rr, rl, c, cu);
                return;
            }
        }
        if (__any_sync(0xffffffffu, bad)) {
#pragma unroll
            for (int q = 0; q < K; q++) add(P, in[q], idx[q], pp[q], xx[q]);
            return;
        }
        const int w_lo = (int)__reduce_min_sync(0xffffffffu, lo);
        const int w_hi = (int)__reduce_max_sync(0xffffffffu, hi);
        if (w_lo == -1) return;   /* no lane reaches a gate */
        float rkj = MODE == 0 ? __ldg(P.rk + w_lo) : 0.0f;
        for (int gate = w_lo; gate <= w_hi; gate++) {
            float rk_hi = 0.0f, rk_lo = 0.0f;
            if constexpr (MODE == 1) {
                rk_hi = __ldg(P.rk + gate);
                rk_lo = __ldg(P.rk_lo + gate);
            }
            if constexpr (MODE == 1) {
                /* the lane's K weighted terms of the gate as double-floats,
                 * added error-free (heads) before the warp's reduction */
                float vh[4] = {0.0f, 0.0f, 0.0f, 0.0f}, vl[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
                for (int q = 0; q < K; q++) {
                    float w = 0.0f, wl = 0.0f;
                    if (gate >= klo[q] && gate <= khi[q]) {
                        range_weight_comp_df(P.rw, P.rwd, TRI == 1 ? 1 : P.rw_tri, rr[q] - rk_hi, rl[q] - rk_lo, w,
                                             wl);
                    }
#pragma unroll
                    for (int l = 0; l < 4; l++) {
                        float th, tl;
                        df_mul_pair(c[q][l], cu[q][l], w, wl, th, tl);
                        if (q == 0) {
                            vh[l] = th;
                            vl[l] = tl;
                        } else {
                            float a, e;
                            two_sum(vh[l], th, a, e);
                            vh[l] = a;
                            vl[l] = vl[l] + (tl + e);
                        }
                    }
                }
                warp_reduce4_add_df(reinterpret_cast<float *>(wbins) + (size_t)gate * 8, lane, vh, vl);
            } else {
                float v0 = 0.0f, v1 = 0.0f, v2 = 0.0f, v3 = 0.0f;
#pragma unroll
                for (int q = 0; q < K; q++) {
                    float w = 0.0f;
                    if constexpr (TRI == 1) {
                        /* every gate of the warp's window: outside the
                         * lane's own candidate gates the triangle gives 0,
                         * and 0 x c adds nothing to the sums, so the
                         * per-gate test is left out */
                        w = range_weight_tri(P.rwd, rr[q] - rkj);
                    } else if (gate >= klo[q] && gate <= khi[q]) {
                        w = range_weight_reg(P, rr[q] - rkj);
                    }
                    /* fused: the lane's K terms of a gate in one rounding each */
                    fma_pair(w, c[q][0], c[q][1], v0, v1);
                    fma_pair(w, c[q][2], c[q][3], v2, v3);
                }
                warp_reduce4_add(fbins + (size_t)gate * kBinStride32, lane, v0, v1, v2, v3);
            }
            rkj = rkj + P.rdelta;
        }
    }

    /* The moment form's block sums: each interval's moments summed over
     * the warps (into warp 0's rows), then gate k of lane l from the
     * intervals j = k - mom .. k + mom - 1 of its support,
     * sum (1 - |j - k| delta s) S0_j -+ s S1_j, as a double-float. */
    __device__ __forceinline__ double moment_gate(const PulseArgs &P, unsigned k, unsigned l) const {
        const float *all = reinterpret_cast<const float *>(bins);
        const float sf = P.rwd[0];
        float dsh, dsl;
        two_prod(P.rdelta, sf, dsh, dsl);
        float gh = 0.0f, gl = 0.0f;
        for (int j = (int)k - mom; j <= (int)k + mom - 1; j++) {
            const float *row = all + (size_t)(j + mom) * 16;
            const int m = j >= (int)k ? j - (int)k : (int)k - j;
            float mh, ml, ah, ae, t0h, t0l, t1h, t1l, x, e;
            two_prod((float)m, dsh, mh, ml);
            ml = fmaf((float)m, dsl, ml);
            two_sum(1.0f, -mh, ah, ae);
            df_mul_pair(ah, ae - ml, row[l], row[4 + l], t0h, t0l);
            const float sg = j >= (int)k ? -sf : sf;
            two_prod(sg, row[8 + l], t1h, t1l);
            t1l = fmaf(sg, row[12 + l], t1l);
            two_sum(gh, t0h, x, e);
            gh = x;
            gl = gl + (t0l + e);
            two_sum(gh, t1h, x, e);
            gh = x;
            gl = gl + (t1l + e);
        }
        return (double)gh + (double)gl;
    }

    __device__ __forceinline__ void finish(const PulseArgs &P, unsigned nblk) {
        __syncthreads();
        if (MODE == 1 && mom) {
            float *all = reinterpret_cast<float *>(bins);
            const unsigned rows = (G + 2 * mom - 1) * 8;
            for (unsigned o = threadIdx.x; o < rows; o += blockDim.x) {
                const unsigned off = (o >> 3) * 16 + ((o >> 2) & 1u) * 8, l = o & 3u;
                float hi = 0.0f, lo = 0.0f;
                for (unsigned wv = 0; wv < nwarps; wv++) {
                    const float *b = all + (size_t)wv * words + off;
                    float x, e;
                    two_sum(hi, b[l], x, e);
                    hi = x;
                    lo = lo + (e + b[4 + l]);
                }
                all[off + l] = hi;
                all[off + 4 + l] = lo;
            }
            __syncthreads();
        }
        /* block sum of each output (warp bins in warp order), added into the
         * grid's FP64 accumulator with one global atomic per output: no block
         * waits on another, and FP64 carries the FP32 and double-float block sums
         * exactly enough that the order of the atomics does not show */
        const unsigned outs = G * 4;
        for (unsigned o = threadIdx.x; o < outs; o += blockDim.x) {
            const unsigned k = o >> 2, l = o & 3u;
            double v;
            if (MODE == 1 && mom) {
                v = ((pulse_poison() >> l) & 1) ? (double)NAN : moment_gate(P, k, l);
            } else if constexpr (Acc::kWords == 2) {
                float hi = 0.0f, lo = 0.0f;
                for (unsigned wv = 0; wv < nwarps; wv++) {
                    const float *b = reinterpret_cast<const float *>(bins) + (size_t)wv * words + k * 8;
                    float s, e;
                    two_sum(hi, b[l], s, e);
                    hi = s;
                    lo = lo + (e + b[4 + l]);
                }
                v = (double)hi + (double)lo;
            } else {
                bin_t acc = (bin_t)0;
                for (unsigned wv = 0; wv < nwarps; wv++) acc = acc + bins[(size_t)wv * words + k * kMain + l];
                v = (double)acc;
            }
            if (v != 0.0) atomicAdd(P.acc64 + o, v);
        }
        __threadfence();
        __syncthreads();
        __shared__ bool s_last;
        if (threadIdx.x == 0) {
            unsigned ticket = atomicAdd(P.counter, 1u);
            s_last = (ticket == nblk - 1);
        }
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        /* last block: every other block's atomics are visible (each fenced
         * before taking its ticket); convert, and leave the accumulator and the
         * counter at zero for the next launch */
        for (unsigned o = threadIdx.x; o < outs; o += blockDim.x) {
            const double v = __ldcg(P.acc64 + o);
            reinterpret_cast<float *>(P.pulse)[o] = (float)v;
            if (MODE == 2) P.pulse64[o] = v;
            P.acc64[o] = 0.0;
        }
        if (threadIdx.x == 0) {
            *P.counter = 0u;
            if (P.runs != nullptr) *P.runs = 0ull;
        }
    }
};

template <int MODE, int PATH = -1>
__device__ __forceinline__ void pulse_body(const PulseArgs &P, unsigned blk, unsigned nblk) {
    PulseBins<MODE, PATH> B;
    B.init(P);
    const unsigned long long stride = (unsigned long long)nblk * blockDim.x;
    const unsigned long long n = P.n;
    /* every lane of a warp runs the same number of iterations so the warp
     * collectives see the full warp */
    const unsigned long long base0 = (unsigned long long)blk * blockDim.x + (threadIdx.x & ~31u);
    for (unsigned long long base = base0; base < n; base += stride) {
        const unsigned long long i = base + B.lane;
        const bool in = i < n;
        float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f), x = p;
        if (in) {
            p = __ldg(P.pos + i);
            x = __ldg(P.rcs + i);
        }
        B.add(P, in, i, p, x);
    }
    B.finish(P, nblk);
}

template <int MODE, int PATH>
__global__ void __launch_bounds__(512) k_pulse(const PulseArgs P) {
    pulse_body<MODE, PATH>(P, blockIdx.x, gridDim.x);
}

/* Block blk of the nblk blocks forming one pulse, over a state in spatial
 * order, K scatterers per lane (PulseBins::add_k): warp w of a block takes
 * runs of 32 K neighbours. */
template <int MODE, int K, int TRI = -1>
__device__ __forceinline__ void pulse_group_run(const PulseArgs &P, PulseBins<MODE, 1> &B, unsigned long long base) {
    const unsigned long long n = P.n;
    bool in[K];
    unsigned long long idx[K];
    float4 pp[K], xx[K];
#pragma unroll
    for (int q = 0; q < K; q++) {
        idx[q] = base + 32u * q + B.lane;
        in[q] = idx[q] < n;
        pp[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        xx[q] = pp[q];
        if (in[q]) {
            pp[q] = __ldg(P.pos + idx[q]);
            xx[q] = __ldg(P.rcs + idx[q]);
        }
    }
    B.template add_k<K, TRI>(P, in, idx, pp, xx);
}

/* Warps take runs of 32 K neighbours: in fixed strides, or -- the
 * compensated form, whose sums are exact in any order -- the next run from
 * a counter as each finishes its last, so that the block's warps reach its
 * final sums together instead of some idling at the barrier while others do
 * one more run (the counter is left at zero by the last block). */
template <int MODE, int K, int TRI = -1>
__device__ __forceinline__ void pulse_body_group(const PulseArgs &P, unsigned blk, unsigned nblk) {
    PulseBins<MODE, 1> B;
    B.init(P);
    const unsigned long long n = P.n;
    if (MODE == 1 && P.runs != nullptr) {
        const unsigned long long runs_n = (n + 32ull * K - 1) / (32ull * K);
        for (;;) {
            unsigned long long r = 0;
            if (B.lane == 0) r = atomicAdd(P.runs, 1ull);
            r = __shfl_sync(0xffffffffu, r, 0);
            if (r >= runs_n) break;
            pulse_group_run<MODE, K, TRI>(P, B, r * 32ull * K);
        }
    } else {
        const unsigned long long stride = (unsigned long long)K * nblk * blockDim.x;
        const unsigned long long base0 =
            (unsigned long long)K * ((unsigned long long)blk * blockDim.x + (threadIdx.x & ~31u));
        for (unsigned long long base = base0; base < n; base += stride) pulse_group_run<MODE, K, TRI>(P, B, base);
    }
    B.finish(P, nblk);
}
template <int MODE, int K, int TRI = -1>
__global__ void __launch_bounds__(512) k_pulse_group(const PulseArgs P) {
    pulse_body_group<MODE, K, TRI>(P, blockIdx.x, gridDim.x);
}

}  // namespace rsc

#endif
