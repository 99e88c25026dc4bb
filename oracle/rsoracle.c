/*
 * rsoracle.c -- CPU oracle: plain-C restatement of the SimRadar OpenCL kernels.
 *
 * TEST INFRASTRUCTURE ONLY (see rsoracle.h).  Compile with -ffp-contract=off.
 * Line references are to rs.cl and rs.c of the reference.
 */
#include "rsoracle.h"
#include "../simradar_gb300/csrc/rsmath.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MIN_HEIGHT 2.0f                             /* rs.cl:1 */
#define M_PI_F 3.14159274f
#define M_PI_2_F 1.57079637f
#define M_SQRT1_2_F 0.707106769f
#define RADIANS_PER_DEGREE 0.0174532924f            /* float(pi / 180) */

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---- OpenCL built-ins on single-precision scalars (OpenCL 1.2 sec. 6.12) ---- */

static inline float cl_clamp(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
static inline float cl_fract(float x, float *ip) {
    float fl = floorf(x);
    *ip = fl;
    return fminf(x - fl, 0x1.fffffep-1f);
}
static inline float cl_mix(float a, float b, float t) { return a + (b - a) * t; }
static inline float cl_sign(float x) {
    if (x > 0.0f) return 1.0f;
    if (x < 0.0f) return -1.0f;
    if (x == 0.0f) return x;
    return 0.0f;
}
static inline uint32_t cl_f2u_rtz(float f) {
    /* convert_uint: round toward zero; out-of-range values saturate to the
     * nearest representable value (the kernels only convert clamped indices). */
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)f;
}
static inline float len3(float x, float y, float z) { return sqrtf(x * x + y * y + z * z); }
static inline float len4(of4 v) { return sqrtf(v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w); }
static inline of4 normalize4(of4 v) {
    float l = len4(v);
    of4 r = {v.x / l, v.y / l, v.z / l, v.w / l};
    return r;
}
static inline of4 f4(float x, float y, float z, float w) { of4 r = {x, y, z, w}; return r; }

/* ---- rand (rs.cl:35-44) ---- */
static inline of4 cl_rand(ou4 *seed) {
    const float n = 1.0f / 2147483647.0f;
    seed->x = (seed->x * 16807u) & 0x7FFFFFFFu;
    seed->y = (seed->y * 16807u) & 0x7FFFFFFFu;
    seed->z = (seed->z * 16807u) & 0x7FFFFFFFu;
    seed->w = (seed->w * 16807u) & 0x7FFFFFFFu;
    return f4((float)seed->x * n, (float)seed->y * n, (float)seed->z * n, (float)seed->w * n);
}

/* ---- quaternions (rs.cl:53-85) ---- */
static inline of4 quat_mult(of4 l, of4 r) {
    return f4(l.w * r.x - l.z * r.y + l.y * r.z + l.x * r.w,
              l.w * r.y + l.z * r.x + l.y * r.w - l.x * r.z,
              l.w * r.z + l.z * r.w - l.y * r.x + l.x * r.y,
              l.w * r.w - l.z * r.z - l.y * r.y - l.x * r.x);
}
static inline of4 quat_conj(of4 q) { return f4(-q.x, -q.y, -q.z, q.w); }
static inline of4 quat_rotate(of4 v, of4 q) { return quat_mult(quat_mult(q, v), quat_conj(q)); }

/* ---- read_imagef, unnormalized / clamp-to-edge / linear (rs.cl:8) ---- */
static inline void tex_axis(float u, int n, int *i0, int *i1, float *a) {
    float uu = u - 0.5f;
    float fl = floorf(uu);
    *a = uu - fl;
    float flc = fminf(fmaxf(fl, -1.0f), (float)n);
    int i = (int)flc;
    *i0 = i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
    *i1 = i + 1 < 0 ? 0 : (i + 1 > n - 1 ? n - 1 : i + 1);
}

static of4 read_image3d(or_image im, float u, float v, float w) {
    int i0, i1, j0, j1, k0, k1;
    float a, b, c;
    tex_axis(u, im.nx, &i0, &i1, &a);
    tex_axis(v, im.ny, &j0, &j1, &b);
    tex_axis(w, im.nz, &k0, &k1, &c);
    const size_t sx = 1, sy = (size_t)im.nx, sz = (size_t)im.nx * (size_t)im.ny;
    const of4 *d = im.data;
    of4 t000 = d[i0 * sx + j0 * sy + k0 * sz], t100 = d[i1 * sx + j0 * sy + k0 * sz];
    of4 t010 = d[i0 * sx + j1 * sy + k0 * sz], t110 = d[i1 * sx + j1 * sy + k0 * sz];
    of4 t001 = d[i0 * sx + j0 * sy + k1 * sz], t101 = d[i1 * sx + j0 * sy + k1 * sz];
    of4 t011 = d[i0 * sx + j1 * sy + k1 * sz], t111 = d[i1 * sx + j1 * sy + k1 * sz];
    float ma = 1.0f - a, mb = 1.0f - b, mc = 1.0f - c;
    float w000 = ma * mb * mc, w100 = a * mb * mc, w010 = ma * b * mc, w110 = a * b * mc;
    float w001 = ma * mb * c, w101 = a * mb * c, w011 = ma * b * c, w111 = a * b * c;
#define TRI(L) (w000 * t000.L + w100 * t100.L + w010 * t010.L + w110 * t110.L + \
                w001 * t001.L + w101 * t101.L + w011 * t011.L + w111 * t111.L)
    of4 r = f4(TRI(x), TRI(y), TRI(z), TRI(w));
#undef TRI
    return r;
}

static of4 read_image2d(or_image im, float u, float v) {
    int i0, i1, j0, j1;
    float a, b;
    tex_axis(u, im.nx, &i0, &i1, &a);
    tex_axis(v, im.ny, &j0, &j1, &b);
    const size_t sy = (size_t)im.nx;
    const of4 *d = im.data;
    of4 t00 = d[i0 + j0 * sy], t10 = d[i1 + j0 * sy], t01 = d[i0 + j1 * sy], t11 = d[i1 + j1 * sy];
    float ma = 1.0f - a, mb = 1.0f - b;
    float w00 = ma * mb, w10 = a * mb, w01 = ma * b, w11 = a * b;
#define BIL(L) (w00 * t00.L + w10 * t10.L + w01 * t01.L + w11 * t11.L)
    of4 r = f4(BIL(x), BIL(y), BIL(z), BIL(w));
#undef BIL
    return r;
}

/* ---- wind_table_index (rs.cl:123-188); only the x, y, z lanes address a
 * 3-D image, so the w lane is not formed ---- */
static inline void wind_table_index(float out[3], of4 pos, const float *wd, const float *sd) {
    uint32_t spacing = rsm_f2u(wd[7]);
    if (spacing == 7u) {
        float pr[3];
        pr[0] = pos.x - (sd[8] + 0.5f * sd[12]);
        pr[1] = pos.y - (sd[9] + 0.5f * sd[13]);
        pr[2] = pos.z - 0.0f;
        for (int l = 0; l < 3; l++) {
            out[l] = copysignf(wd[l], pr[l]) * rsm_log1pf(wd[4 + l] * fabsf(pr[l])) + wd[8 + l];
        }
    } else if (spacing == 0u) {
        out[0] = fmaf(pos.x, wd[0], wd[4]);
        out[1] = fmaf(pos.y, wd[1], wd[5]);
        out[2] = fmaf(pos.z, wd[2], wd[6]);
    } else {
        out[0] = out[1] = out[2] = 0.0f;
    }
}

static inline of4 compute_bg_vel(of4 pos, or_image uvwt, const float *wd, const float *sd) {
    float c[3];
    wind_table_index(c, pos, wd, sd);
    return read_image3d(uvwt, c[0], c[1], c[2]);
}

/* ---- compute_dudt_dwdt (rs.cl:195-261) ---- */
static of4 compute_dudt_dwdt(of4 *dwdt, of4 vel, of4 vel_bg, of4 ori, or_image cdimg, or_image cmimg,
                             const float *ad) {
    of4 ur = f4(vel_bg.x - vel.x, vel_bg.y - vel.y, vel_bg.z - vel.z, vel_bg.w - vel.w);
    of4 u_hat = quat_rotate(normalize4(ur), quat_conj(ori));
    float beta = rsm_acosf(u_hat.x);
    float alpha = rsm_atan2f(u_hat.z, u_hat.y);
    if (alpha < 0.0f) {
        alpha = M_PI_F + alpha;
        beta = -beta;
    }
    float cu = fmaf(beta, ad[0], ad[4]);
    float cv = fmaf(alpha, ad[1], ad[5]);
    of4 cd = read_image2d(cdimg, cu, cv);
    of4 cm = read_image2d(cmimg, cu, cv);
    const float Ta = ad[15];
    cd = quat_rotate(cd, ori);
    float ur_norm_sq = ur.x * ur.x + ur.y * ur.y + ur.z * ur.z;
    float tu = Ta * ur_norm_sq;
    of4 dudt = f4(tu * cd.x + 0.0f, tu * cd.y + 0.0f, tu * cd.z + -9.8f, tu * cd.w + 0.0f);
    dwdt->x = ((tu * ad[12]) * cm.x) * RADIANS_PER_DEGREE;
    dwdt->y = ((tu * ad[13]) * cm.y) * RADIANS_PER_DEGREE;
    dwdt->z = ((tu * ad[14]) * cm.z) * RADIANS_PER_DEGREE;
    dwdt->w = ((tu * 0.0f) * cm.w) * RADIANS_PER_DEGREE;
    return dudt;
}

/* ---- compute_ellipsoid_rcs (rs.cl:268-280) ---- */
static inline of4 compute_ellipsoid_rcs(of4 pos, const of4 *table, const float *td) {
    float fidx = cl_clamp(fmaf(pos.w, td[0], td[1]), 0.0f, td[2]);
    uint32_t idx = cl_f2u_rtz(fidx);
    of4 xz = table[idx];
    /* cos^2 of the elevation beta = atan2(z, |xy|), formed as |xy|^2 / |xyz|^2:
     * the same quantity as cos(beta) * cos(beta) without the two
     * transcendental calls (1 at the origin, where atan2(0, 0) = 0) */
    const float h2 = pos.x * pos.x + pos.y * pos.y;
    const float r2 = h2 + pos.z * pos.z;
    const float cb2 = r2 > 0.0f ? h2 / r2 : 1.0f;
    return f4(xz.x, xz.y, xz.x + (xz.z - xz.x) * cb2, xz.y + (xz.w - xz.y) * cb2);
}

/* ---- compute_debris_rcs (rs.cl:282-359) ---- */
static of4 compute_debris_rcs(of4 pos, of4 ori, or_image re_img, or_image im_img, const float *rd,
                              const float *sd) {
    uint32_t concept = rsm_f2u(sd[5]);
    float el = rsm_atan2f(pos.z, sqrtf(pos.x * pos.x + pos.y * pos.y));
    float az = rsm_atan2f(pos.x, pos.y);
    float se, ce, sa, ca;
    rsm_sincosf(0.5f * (el + M_PI_2_F), &se, &ce);
    rsm_sincosf(0.5f * (az), &sa, &ca);
    of4 o_conj = f4((-se * ca + ce * sa) * M_SQRT1_2_F,
                    (ce * ca + se * sa) * M_SQRT1_2_F,
                    (se * ca + ce * sa) * M_SQRT1_2_F,
                    (ce * ca + -se * sa) * M_SQRT1_2_F);
    of4 R = quat_mult(ori, o_conj);
    of4 q = f4(R.x, R.z, -R.y, R.w);
    float alpha, beta, gamma;
    float beta_arg = q.w * q.w + q.z * q.z - q.y * q.y - q.x * q.x;
    if (beta_arg > 0.999847f || beta_arg < -0.999847f) {
        alpha = 0.0f;
        beta = 0.0f;
        gamma = cl_sign(q.z) * rsm_acosf(q.w) * 2.0f;
    } else {
        alpha = rsm_atan2f(q.y * q.z - q.w * q.x, q.x * q.z + q.w * q.y);
        beta = rsm_acosf(q.w * q.w + q.z * q.z - q.y * q.y - q.x * q.x);
        gamma = rsm_atan2f(q.y * q.z + q.w * q.x, q.w * q.y - q.x * q.z);
    }
    float cu = fmaf(alpha, rd[0], rd[4]);
    float cv = fmaf(beta, rd[1], rd[5]);
    of4 re = read_image2d(re_img, cu, cv);
    of4 im = read_image2d(im_img, cu, cv);
    float sg, cg;
    rsm_sincosf(gamma, &sg, &cg);
    float hh_real = cg * (cg * re.x - re.z * sg) - sg * (cg * re.z - re.y * sg);
    float hh_imag = cg * (cg * im.x - im.z * sg) - sg * (cg * im.z - im.y * sg);
    float vv_real = cg * (cg * re.y + re.z * sg) + sg * (cg * re.z + re.x * sg);
    float vv_imag = cg * (cg * im.y + im.z * sg) + sg * (cg * im.z + im.x * sg);
    of4 ss = f4(hh_real, hh_imag, vv_real, vv_imag);
    if (concept & OR_CONCEPT_CROSS_POL) {
        float hv_real = cg * (cg * re.z + re.x * sg) - sg * (cg * re.y + re.z * sg);
        float hv_imag = cg * (cg * im.z + im.x * sg) - sg * (cg * im.y + im.z * sg);
        float vh_real = cg * (cg * re.z - re.y * sg) + sg * (cg * re.x - re.z * sg);
        float vh_imag = cg * (cg * im.z - im.y * sg) + sg * (cg * im.x - im.z * sg);
        ss.x = ss.x + vh_real;
        ss.y = ss.y + vh_imag;
        ss.z = ss.z + hv_real;
        ss.w = ss.w + hv_imag;
    }
    return ss;
}

static inline int is_outside(of4 pos, const float *sd) {
    return (pos.x <= sd[8]) | (pos.y <= sd[9]) | (pos.z <= sd[10]) |
           (pos.x >= sd[8] + sd[12]) | (pos.y >= sd[9] + sd[13]) | (pos.z >= sd[10] + sd[14]);
}

/* ---- bg_atts (rs.cl:533-580) ---- */
void or_bg_atts(of4 *p, of4 *v, of4 *x, ou4 *y, or_image uvwt, const float *wd, const of4 *drop_rcs,
                const float *drd, const float *sd, size_t origin, size_t count) {
    const float dt = sd[11];
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < (long long)count; ii++) {
        size_t i = origin + (size_t)ii;
        of4 pos = p[i];
        of4 vel = v[i];
        pos.x = pos.x + vel.x * dt;
        pos.y = pos.y + vel.y * dt;
        pos.z = pos.z + vel.z * dt;
        pos.w = pos.w + vel.w * 0.0f;
        if (is_outside(pos, sd)) {
            ou4 seed = y[i];
            of4 r = cl_rand(&seed);
            pos.x = r.x * sd[12] + sd[8];
            pos.y = r.y * sd[13] + sd[9];
            pos.z = r.z * sd[14] + sd[10];
            vel = f4(0.0f, 0.0f, 0.0f, 0.0f);
            p[i] = pos;
            v[i] = vel;
            y[i] = seed;
            continue;
        }
        vel = compute_bg_vel(pos, uvwt, wd, sd);
        of4 rcs = compute_ellipsoid_rcs(pos, drop_rcs, drd);
        p[i] = pos;
        v[i] = vel;
        x[i] = rcs;
    }
}

/* ---- fp_atts (rs.cl:590-648) ---- */
void or_fp_atts(of4 *p, of4 *v, of4 *x, or_image uvwt, or_image cpxx, const float *wd, const float *sd,
                size_t origin, size_t count) {
    const float wav_num = sd[4];
    const float dt = sd[11];
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < (long long)count; ii++) {
        size_t i = origin + (size_t)ii;
        of4 pos = p[i];
        of4 vel = v[i];
        of4 rcs = x[i];
        float c3[3];
        wind_table_index(c3, pos, wd, sd);
        of4 uv = read_image3d(uvwt, c3[0], c3[1], c3[2]);
        of4 cp = read_image3d(cpxx, c3[0], c3[1], c3[2]);
        float l = len3(pos.x, pos.y, pos.z);
        float nx = pos.x / l, ny = pos.y / l, nz = pos.z / l;
        float phi = rcs.w - wav_num * (nx * uv.x + ny * uv.y + nz * uv.z) * dt;
        float cn2 = cp.x;
        float a = rsm_powf(10.0f, cn2);
        float s, c;
        rsm_sincosf(phi, &s, &c);
        rcs.x = a * c;
        rcs.y = a * s;
        rcs.z = cn2;
        rcs.w = rsm_atan2f(s, c);
        vel.x = uv.x;
        vel.y = uv.y;
        vel.z = uv.z;
        v[i] = vel;
        x[i] = rcs;
        p[i] = pos;
    }
}

/* ---- el_atts (rs.cl:653-739) ---- */
void or_el_atts(of4 *p, of4 *v, of4 *x, ou4 *y, or_image uvwt, const float *wd, const of4 *drop_rcs,
                const float *drd, const float *sd, size_t origin, size_t count) {
    const float dt = sd[11];
    const uint32_t concept = rsm_f2u(sd[5]);
    const float rho_air = 1.225f;
    const float rho_over_mu_air = 6.7308e4f;
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < (long long)count; ii++) {
        size_t i = origin + (size_t)ii;
        of4 pos = p[i];
        of4 vel = v[i];
        of4 rcs = x[i];
        ou4 seed = y[i];
        pos.x = fmaf(vel.x, dt, pos.x);
        pos.y = fmaf(vel.y, dt, pos.y);
        pos.z = fmaf(vel.z, dt, pos.z);
        pos.w = fmaf(vel.w, 0.0f, pos.w);
        const float area_over_mass_particle = 0.003006012f / pos.w;
        if (is_outside(pos, sd)) {
            of4 r = cl_rand(&seed);
            pos.x = fmaf(r.x, sd[12], sd[8]);
            pos.y = fmaf(r.y, sd[13], sd[9]);
            pos.z = fmaf(r.z, sd[14], sd[10]);
            vel = f4(0.0f, 0.0f, 0.0f, 0.0f);
        } else {
            of4 bg_vel = compute_bg_vel(pos, uvwt, wd, sd);
            of4 dv = f4(bg_vel.x - vel.x, bg_vel.y - vel.y, bg_vel.z - vel.z, bg_vel.w - vel.w);
            float dva = len3(dv.x, dv.y, dv.z);
            const float g_dt = -9.8f * dt;
            if (dva > 1.0e-3f) {
                float re = rho_over_mu_air * (2.0f * pos.w) * dva;
                float cd = 24.0f / re + 6.0f / (1.0f + sqrtf(re)) + 0.4f;
                float k = 0.5f * rho_air * cd * area_over_mass_particle * dva;
                of4 dudt = f4(k * dv.x + 0.0f, k * dv.y + 0.0f, k * dv.z + -9.8f, k * dv.w + 0.0f);
                vel.x = vel.x + dudt.x * dt;
                vel.y = vel.y + dudt.y * dt;
                vel.z = vel.z + dudt.z * dt;
                vel.w = vel.w + dudt.w * 0.0f;
                if ((concept & OR_CONCEPT_BOUNDED) && len4(vel) > fmaxf(1.0f, 3.0f * len4(bg_vel))) {
                    vel.x = bg_vel.x + 0.0f * dt;
                    vel.y = bg_vel.y + 0.0f * dt;
                    vel.z = bg_vel.z + g_dt;
                    vel.w = bg_vel.w + 0.0f * 0.0f;
                }
            } else {
                vel.x = vel.x + 0.0f * dt;
                vel.y = vel.y + 0.0f * dt;
                vel.z = vel.z + g_dt;
                vel.w = vel.w + 0.0f * 0.0f;
            }
            rcs = compute_ellipsoid_rcs(pos, drop_rcs, drd);
        }
        p[i] = pos;
        v[i] = vel;
        x[i] = rcs;
        y[i] = seed;
    }
}

/* ---- db_atts (rs.cl:744-907) ---- */
void or_db_atts(of4 *p, of4 *o, of4 *v, of4 *t, of4 *x, ou4 *y, or_image uvwt, const float *wd,
                or_image adm_cd, or_image adm_cm, const float *ad, or_image rcs_real, or_image rcs_imag,
                const float *rd, const float *dff_icdf, const float *fd, const float *sd,
                size_t origin, size_t count) {
    const uint32_t concept = rsm_f2u(sd[5]);
    const float dt = sd[11];
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < (long long)count; ii++) {
        size_t i = origin + (size_t)ii;
        of4 pos = p[i];
        of4 ori = o[i];
        of4 vel = v[i];
        of4 tum = t[i];
        of4 rcs;
        ori = normalize4(quat_mult(ori, tum));
        pos.x = pos.x + vel.x * dt;
        pos.y = pos.y + vel.y * dt;
        pos.z = pos.z + vel.z * dt;
        pos.w = pos.w + vel.w * 0.0f;
        if (is_outside(pos, sd)) {
            ou4 seed = y[i];
            of4 r = cl_rand(&seed);
            if (concept & OR_CONCEPT_DFF) {
                /* debris flux field, inverse-CDF placement (rs.cl:795-835) */
                float fi0, fi1;
                float raw0 = cl_clamp(fmaf(r.x, fd[15], 0.0f), 0.0f, fd[15]);
                float raw1 = cl_clamp(fmaf(r.x, fd[15], 1.0f), 0.0f, fd[15]);
                float dec0 = cl_fract(raw0, &fi0);
                (void)cl_fract(raw1, &fi1);
                uint32_t i0 = cl_f2u_rtz(fi0), i1 = cl_f2u_rtz(fi1);
                float cidx = cl_mix(dff_icdf[i0], dff_icdf[i1], dec0);
                pos.y = floorf(cidx / fd[13]);
                pos.x = fmaf(pos.y, -fd[13], cidx);
                pos.y = pos.y + r.y;
                if (fd[14] == 1.0f) {
                    float rx = pos.x - fmaf(0.5f, fd[8], 0.5f);
                    float ry = pos.y - fmaf(0.5f, fd[9], 0.5f);
                    float px = fmaf(rsm_powf(fd[4], fabsf(rx)), -fd[0], fd[0]);
                    float py = fmaf(rsm_powf(fd[5], fabsf(ry)), -fd[1], fd[1]);
                    pos.x = copysignf(px, rx) + fmaf(0.5f, sd[12], sd[8]);
                    pos.y = copysignf(py, ry) + fmaf(0.5f, sd[13], sd[9]);
                } else if (fd[14] == 2.0f) {
                    pos.x = fmaf(pos.x, sd[12] * fd[0], sd[8]);
                    pos.y = fmaf(pos.y, sd[13] * fd[1], sd[9]);
                } else {
                    pos.x = fmaf(pos.x, fd[0], sd[8]);
                    pos.y = fmaf(pos.y, fd[1], sd[9]);
                }
                pos.z = MIN_HEIGHT;
            } else {
                pos.x = fmaf(r.x, sd[12], sd[8]);
                pos.y = fmaf(r.y, sd[13], sd[9]);
                pos.z = sd[10] + MIN_HEIGHT;
            }
            r = cl_rand(&seed);
            of4 c = f4(sqrtf(-2.0f * rsm_logf(r.x)), sqrtf(-2.0f * rsm_logf(r.y)), sqrtf(-2.0f * rsm_logf(r.z)), r.w);
            r = cl_rand(&seed);
            c.x = c.x * rsm_cosf(2.0f * M_PI_F * r.x);
            c.y = c.y * rsm_cosf(2.0f * M_PI_F * r.y);
            c.z = c.z * rsm_cosf(2.0f * M_PI_F * r.z);
            float sin_th_2, cos_th_2;
            rsm_sincosf(M_PI_F * c.w, &sin_th_2, &cos_th_2);
            float sqxy = sqrtf(c.x * c.x + c.z * c.z);
            float sqxyz = sqrtf(c.x * c.x + c.y * c.y + c.z * c.z);
            float sa, ca;
            rsm_sincosf(0.5f * rsm_acosf(c.y / sqxyz), &sa, &ca);
            ori.x = c.x * ca * sin_th_2 / sqxyz - c.x * c.y * sin_th_2 / sqxyz * sa / sqxy + c.z * cos_th_2 * sa / sqxy;
            ori.y = sin_th_2 / sqxyz * (sqxy * sa + c.y * ca);
            ori.z = c.z * ca * sin_th_2 / sqxyz - c.x * cos_th_2 * sa / sqxy - c.y * c.z * sin_th_2 * sa / sqxy / sqxyz;
            ori.w = cos_th_2 * ca;
            vel = f4(0.0f, 0.0f, 0.0f, 0.0f);
            tum = f4(0.0f, 0.0f, 0.0f, 1.0f);
            rcs = f4(0.0f, 0.0f, 0.0f, 0.0f);
            p[i] = pos;
            o[i] = ori;
            v[i] = vel;
            t[i] = tum;
            x[i] = rcs;
            y[i] = seed;
            continue;
        }
        of4 vel_bg = compute_bg_vel(pos, uvwt, wd, sd);
        of4 dwdt;
        of4 dudt = compute_dudt_dwdt(&dwdt, vel, vel_bg, ori, adm_cd, adm_cm, ad);
        if ((concept & OR_CONCEPT_BOUNDED) &&
            sqrtf((vel.x + dudt.x * dt) * (vel.x + dudt.x * dt) + (vel.y + dudt.y * dt) * (vel.y + dudt.y * dt)) >
                3.0f * sqrtf(vel_bg.x * vel_bg.x + vel_bg.y * vel_bg.y)) {
            vel.x = vel_bg.x;
            vel.y = vel_bg.y;
            vel.z = vel.z + dudt.z * dt;
        } else {
            vel.x = vel.x + dudt.x * dt;
            vel.y = vel.y + dudt.y * dt;
            vel.z = vel.z + dudt.z * dt;
            vel.w = vel.w + dudt.w * 0.0f;
        }
        float dw[4] = {dwdt.x * dt, dwdt.y * dt, dwdt.z * dt, dwdt.w * 0.0f};
        float s[4], c[4];
        for (int l = 0; l < 4; l++) {
            rsm_sincosf(dw[l], &s[l], &c[l]);
        }
        tum = f4(c[0] * s[1] * s[2] + s[0] * c[1] * c[2],
                 c[0] * s[1] * c[2] - s[0] * c[1] * s[2],
                 c[0] * c[1] * s[2] + s[0] * s[1] * c[2],
                 c[0] * c[1] * c[2] - s[0] * s[1] * s[2]);
        tum = normalize4(tum);
        rcs = compute_debris_rcs(pos, ori, rcs_real, rcs_imag, rd, sd);
        p[i] = pos;
        o[i] = ori;
        v[i] = vel;
        t[i] = tum;
        x[i] = rcs;
    }
}

/* ---- db_rcs (rs.cl:909-919) ---- */
void or_db_rcs(const of4 *p, const of4 *o, of4 *x, or_image rcs_real, or_image rcs_imag, const float *rd,
               const float *sd, size_t origin, size_t count) {
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < (long long)count; ii++) {
        size_t i = origin + (size_t)ii;
        x[i] = compute_debris_rcs(p[i], o[i], rcs_real, rcs_imag, rd, sd);
    }
}

/* ---- scat_sig_aux (rs.cl:1050-1110) ---- */
static inline void sig_aux_one(of4 *sig_out, of4 *aux, of4 p, of4 rcs, const float *aw, const float *awd,
                               const float *sd) {
    float l = len3(p.x, p.y, p.z);
    float nx = p.x / l, ny = p.y / l, nz = p.z / l;
    float angle = rsm_acosf(sd[0] * nx + sd[1] * ny + sd[2] * nz);
    float fi0, fi1;
    float raw0 = cl_clamp(fmaf(angle, awd[0], awd[1] + 0.0f), 0.0f, awd[2]);
    float raw1 = cl_clamp(fmaf(angle, awd[0], awd[1] + 1.0f), 0.0f, awd[2]);
    float dec0 = cl_fract(raw0, &fi0);
    (void)cl_fract(raw1, &fi1);
    uint32_t i0 = cl_f2u_rtz(fi0), i1 = cl_f2u_rtz(fi1);
    aux->x = len3(p.x, p.y, p.z);
    aux->y = aux->y + sd[15];
    aux->w = cl_mix(aw[i0], aw[i1], dec0);
    float atten = 1.0f / (aux->x * aux->x);
    float phase = aux->x * sd[4];
    float ss, cc;
    rsm_sincosf(phase, &ss, &cc);
    /* cl_complex_multiply(x, (cc, -ss, cc, -ss)) * atten */
    float ms = -ss;
    of4 s = f4((rcs.x * cc - rcs.y * ms) * atten, (rcs.y * cc + rcs.x * ms) * atten,
               (rcs.z * cc - rcs.w * ms) * atten, (rcs.w * cc + rcs.z * ms) * atten);
    *sig_out = s;
}

void or_scat_sig_aux(of4 *s, of4 *a, const of4 *p, const of4 *x, const float *aw, const float *awd,
                     const float *sd, size_t count) {
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < (long long)count; ii++) {
        size_t i = (size_t)ii;
        of4 aux = a[i];
        sig_aux_one(&s[i], &aux, p[i], x[i], aw, awd, sd);
        a[i] = aux;
    }
}

/* ---- pop (rs.cl:1444-1453) ---- */
void or_pop(of4 *rcs, of4 *aux, of4 *pos, const float *sd, size_t count) {
    for (size_t k = 0; k < count; k++) {
        of4 p = f4((float)(uint32_t)(k % 9) - 4.0f, (float)(uint32_t)k / 90000.0f + 1.0f, 0.1f, 1.0f);
        rcs[k] = f4(1.0f, 0.5f, 1.0f, 0.5f);
        float l = len3(p.x, p.y, p.z);
        float nx = p.x / l, ny = p.y / l, nz = p.z / l;
        aux[k] = f4(len3(p.x, p.y, p.z), 1.0f, rsm_acosf(sd[0] * nx + sd[1] * ny + sd[2] * nz), 1.0f);
        pos[k] = p;
    }
}

/* ---- RS_make_pulse_params (rs.c:1284-1386) ---- */
int or_make_pulse_params(or_pulse_params *P, uint32_t count, uint32_t group_size_multiple,
                         uint32_t user_max_groups, uint32_t max_local_mem_size, float range_start,
                         float range_delta, uint32_t range_count) {
    memset(P, 0, sizeof(*P));
    P->num_scats = count;
    P->user_max_groups = user_max_groups;
    P->user_max_work_items = group_size_multiple;
    P->range_start = range_start;
    P->range_delta = range_delta;
    P->range_count = range_count > 1 ? range_count : 1;
    if (user_max_groups > 1024) {
        P->user_max_groups = 1024;
    }
    uint32_t work_items = count > P->user_max_work_items * 2 ? P->user_max_work_items : count / 2;
    if (work_items == 0) {
        return -3;   /* count < 2: the reference divides by zero on the next line (rs.c:1308-1311) */
    }
    uint32_t group_count = count <= work_items * 2 ? 1 : (count + work_items * 2 - 1) / (work_items * 2);
    if (group_count > P->user_max_groups) {
        group_count = P->user_max_groups;
    }
    P->entry_counts[0] = count;
    P->group_counts[0] = group_count;
    P->global[0] = (size_t)group_count * work_items;
    P->local[0] = work_items;
    P->local_mem_size[0] = (size_t)range_count * work_items * 16;
    while (P->local_mem_size[0] > max_local_mem_size) {
        if (range_count % 2 == 0) {
            work_items /= 2;
            group_count *= 2;
            if (group_count > P->user_max_groups) {
                group_count = P->user_max_groups;
            }
            P->group_counts[0] = group_count;
            P->global[0] = (size_t)group_count * work_items;
            P->local[0] = work_items;
            P->local_mem_size[0] = (size_t)range_count * work_items * 16;
        } else {
            return -1;   /* the reference exits here (rs.c:1341-1344) */
        }
    }
    uint32_t work_count = group_count * P->range_count;
    P->entry_counts[1] = work_count;
    work_items = work_count / (P->range_count * 2);
    if (work_items < 1) {
        work_items = 1;
    }
    if (P->local[0] % P->range_count == 0 && group_size_multiple >= work_items) {
        P->pass_2_method = OR_PASS_2_UNIVERSAL;
        P->group_counts[1] = 1;
        P->global[1] = work_items;
        P->local[1] = work_items;
        P->local_mem_size[1] = work_items * 16;
    } else if (group_count >= 2 * P->range_count && group_size_multiple >= work_items) {
        P->pass_2_method = OR_PASS_2_IN_LOCAL;
        P->group_counts[1] = 1;
        P->global[1] = work_items;
        P->local[1] = work_items;
        P->local_mem_size[1] = work_items * 16;
    } else {
        P->pass_2_method = OR_PASS_2_IN_RANGE;
        P->group_counts[1] = 1;
        P->global[1] = P->range_count;
        P->local[1] = 1;
        P->local_mem_size[1] = 16;
    }
    return 0;
}

/* ---- make_pulse_pass_1 (rs.cl:1125-1301) ---- */
static inline of4 ld_or_zero(const of4 *a, size_t n_alloc, size_t i) {
    if (i < n_alloc) return a[i];
    return f4(0.0f, 0.0f, 0.0f, 0.0f);
}

void or_make_pulse_pass_1(of4 *out, const of4 *sig, const of4 *aux, size_t n_alloc, const float *W,
                          const float *wd, float range_start, float range_delta, uint32_t range_count,
                          uint32_t group_count, uint32_t n, uint32_t local_size) {
    const uint32_t G = range_count;
    const uint32_t group_stride = 2 * local_size;
    const uint32_t local_stride = group_stride * group_count;
    const float xs = wd[0];
    const float x0_0 = wd[1] + 0.0f;
    const float x0_1 = wd[1] + 1.0f;
    const float xm = wd[2];
    /* the gate origins of every work item: range_start advanced by the
     * kernel's repeated FP32 additions (rs.cl:1214), the same bits */
    float *rk = (float *)malloc(sizeof(float) * (G ? G : 1));
    float r = range_start;
    for (uint32_t k = 0; k < G; k++) {
        rk[k] = r;
        r = r + range_delta;
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (long long gg = 0; gg < (long long)group_count; gg++) {
        uint32_t group_id = (uint32_t)gg;
        /* local_size extra zero entries: the tree below assumes a power-of-two
         * local size; with any other size (counts < 128, work_items = count / 2)
         * it adds entries of the next gate's column, and for the last gate it
         * reads past the G x local_size array of the reference */
        of4 *shared = (of4 *)calloc((size_t)G * local_size + local_size, sizeof(of4));
        /* one work item's G x 4 sums, gate-major: its entries of `shared`
         * (shared[lid + k local_size]) receive the same additions in the same
         * order from zero, so they are copied there when it is done; the gate
         * loop then runs over contiguous memory */
        float *acc = (float *)malloc(sizeof(float) * 4 * (G ? G : 1));
        for (uint32_t lid = 0; lid < local_size; lid++) {
            memset(acc, 0, sizeof(float) * 4 * G);
            uint32_t i = group_id * group_stride + lid;
            while (i < n) {
                uint32_t j = i + local_size;
                of4 s_a = ld_or_zero(sig, n_alloc, i);
                of4 s_b = ld_or_zero(sig, n_alloc, j);
                of4 a_a = ld_or_zero(aux, n_alloc, i);
                of4 a_b = ld_or_zero(aux, n_alloc, j);
                const float r_a = a_a.x, r_b = a_b.x;
                const float sax = s_a.x * a_a.w, say = s_a.y * a_a.w, saz = s_a.z * a_a.w, saw = s_a.w * a_a.w;
                const float sbx = s_b.x * a_b.w, sby = s_b.y * a_b.w, sbz = s_b.z * a_b.w, sbw = s_b.w * a_b.w;
                /* the four table coordinates of rs.cl's float4 fidx_raw
                 * (r_a, r_a, r_b, r_b) - r, lane by lane */
                const float x04[4] = {x0_0, x0_1, x0_0, x0_1};
                for (uint32_t k = 0; k < G; k++) {
                    const float d4[4] = {r_a - rk[k], r_a - rk[k], r_b - rk[k], r_b - rk[k]};
                    float fl[4], dec[4], w[4];
                    for (int l = 0; l < 4; l++) {
                        const float v = cl_clamp(fmaf(d4[l], xs, x04[l]), 0.0f, xm);
                        fl[l] = floorf(v);
                        dec[l] = fminf(v - fl[l], 0x1.fffffep-1f);   /* fract */
                    }
                    /* the indices are floors of values clamped to [0, xm]: in
                     * range, so the conversion is convert_uint's */
                    for (int l = 0; l < 4; l++) w[l] = W[(uint32_t)fl[l]];
                    const float w_a = cl_mix(w[0], w[1], dec[0]);
                    const float w_b = cl_mix(w[2], w[3], dec[2]);
                    float *a = acc + 4 * k;
                    a[0] = a[0] + (w_a * sax + w_b * sbx);
                    a[1] = a[1] + (w_a * say + w_b * sby);
                    a[2] = a[2] + (w_a * saz + w_b * sbz);
                    a[3] = a[3] + (w_a * saw + w_b * sbw);
                }
                i += local_stride;
            }
            for (uint32_t k = 0; k < G; k++) {
                of4 *sh = &shared[lid + (size_t)k * local_size];
                sh->x = acc[4 * k];
                sh->y = acc[4 * k + 1];
                sh->z = acc[4 * k + 2];
                sh->w = acc[4 * k + 3];
            }
        }
        free(acc);
        /* the log-step tree of rs.cl:1224-1290 */
        const uint32_t local_numel = G * local_size;
        for (uint32_t half = 512; half >= 1; half >>= 1) {
            if (local_size > half) {
                for (uint32_t lid = 0; lid < half; lid++) {
                    for (uint32_t k = 0; k < local_numel; k += local_size) {
                        of4 *a = &shared[lid + k];
                        const of4 *b = &shared[lid + k + half];
                        a->x = a->x + b->x;
                        a->y = a->y + b->y;
                        a->z = a->z + b->z;
                        a->w = a->w + b->w;
                    }
                }
            }
        }
        of4 *o = &out[(size_t)group_id * G];
        for (uint32_t k = 0; k < G; k++) {
            o[k] = shared[(size_t)k * local_size];
        }
        free(shared);
    }
    free(rk);
}

/* ---- make_pulse_pass_2_local body (rs.cl:1304-1338) ---- */
void or_make_pulse_pass_2_local_body(of4 *out, const of4 *in, size_t in_alloc, uint32_t range_count, uint32_t n,
                                     size_t global, size_t local) {
    (void)local;
    const uint32_t group_stride = 2 * range_count;
    for (size_t gid = 0; gid < global; gid++) {
        of4 acc = f4(0.0f, 0.0f, 0.0f, 0.0f);
        uint32_t i = (uint32_t)gid;
        while (i < n) {
            of4 a = ld_or_zero(in, in_alloc, i);
            of4 b = ld_or_zero(in, in_alloc, (size_t)i + range_count);
            acc.x = acc.x + (a.x + b.x);
            acc.y = acc.y + (a.y + b.y);
            acc.z = acc.z + (a.z + b.z);
            acc.w = acc.w + (a.w + b.w);
            i += group_stride;
        }
        out[gid] = acc;
    }
}

/* ---- make_pulse_pass_2_range body (rs.cl:1341-1359) ---- */
void or_make_pulse_pass_2_range_body(of4 *out, const of4 *in, size_t in_alloc, uint32_t range_count, uint32_t n,
                                     size_t global) {
    for (size_t rid = 0; rid < global; rid++) {
        of4 tmp = f4(0.0f, 0.0f, 0.0f, 0.0f);
        for (uint32_t i = (uint32_t)rid; i < n; i += range_count) {
            of4 a = ld_or_zero(in, in_alloc, i);
            tmp.x = tmp.x + a.x;
            tmp.y = tmp.y + a.y;
            tmp.z = tmp.z + a.z;
            tmp.w = tmp.w + a.w;
        }
        out[rid] = tmp;
    }
}

/* ---- make_pulse_pass_2_group body (rs.cl:1362-1441), one work group ---- */
void or_make_pulse_pass_2_group_body(of4 *out, const of4 *in, size_t in_alloc, uint32_t range_count,
                                     size_t local) {
    const size_t group_stride = (size_t)range_count * local;
    of4 *shared = (of4 *)calloc(local, sizeof(of4));
    for (uint32_t k = 0; k < range_count; k++) {
        for (size_t lid = 0; lid < local; lid++) {
            size_t i = lid * range_count;
            of4 a = ld_or_zero(in, in_alloc, i + k);
            of4 b = ld_or_zero(in, in_alloc, i + k + group_stride);
            shared[lid] = f4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
        }
        for (size_t half = 512; half >= 1; half >>= 1) {
            if (local > half) {
                for (size_t lid = 0; lid < half; lid++) {
                    shared[lid].x = shared[lid].x + shared[lid + half].x;
                    shared[lid].y = shared[lid].y + shared[lid + half].y;
                    shared[lid].z = shared[lid].z + shared[lid + half].z;
                    shared[lid].w = shared[lid].w + shared[lid + half].w;
                }
            }
        }
        out[k] = shared[0];
    }
    free(shared);
}

/* ---- RS_make_pulse (rs.c:5563-5573) with RS_worker_malloc's kernel choice
 * (rs.c:905-911).  rs.c binds its "_local" handle to the kernel built from
 * "make_pulse_pass_2_range" and its "_range" handle to "make_pulse_pass_2_local"
 * (rs.c:506-507); name_swap = 1 reproduces that, name_swap = 0 the direct
 * binding test_make_pulse.c uses (test_make_pulse.c:468-474).  Pass 2 may write
 * up to global[1] entries (more than range_count in the "_local" geometry), so
 * it writes to a scratch buffer of that size and the first range_count
 * entries are returned. ---- */
int or_make_pulse(of4 *pulse, of4 *sig, of4 *aux, const of4 *pos, const of4 *rcs, size_t num_scats, size_t n_alloc,
                  const float *aw, const float *awd, const float *rw, const float *rwd, float range_start,
                  float range_delta, uint32_t range_count, const float *sd, uint32_t group_size_multiple,
                  uint32_t max_work_group_size, uint32_t local_mem_size, int name_swap) {
    or_pulse_params P;
    if (or_make_pulse_params(&P, (uint32_t)num_scats, group_size_multiple, max_work_group_size, local_mem_size,
                             range_start, range_delta, range_count) != 0) {
        return -1;
    }
    or_scat_sig_aux(sig, aux, pos, rcs, aw, awd, sd, num_scats);
    size_t work_alloc = P.global[0] * P.local[0] * range_count;
    of4 *work = (of4 *)calloc(work_alloc, sizeof(of4));
    size_t out_n = P.global[1] > range_count ? P.global[1] : range_count;
    of4 *out = (of4 *)calloc(out_n, sizeof(of4));
    if (work == NULL || out == NULL) {
        free(work);
        free(out);
        return -2;
    }
    or_make_pulse_pass_1(work, sig, aux, n_alloc, rw, rwd, range_start, range_delta, range_count,
                         P.group_counts[0], P.entry_counts[0], (uint32_t)P.local[0]);
    int use_range_body;
    if (P.pass_2_method == OR_PASS_2_IN_LOCAL) {
        use_range_body = name_swap ? 1 : 0;
    } else if (P.pass_2_method == OR_PASS_2_IN_RANGE) {
        use_range_body = name_swap ? 0 : 1;
    } else {
        use_range_body = -1;
    }
    if (use_range_body == 1) {
        or_make_pulse_pass_2_range_body(out, work, work_alloc, range_count, P.entry_counts[1], P.global[1]);
    } else if (use_range_body == 0) {
        or_make_pulse_pass_2_local_body(out, work, work_alloc, range_count, P.entry_counts[1], P.global[1],
                                        P.local[1]);
    } else {
        or_make_pulse_pass_2_group_body(out, work, work_alloc, range_count, P.local[1]);
    }
    memcpy(pulse, out, sizeof(of4) * range_count);
    free(work);
    free(out);
    return 0;
}

/* ---- the FP32 per-scatterer, per-gate contributions of scat_sig_aux +
 * pass 1 (rs.cl:1050-1217: w * (sig * angular weight), the gate origin
 * advanced by FP32 additions), summed exactly in double ---- */
void or_make_pulse_direct(double *pulse4, double *abs4, const of4 *pos, const of4 *rcs, size_t n, const float *aw,
                          const float *awd, const float *rw, const float *rwd, float range_start, float range_delta,
                          uint32_t G, const float *sd) {
    memset(pulse4, 0, sizeof(double) * 4 * G);
    if (abs4) memset(abs4, 0, sizeof(double) * 4 * G);
    const float xs = rwd[0], x0_0 = rwd[1] + 0.0f, x0_1 = rwd[1] + 1.0f, xm = rwd[2];
    int nt = or_num_threads();
    double *acc = (double *)calloc((size_t)nt * 8 * G, sizeof(double));
#pragma omp parallel
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double *my = acc + (size_t)tid * 8 * G;
#pragma omp for schedule(static)
        for (long long ii = 0; ii < (long long)n; ii++) {
            of4 sig, aux = f4(0.0f, 0.0f, 0.0f, 0.0f);
            sig_aux_one(&sig, &aux, pos[ii], rcs[ii], aw, awd, sd);
            float s[4] = {sig.x * aux.w, sig.y * aux.w, sig.z * aux.w, sig.w * aux.w};
            float r = range_start;
            for (uint32_t k = 0; k < G; k++) {
                float d = aux.x - r;
                float f0, f1;
                float dec0 = cl_fract(cl_clamp(fmaf(d, xs, x0_0), 0.0f, xm), &f0);
                (void)cl_fract(cl_clamp(fmaf(d, xs, x0_1), 0.0f, xm), &f1);
                float w = cl_mix(rw[cl_f2u_rtz(f0)], rw[cl_f2u_rtz(f1)], dec0);
                for (int l = 0; l < 4; l++) {
                    float c = w * s[l];
                    my[k * 8 + l] += (double)c;
                    my[k * 8 + 4 + l] += fabs((double)c);
                }
                r = r + range_delta;
            }
        }
    }
    for (int t = 0; t < nt; t++) {
        for (uint32_t k = 0; k < G; k++) {
            for (int l = 0; l < 4; l++) {
                pulse4[k * 4 + l] += acc[((size_t)t * G + k) * 8 + l];
                if (abs4) abs4[k * 4 + l] += acc[((size_t)t * G + k) * 8 + 4 + l];
            }
        }
    }
    free(acc);
}

/* ---- FP64 reference pulse ---- */
static double read_table_lerp_f64(const float *W, double desc_s, double desc_o, double desc_m, double x) {
    double f = desc_s * x + desc_o;
    if (f < 0.0) f = 0.0;
    if (f > desc_m) f = desc_m;
    double fl = floor(f);
    double a = f - fl;
    size_t i0 = (size_t)fl;
    size_t i1 = fl + 1.0 > desc_m ? (size_t)desc_m : (size_t)fl + 1;
    return (double)W[i0] + ((double)W[i1] - (double)W[i0]) * a;
}

void or_make_pulse_f64(double *pulse4, double *abs4, const of4 *pos, const of4 *rcs, size_t n, const float *aw,
                       const float *awd, const float *rw, const float *rwd, double range_start, double range_delta,
                       uint32_t G, const float *sd) {
    memset(pulse4, 0, sizeof(double) * 4 * G);
    if (abs4) memset(abs4, 0, sizeof(double) * 4 * G);
    const double k_wav = (double)sd[4];
    const double bx = sd[0], by = sd[1], bz = sd[2];
    const double rs_ = rwd[0], ro_ = rwd[1], rm_ = rwd[2];
    const double as_ = awd[0], ao_ = awd[1], am_ = awd[2];
    int nt = or_num_threads();
    double *acc = (double *)calloc((size_t)nt * 8 * G, sizeof(double));
#pragma omp parallel
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double *my = acc + (size_t)tid * 8 * G;
#pragma omp for schedule(static)
        for (long long ii = 0; ii < (long long)n; ii++) {
            of4 p = pos[ii];
            of4 x = rcs[ii];
            double px = p.x, py = p.y, pz = p.z;
            double r = sqrt(px * px + py * py + pz * pz);
            double cx = by * pz - bz * py, cy = bz * px - bx * pz, cz = bx * py - by * px;
            double ang = atan2(sqrt(cx * cx + cy * cy + cz * cz), bx * px + by * py + bz * pz);
            double wa = read_table_lerp_f64(aw, as_, ao_, am_, ang);
            double atten = 1.0 / (r * r);
            double ph = k_wav * r;
            double s = sin(ph), c = cos(ph);
            double sig[4] = {((double)x.x * c + (double)x.y * s) * atten * wa, ((double)x.y * c - (double)x.x * s) * atten * wa,
                             ((double)x.z * c + (double)x.w * s) * atten * wa, ((double)x.w * c - (double)x.z * s) * atten * wa};
            for (uint32_t k = 0; k < G; k++) {
                double rk = range_start + (double)k * range_delta;
                double w = read_table_lerp_f64(rw, rs_, ro_, rm_, r - rk);
                if (w == 0.0) continue;
                for (int l = 0; l < 4; l++) {
                    my[k * 8 + l] += w * sig[l];
                    my[k * 8 + 4 + l] += fabs(w * sig[l]);
                }
            }
        }
    }
    for (int t = 0; t < nt; t++) {
        for (uint32_t k = 0; k < G; k++) {
            for (int l = 0; l < 4; l++) {
                pulse4[k * 4 + l] += acc[((size_t)t * G + k) * 8 + l];
                if (abs4) abs4[k * 4 + l] += acc[((size_t)t * G + k) * 8 + 4 + l];
            }
        }
    }
    free(acc);
}

/* ---- diagnostics ---- */
void or_eval_math(int fn, const float *a, const float *b, float *out, size_t n) {
    for (size_t i = 0; i < n; i++) {
        float s, c;
        switch (fn) {
            case 0: rsm_sincosf(a[i], &s, &c); out[i] = s; break;
            case 1: rsm_sincosf(a[i], &s, &c); out[i] = c; break;
            case 2: out[i] = rsm_logf(a[i]); break;
            case 3: out[i] = rsm_log1pf(a[i]); break;
            case 4: out[i] = rsm_acosf(a[i]); break;
            case 5: out[i] = rsm_atan2f(a[i], b[i]); break;
            case 6: out[i] = rsm_expf(a[i]); break;
            case 7: out[i] = rsm_powf(a[i], b[i]); break;
            case 8: {
                /* the pass-1 range weight (rs.cl:1196-1209) of d = a[i] on the
                 * triangle {0, 1, 0} with scale b[i], origin 1, max 2 */
                static const float W[3] = {0.0f, 1.0f, 0.0f};
                float f0, f1;
                const float dec0 = cl_fract(cl_clamp(fmaf(a[i], b[i], 1.0f + 0.0f), 0.0f, 2.0f), &f0);
                (void)cl_fract(cl_clamp(fmaf(a[i], b[i], 1.0f + 1.0f), 0.0f, 2.0f), &f1);
                out[i] = cl_mix(W[(uint32_t)f0], W[(uint32_t)f1], dec0);
                break;
            }
            default: out[i] = 0.0f; break;
        }
    }
}
