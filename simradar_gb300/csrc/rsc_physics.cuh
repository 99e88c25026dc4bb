/*
 * rsc_physics.cuh -- per-scatterer physics of the SimRadar emulation loop on
 * sm_103a.  Each function computes, operation for operation, what the named
 * rs.cl routine computes (this translation unit is compiled with -fmad=false;
 * fmaf appears exactly where rs.cl writes fma), with the elementary functions
 * of rsmath.h.  Texture reads are software filters over float4 arrays in HBM
 * (L2-resident), because the texture unit's 8-bit filter weights would not
 * reproduce OpenCL's single-precision linear filter; the LES wind volume is
 * kept in an x-pair layout so that the filter reads it in four 32-byte loads.
 */
#ifndef SIMRADAR_GB300_RSC_PHYSICS_CUH
#define SIMRADAR_GB300_RSC_PHYSICS_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "rsmath.h"

namespace rsc {

#define RSC_MIN_HEIGHT 2.0f
#define RSC_PI_F 3.14159274f
#define RSC_PI_2_F 1.57079637f
#define RSC_SQRT1_2_F 0.707106769f
#define RSC_RAD_PER_DEG 0.0174532924f

enum : uint32_t {
    kConceptCrossPol = 1u,
    kConceptDragged = 1u << 1,
    kConceptTransparent = 1u << 2,
    kConceptBounded = 1u << 3,
    kConceptUniformDSD = 1u << 4,
    kConceptFixedPos = 1u << 5,
    kConceptVertical = 1u << 6,
    kConceptDFF = 1u << 7
};

/* float4 image, x fastest */
struct Image {
    const float4 *data;
    int nx, ny, nz;
};

__device__ __forceinline__ float4 f4(float x, float y, float z, float w) { return make_float4(x, y, z, w); }

/* ---- OpenCL built-ins (OpenCL 1.2 sec. 6.12) ---- */
__device__ __forceinline__ float cl_clamp(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float cl_fract(float x, float *ip) {
    float fl = floorf(x);
    *ip = fl;
    return fminf(x - fl, 0x1.fffffep-1f);
}
__device__ __forceinline__ float cl_mix(float a, float b, float t) { return a + (b - a) * t; }
__device__ __forceinline__ float cl_sign(float x) {
    if (x > 0.0f) return 1.0f;
    if (x < 0.0f) return -1.0f;
    if (x == 0.0f) return x;
    return 0.0f;
}
__device__ __forceinline__ uint32_t cl_f2u_rtz(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)f;
}
__device__ __forceinline__ float len3(float x, float y, float z) { return sqrtf(x * x + y * y + z * z); }
__device__ __forceinline__ float len4(float4 v) { return sqrtf(v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w); }
/* len4(v) > max(1, 3 len4(b)) (el_atts' bound on the drop's velocity,
 * rs.cl:714), decided as those FP32 operations decide it.  When the squared
 * lengths are 0.1% or more below the squared bound -- far beyond the few
 * roundings between them and the two lengths -- the answer is false without
 * the square roots; otherwise (and for NaN or infinite lengths) the
 * reference's operations decide. */
__device__ __forceinline__ bool len4_exceeds_bound(float4 v, float4 b) {
    const float a2 = v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w;
    const float b2 = b.x * b.x + b.y * b.y + b.z * b.z + b.w * b.w;
    if (a2 < 0.999f * fmaxf(1.0f, 9.0f * b2)) return false;
    return sqrtf(a2) > fmaxf(1.0f, 3.0f * sqrtf(b2));
}
__device__ __forceinline__ float4 normalize4(float4 v) {
    float l = len4(v);
    return f4(v.x / l, v.y / l, v.z / l, v.w / l);
}

/* rand (rs.cl:35-44): 16807 * seed, masked to 31 bits, lane by lane */
__device__ __forceinline__ float4 cl_rand(uint4 *seed) {
    const float n = 1.0f / 2147483647.0f;
    seed->x = (seed->x * 16807u) & 0x7FFFFFFFu;
    seed->y = (seed->y * 16807u) & 0x7FFFFFFFu;
    seed->z = (seed->z * 16807u) & 0x7FFFFFFFu;
    seed->w = (seed->w * 16807u) & 0x7FFFFFFFu;
    return f4(__uint2float_rn(seed->x) * n, __uint2float_rn(seed->y) * n, __uint2float_rn(seed->z) * n,
              __uint2float_rn(seed->w) * n);
}

/* quaternions (rs.cl:53-85) */
__device__ __forceinline__ float4 quat_mult(float4 l, float4 r) {
    return f4(l.w * r.x - l.z * r.y + l.y * r.z + l.x * r.w,
              l.w * r.y + l.z * r.x + l.y * r.w - l.x * r.z,
              l.w * r.z + l.z * r.w - l.y * r.x + l.x * r.y,
              l.w * r.w - l.z * r.z - l.y * r.y - l.x * r.x);
}
__device__ __forceinline__ float4 quat_conj(float4 q) { return f4(-q.x, -q.y, -q.z, q.w); }
__device__ __forceinline__ float4 quat_rotate(float4 v, float4 q) { return quat_mult(quat_mult(q, v), quat_conj(q)); }

/* one axis of the OpenCL linear filter with unnormalized coordinates and
 * CLK_ADDRESS_CLAMP_TO_EDGE: i0 = floor(u - 0.5), a = frac(u - 0.5) */
__device__ __forceinline__ void tex_axis(float u, int n, int *i0, int *i1, float *a) {
    float uu = u - 0.5f;
    float fl = floorf(uu);
    *a = uu - fl;
    /* the texel pair clamp(i), clamp(i + 1) to [0, n - 1]: with i first
     * clamped to [-1, n - 1] (NaN -> -1) only one side of each can go out */
    int i = (int)fminf(fmaxf(fl, -1.0f), (float)(n - 1));
    *i0 = max(i, 0);
    *i1 = min(i + 1, n - 1);
}

__device__ __forceinline__ float4 ldg4(const float4 *p) { return __ldg(p); }

/* read_imagef on an image3d_t (sampler rs.cl:8) */
__device__ __forceinline__ float4 read_image3d(const Image &im, float u, float v, float w) {
    int i0, i1, j0, j1, k0, k1;
    float a, b, c;
    tex_axis(u, im.nx, &i0, &i1, &a);
    tex_axis(v, im.ny, &j0, &j1, &b);
    tex_axis(w, im.nz, &k0, &k1, &c);
    /* texel indices in 32 bits: the host keeps a volume below 2^31 texels */
    const unsigned sy = (unsigned)im.nx, sz = (unsigned)im.nx * (unsigned)im.ny;
    const float4 *d = im.data;
    const unsigned r00 = j0 * sy + k0 * sz, r10 = j1 * sy + k0 * sz, r01 = j0 * sy + k1 * sz, r11 = j1 * sy + k1 * sz;
    float4 t000 = ldg4(d + (r00 + i0)), t100 = ldg4(d + (r00 + i1));
    float4 t010 = ldg4(d + (r10 + i0)), t110 = ldg4(d + (r10 + i1));
    float4 t001 = ldg4(d + (r01 + i0)), t101 = ldg4(d + (r01 + i1));
    float4 t011 = ldg4(d + (r11 + i0)), t111 = ldg4(d + (r11 + i1));
    float ma = 1.0f - a, mb = 1.0f - b, mc = 1.0f - c;
    float w000 = ma * mb * mc, w100 = a * mb * mc, w010 = ma * b * mc, w110 = a * b * mc;
    float w001 = ma * mb * c, w101 = a * mb * c, w011 = ma * b * c, w111 = a * b * c;
#define RSC_TRI(L) (w000 * t000.L + w100 * t100.L + w010 * t010.L + w110 * t110.L + \
                    w001 * t001.L + w101 * t101.L + w011 * t011.L + w111 * t111.L)
    float4 r = f4(RSC_TRI(x), RSC_TRI(y), RSC_TRI(z), RSC_TRI(w));
#undef RSC_TRI
    return r;
}

/* The LES wind volume (uvwt) in x-pair layout: every row (j, k) holds nx + 2
 * pairs of texels, pair q = (T[clamp(q - 1)], T[clamp(q)]) with the clamp to
 * [0, nx - 1], 32 bytes each.  The linear filter's x axis reads texels
 * i0 = clamp(i) and i1 = clamp(i + 1) for i = floor(u - 0.5) in [-1, nx]:
 * both are pair i + 1, one 32-byte aligned load instead of two gathers. */
struct PairImage {
    const float4 *data;   /* 2 * (nx + 2) * ny * nz float4 */
    int nx, ny, nz;
};

/* one 32-byte load of two texels (the pointer is 32-byte aligned) */
__device__ __forceinline__ void ldg_pair(const float4 *p, float4 &a, float4 &b) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

/* read_image3d on the x-pair layout: the same texels, weights and sums */
__device__ __forceinline__ float4 read_pair_image3d(const PairImage &im, float u, float v, float w) {
    int j0, j1, k0, k1;
    float b, c;
    tex_axis(v, im.ny, &j0, &j1, &b);
    tex_axis(w, im.nz, &k0, &k1, &c);
    const float uu = u - 0.5f;
    const float fl = floorf(uu);
    const float a = uu - fl;
    const unsigned q = (unsigned)((int)fminf(fmaxf(fl, -1.0f), (float)im.nx) + 1);
    const unsigned sy = (unsigned)im.nx + 2u, sz = sy * (unsigned)im.ny;
    const float4 *d = im.data;
    float4 t000, t100, t010, t110, t001, t101, t011, t111;
    ldg_pair(d + 2 * (size_t)(j0 * sy + k0 * sz + q), t000, t100);
    ldg_pair(d + 2 * (size_t)(j1 * sy + k0 * sz + q), t010, t110);
    ldg_pair(d + 2 * (size_t)(j0 * sy + k1 * sz + q), t001, t101);
    ldg_pair(d + 2 * (size_t)(j1 * sy + k1 * sz + q), t011, t111);
    float ma = 1.0f - a, mb = 1.0f - b, mc = 1.0f - c;
    float w000 = ma * mb * mc, w100 = a * mb * mc, w010 = ma * b * mc, w110 = a * b * mc;
    float w001 = ma * mb * c, w101 = a * mb * c, w011 = ma * b * c, w111 = a * b * c;
#define RSC_TRI(L) (w000 * t000.L + w100 * t100.L + w010 * t010.L + w110 * t110.L + \
                    w001 * t001.L + w101 * t101.L + w011 * t011.L + w111 * t111.L)
    float4 r = f4(RSC_TRI(x), RSC_TRI(y), RSC_TRI(z), RSC_TRI(w));
#undef RSC_TRI
    return r;
}

/* read_imagef on an image2d_t */
__device__ __forceinline__ float4 read_image2d(const Image &im, float u, float v) {
    int i0, i1, j0, j1;
    float a, b;
    tex_axis(u, im.nx, &i0, &i1, &a);
    tex_axis(v, im.ny, &j0, &j1, &b);
    const unsigned sy = (unsigned)im.nx;
    const float4 *d = im.data;
    const unsigned r0 = j0 * sy, r1 = j1 * sy;
    float4 t00 = ldg4(d + (r0 + i0)), t10 = ldg4(d + (r0 + i1));
    float4 t01 = ldg4(d + (r1 + i0)), t11 = ldg4(d + (r1 + i1));
    float ma = 1.0f - a, mb = 1.0f - b;
    float w00 = ma * mb, w10 = a * mb, w01 = ma * b, w11 = a * b;
#define RSC_BIL(L) (w00 * t00.L + w10 * t10.L + w01 * t01.L + w11 * t11.L)
    float4 r = f4(RSC_BIL(x), RSC_BIL(y), RSC_BIL(z), RSC_BIL(w));
#undef RSC_BIL
    return r;
}

/* wind_table_index (rs.cl:123-188), x/y/z lanes */
/* SP >= 0: the descriptor's spacing code (wd[7]) known at compile time */
template <int SP = -1>
__device__ __forceinline__ void wind_table_index(float out[3], float4 pos, const float *wd, const float *sd) {
    const uint32_t spacing = SP >= 0 ? (uint32_t)SP : __float_as_uint(wd[7]);
    if (spacing == 7u) {
        float pr0 = pos.x - (sd[8] + 0.5f * sd[12]);
        float pr1 = pos.y - (sd[9] + 0.5f * sd[13]);
        float pr2 = pos.z - 0.0f;
        out[0] = copysignf(wd[0], pr0) * rsm_log1pf(wd[4] * fabsf(pr0)) + wd[8];
        out[1] = copysignf(wd[1], pr1) * rsm_log1pf(wd[5] * fabsf(pr1)) + wd[9];
        out[2] = copysignf(wd[2], pr2) * rsm_log1pf(wd[6] * fabsf(pr2)) + wd[10];
    } else if (spacing == 0u) {
        out[0] = fmaf(pos.x, wd[0], wd[4]);
        out[1] = fmaf(pos.y, wd[1], wd[5]);
        out[2] = fmaf(pos.z, wd[2], wd[6]);
    } else {
        out[0] = out[1] = out[2] = 0.0f;
    }
}

template <int SP = -1>
__device__ __forceinline__ float4 compute_bg_vel(float4 pos, const PairImage &uvwt, const float *wd, const float *sd) {
    float c[3];
    wind_table_index<SP>(c, pos, wd, sd);
    return read_pair_image3d(uvwt, c[0], c[1], c[2]);
}

/* compute_dudt_dwdt (rs.cl:195-261) */
__device__ __forceinline__ float4 compute_dudt_dwdt(float4 *dwdt, float4 vel, float4 vel_bg, float4 ori,
                                                    const Image &cdimg, const Image &cmimg, const float *ad) {
    float4 ur = f4(vel_bg.x - vel.x, vel_bg.y - vel.y, vel_bg.z - vel.z, vel_bg.w - vel.w);
    float4 u_hat = quat_rotate(normalize4(ur), quat_conj(ori));
    float beta = rsm_acosf(u_hat.x);
    float alpha = rsm_atan2f(u_hat.z, u_hat.y);
    if (alpha < 0.0f) {
        alpha = RSC_PI_F + alpha;
        beta = -beta;
    }
    float cu = fmaf(beta, ad[0], ad[4]);
    float cv = fmaf(alpha, ad[1], ad[5]);
    float4 cd = read_image2d(cdimg, cu, cv);
    float4 cm = read_image2d(cmimg, cu, cv);
    const float Ta = ad[15];
    cd = quat_rotate(cd, ori);
    float ur_norm_sq = ur.x * ur.x + ur.y * ur.y + ur.z * ur.z;
    float tu = Ta * ur_norm_sq;
    float4 dudt = f4(tu * cd.x + 0.0f, tu * cd.y + 0.0f, tu * cd.z + -9.8f, tu * cd.w + 0.0f);
    dwdt->x = ((tu * ad[12]) * cm.x) * RSC_RAD_PER_DEG;
    dwdt->y = ((tu * ad[13]) * cm.y) * RSC_RAD_PER_DEG;
    dwdt->z = ((tu * ad[14]) * cm.z) * RSC_RAD_PER_DEG;
    dwdt->w = ((tu * 0.0f) * cm.w) * RSC_RAD_PER_DEG;
    return dudt;
}

/* compute_ellipsoid_rcs (rs.cl:268-280) */
__device__ __forceinline__ float4 compute_ellipsoid_rcs(float4 pos, const float4 *table, const float *td) {
    float fidx = cl_clamp(fmaf(pos.w, td[0], td[1]), 0.0f, td[2]);
    /* clamped to [0, td[2]] (NaN -> 0), inside the table: the plain
     * truncating conversion is convert_uint's */
    uint32_t idx = (uint32_t)fidx;
    float4 xz = ldg4(table + idx);
    /* cos^2 of the elevation beta = atan2(z, |xy|), formed as |xy|^2 / |xyz|^2:
     * the same quantity as cos(beta) * cos(beta) without the two
     * transcendental calls (1 at the origin, where atan2(0, 0) = 0) */
    const float h2 = pos.x * pos.x + pos.y * pos.y;
    const float r2 = h2 + pos.z * pos.z;
    const float cb2 = r2 > 0.0f ? h2 / r2 : 1.0f;
    return f4(xz.x, xz.y, xz.x + (xz.z - xz.x) * cb2, xz.y + (xz.w - xz.y) * cb2);
}

/* compute_debris_rcs (rs.cl:282-359) */
__device__ __forceinline__ float4 compute_debris_rcs(float4 pos, float4 ori, const Image &re_img, const Image &im_img,
                                                     const float *rd, uint32_t concept) {
    float el = rsm_atan2f(pos.z, sqrtf(pos.x * pos.x + pos.y * pos.y));
    float az = rsm_atan2f(pos.x, pos.y);
    float se, ce, sa, ca;
    rsm_sincosf(0.5f * (el + RSC_PI_2_F), &se, &ce);
    rsm_sincosf(0.5f * (az), &sa, &ca);
    float4 o_conj = f4((-se * ca + ce * sa) * RSC_SQRT1_2_F, (ce * ca + se * sa) * RSC_SQRT1_2_F,
                       (se * ca + ce * sa) * RSC_SQRT1_2_F, (ce * ca + -se * sa) * RSC_SQRT1_2_F);
    float4 R = quat_mult(ori, o_conj);
    float4 q = f4(R.x, R.z, -R.y, R.w);
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
    float4 re = read_image2d(re_img, cu, cv);
    float4 im = read_image2d(im_img, cu, cv);
    float sg, cg;
    rsm_sincosf(gamma, &sg, &cg);
    float hh_real = cg * (cg * re.x - re.z * sg) - sg * (cg * re.z - re.y * sg);
    float hh_imag = cg * (cg * im.x - im.z * sg) - sg * (cg * im.z - im.y * sg);
    float vv_real = cg * (cg * re.y + re.z * sg) + sg * (cg * re.z + re.x * sg);
    float vv_imag = cg * (cg * im.y + im.z * sg) + sg * (cg * im.z + im.x * sg);
    float4 ss = f4(hh_real, hh_imag, vv_real, vv_imag);
    if (concept & kConceptCrossPol) {
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

__device__ __forceinline__ bool is_outside(float4 pos, const float *sd) {
    return (pos.x <= sd[8]) | (pos.y <= sd[9]) | (pos.z <= sd[10]) | (pos.x >= sd[8] + sd[12]) |
           (pos.y >= sd[9] + sd[13]) | (pos.z >= sd[10] + sd[14]);
}

}  // namespace rsc

#endif
