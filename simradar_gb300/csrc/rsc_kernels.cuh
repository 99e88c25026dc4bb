/*
 * rsc_kernels.cuh -- the sm_103a kernels of the emulation loop.
 *
 *   k_advance     one launch per time step: el_atts / bg_atts / fp_atts on the
 *                 background range and db_atts on every debris range
 *                 (rs.cl:533-907), one thread per scatterer, float4 loads.
 *   k_db_rcs      debris RCS refresh after a beam move (rs.cl:909-919).
 *   k_pulse       scat_sig_aux + make_pulse_pass_1 + make_pulse_pass_2
 *                 (rs.cl:1050-1441) fused: each scatterer's signal is formed
 *                 in registers and added only to the gates its range weight
 *                 reaches (the gate weights are the bit-exact pass-1 weights),
 *                 per-warp gate bins in shared memory, one partial per block,
 *                 and the last block to finish sums the partials in block
 *                 order.  Three precisions: plain FP32, compensated FP32
 *                 (double-float range, split phase, double-float sums), FP64.
 *   k_sig_aux     forms aux / sig for RS_download when the pulse kernel did
 *                 not write them.
 */
#ifndef SIMRADAR_GB300_RSC_KERNELS_CUH
#define SIMRADAR_GB300_RSC_KERNELS_CUH

#include "rsc_physics.cuh"

namespace rsc {

constexpr int kAdvanceThreads = 256;
constexpr int kMaxCandidates = 8;

struct DebrisType {
    unsigned long long origin, count;
    Image cd, cm, re, im;
    float adm[16];
    float rcs[16];
};

struct AdvanceArgs {
    float4 *pos, *vel, *ori, *tum, *rcs;
    uint4 *rnd;
    Image uvwt, cpxx;
    float wind[16];
    float sim[16];
    const float4 *drop;
    float drop_desc[4];
    const float *dff;
    float dff_desc[16];
    unsigned long long rain_origin, rain_count;
    int rain_mode; /* 0 bg_atts, 1 el_atts, 2 fp_atts */
    unsigned rain_blocks;
    int ntypes;
    unsigned long long deb_prefix[RSC_MAX_TYPES]; /* cumulative debris counts */
    DebrisType types[RSC_MAX_TYPES - 1];
};

/* ---- el_atts (rs.cl:653-739) ---- */
__device__ __forceinline__ void rain_el(const AdvanceArgs &a, size_t i) {
    const float *sd = a.sim;
    const float dt = sd[11];
    const uint32_t concept = __float_as_uint(sd[5]);
    const float rho_air = 1.225f;
    const float rho_over_mu_air = 6.7308e4f;
    float4 pos = a.pos[i];
    float4 vel = a.vel[i];
    pos.x = fmaf(vel.x, dt, pos.x);
    pos.y = fmaf(vel.y, dt, pos.y);
    pos.z = fmaf(vel.z, dt, pos.z);
    pos.w = fmaf(vel.w, 0.0f, pos.w);
    const float area_over_mass_particle = 0.003006012f / pos.w;
    if (is_outside(pos, sd)) {
        /* respawn: the only time the seed is read or written, and rcs keeps
         * its previous value (el_atts writes x[i] = rcs unchanged) */
        uint4 seed = a.rnd[i];
        float4 r = cl_rand(&seed);
        pos.x = fmaf(r.x, sd[12], sd[8]);
        pos.y = fmaf(r.y, sd[13], sd[9]);
        pos.z = fmaf(r.z, sd[14], sd[10]);
        a.pos[i] = pos;
        a.vel[i] = f4(0.0f, 0.0f, 0.0f, 0.0f);
        a.rnd[i] = seed;
        return;
    }
    float4 bg_vel = compute_bg_vel(pos, a.uvwt, a.wind, sd);
    float4 dv = f4(bg_vel.x - vel.x, bg_vel.y - vel.y, bg_vel.z - vel.z, bg_vel.w - vel.w);
    float dva = len3(dv.x, dv.y, dv.z);
    const float g_dt = -9.8f * dt;
    if (dva > 1.0e-3f) {
        float re = rho_over_mu_air * (2.0f * pos.w) * dva;
        float cd = 24.0f / re + 6.0f / (1.0f + sqrtf(re)) + 0.4f;
        float k = 0.5f * rho_air * cd * area_over_mass_particle * dva;
        float4 dudt = f4(k * dv.x + 0.0f, k * dv.y + 0.0f, k * dv.z + -9.8f, k * dv.w + 0.0f);
        vel.x = vel.x + dudt.x * dt;
        vel.y = vel.y + dudt.y * dt;
        vel.z = vel.z + dudt.z * dt;
        vel.w = vel.w + dudt.w * 0.0f;
        if ((concept & kConceptBounded) && len4(vel) > fmaxf(1.0f, 3.0f * len4(bg_vel))) {
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
    float4 rcs = compute_ellipsoid_rcs(pos, a.drop, a.drop_desc);
    a.pos[i] = pos;
    a.vel[i] = vel;
    a.rcs[i] = rcs;
}

/* ---- bg_atts (rs.cl:533-580) ---- */
__device__ __forceinline__ void rain_bg(const AdvanceArgs &a, size_t i) {
    const float *sd = a.sim;
    const float dt = sd[11];
    float4 pos = a.pos[i];
    float4 vel = a.vel[i];
    pos.x = pos.x + vel.x * dt;
    pos.y = pos.y + vel.y * dt;
    pos.z = pos.z + vel.z * dt;
    pos.w = pos.w + vel.w * 0.0f;
    if (is_outside(pos, sd)) {
        uint4 seed = a.rnd[i];
        float4 r = cl_rand(&seed);
        pos.x = r.x * sd[12] + sd[8];
        pos.y = r.y * sd[13] + sd[9];
        pos.z = r.z * sd[14] + sd[10];
        a.pos[i] = pos;
        a.vel[i] = f4(0.0f, 0.0f, 0.0f, 0.0f);
        a.rnd[i] = seed;
        return;
    }
    vel = compute_bg_vel(pos, a.uvwt, a.wind, sd);
    float4 rcs = compute_ellipsoid_rcs(pos, a.drop, a.drop_desc);
    a.pos[i] = pos;
    a.vel[i] = vel;
    a.rcs[i] = rcs;
}

/* ---- fp_atts (rs.cl:590-648) ---- */
__device__ __forceinline__ void rain_fp(const AdvanceArgs &a, size_t i) {
    const float *sd = a.sim;
    const float wav_num = sd[4];
    const float dt = sd[11];
    float4 pos = a.pos[i];
    float4 vel = a.vel[i];
    float4 rcs = a.rcs[i];
    float c3[3];
    wind_table_index(c3, pos, a.wind, sd);
    float4 uv = read_image3d(a.uvwt, c3[0], c3[1], c3[2]);
    float4 cp = read_image3d(a.cpxx, c3[0], c3[1], c3[2]);
    float l = len3(pos.x, pos.y, pos.z);
    float nx = pos.x / l, ny = pos.y / l, nz = pos.z / l;
    float phi = rcs.w - wav_num * (nx * uv.x + ny * uv.y + nz * uv.z) * dt;
    float cn2 = cp.x;
    float am = rsm_powf(10.0f, cn2);
    float s, c;
    rsm_sincosf(phi, &s, &c);
    rcs.x = am * c;
    rcs.y = am * s;
    rcs.z = cn2;
    rcs.w = rsm_atan2f(s, c);
    vel.x = uv.x;
    vel.y = uv.y;
    vel.z = uv.z;
    a.vel[i] = vel;
    a.rcs[i] = rcs;
}

/* ---- db_atts (rs.cl:744-907) ---- */
__device__ __forceinline__ void debris_step(const AdvanceArgs &a, const DebrisType &T, size_t i) {
    const float *sd = a.sim;
    const uint32_t concept = __float_as_uint(sd[5]);
    const float dt = sd[11];
    float4 pos = a.pos[i];
    float4 ori = a.ori[i];
    float4 vel = a.vel[i];
    float4 tum = a.tum[i];
    ori = normalize4(quat_mult(ori, tum));
    pos.x = pos.x + vel.x * dt;
    pos.y = pos.y + vel.y * dt;
    pos.z = pos.z + vel.z * dt;
    pos.w = pos.w + vel.w * 0.0f;
    if (is_outside(pos, sd)) {
        uint4 seed = a.rnd[i];
        float4 r = cl_rand(&seed);
        if (concept & kConceptDFF) {
            const float *fd = a.dff_desc;
            float fi0, fi1;
            float raw0 = cl_clamp(fmaf(r.x, fd[15], 0.0f), 0.0f, fd[15]);
            float raw1 = cl_clamp(fmaf(r.x, fd[15], 1.0f), 0.0f, fd[15]);
            float dec0 = cl_fract(raw0, &fi0);
            (void)cl_fract(raw1, &fi1);
            float cidx = cl_mix(__ldg(a.dff + cl_f2u_rtz(fi0)), __ldg(a.dff + cl_f2u_rtz(fi1)), dec0);
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
            pos.z = RSC_MIN_HEIGHT;
        } else {
            pos.x = fmaf(r.x, sd[12], sd[8]);
            pos.y = fmaf(r.y, sd[13], sd[9]);
            pos.z = sd[10] + RSC_MIN_HEIGHT;
        }
        r = cl_rand(&seed);
        float4 c = f4(sqrtf(-2.0f * rsm_logf(r.x)), sqrtf(-2.0f * rsm_logf(r.y)), sqrtf(-2.0f * rsm_logf(r.z)), r.w);
        r = cl_rand(&seed);
        c.x = c.x * rsm_cosf(2.0f * RSC_PI_F * r.x);
        c.y = c.y * rsm_cosf(2.0f * RSC_PI_F * r.y);
        c.z = c.z * rsm_cosf(2.0f * RSC_PI_F * r.z);
        float sin_th_2, cos_th_2;
        rsm_sincosf(RSC_PI_F * c.w, &sin_th_2, &cos_th_2);
        float sqxy = sqrtf(c.x * c.x + c.z * c.z);
        float sqxyz = sqrtf(c.x * c.x + c.y * c.y + c.z * c.z);
        float sa, ca;
        rsm_sincosf(0.5f * rsm_acosf(c.y / sqxyz), &sa, &ca);
        ori.x = c.x * ca * sin_th_2 / sqxyz - c.x * c.y * sin_th_2 / sqxyz * sa / sqxy + c.z * cos_th_2 * sa / sqxy;
        ori.y = sin_th_2 / sqxyz * (sqxy * sa + c.y * ca);
        ori.z = c.z * ca * sin_th_2 / sqxyz - c.x * cos_th_2 * sa / sqxy - c.y * c.z * sin_th_2 * sa / sqxy / sqxyz;
        ori.w = cos_th_2 * ca;
        a.pos[i] = pos;
        a.ori[i] = ori;
        a.vel[i] = f4(0.0f, 0.0f, 0.0f, 0.0f);
        a.tum[i] = f4(0.0f, 0.0f, 0.0f, 1.0f);
        a.rcs[i] = f4(0.0f, 0.0f, 0.0f, 0.0f);
        a.rnd[i] = seed;
        return;
    }
    float4 vel_bg = compute_bg_vel(pos, a.uvwt, a.wind, sd);
    float4 dwdt;
    float4 dudt = compute_dudt_dwdt(&dwdt, vel, vel_bg, ori, T.cd, T.cm, T.adm);
    if ((concept & kConceptBounded) &&
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
    float s0, c0, s1, c1, s2, c2;
    rsm_sincosf(dwdt.x * dt, &s0, &c0);
    rsm_sincosf(dwdt.y * dt, &s1, &c1);
    rsm_sincosf(dwdt.z * dt, &s2, &c2);
    tum = f4(c0 * s1 * s2 + s0 * c1 * c2, c0 * s1 * c2 - s0 * c1 * s2, c0 * c1 * s2 + s0 * s1 * c2,
             c0 * c1 * c2 - s0 * s1 * s2);
    tum = normalize4(tum);
    float4 rcs = compute_debris_rcs(pos, ori, T.re, T.im, T.rcs, concept);
    a.pos[i] = pos;
    a.ori[i] = ori;
    a.vel[i] = vel;
    a.tum[i] = tum;
    a.rcs[i] = rcs;
}

__device__ __forceinline__ int debris_type_of(const AdvanceArgs &a, unsigned long long j) {
    int t = 0;
#pragma unroll
    for (int k = 1; k < RSC_MAX_TYPES - 1; k++) {
        if (k < a.ntypes && j >= a.deb_prefix[k]) t = k;
    }
    return t;
}

__global__ void __launch_bounds__(kAdvanceThreads) k_advance(const AdvanceArgs a) {
    const unsigned b = blockIdx.x;
    if (b < a.rain_blocks) {
        unsigned long long j = (unsigned long long)b * kAdvanceThreads + threadIdx.x;
        if (j >= a.rain_count) return;
        size_t i = (size_t)(a.rain_origin + j);
        if (a.rain_mode == 1) {
            rain_el(a, i);
        } else if (a.rain_mode == 0) {
            rain_bg(a, i);
        } else {
            rain_fp(a, i);
        }
        return;
    }
    unsigned long long j = (unsigned long long)(b - a.rain_blocks) * kAdvanceThreads + threadIdx.x;
    if (a.ntypes == 0 || j >= a.deb_prefix[a.ntypes]) return;
    int t = debris_type_of(a, j);
    const DebrisType &T = a.types[t];
    debris_step(a, T, (size_t)(T.origin + (j - a.deb_prefix[t])));
}

/* ---- db_rcs (rs.cl:909-919) for every debris type ---- */
__global__ void __launch_bounds__(kAdvanceThreads) k_db_rcs(const AdvanceArgs a) {
    unsigned long long j = (unsigned long long)blockIdx.x * kAdvanceThreads + threadIdx.x;
    if (a.ntypes == 0 || j >= a.deb_prefix[a.ntypes]) return;
    int t = debris_type_of(a, j);
    const DebrisType &T = a.types[t];
    size_t i = (size_t)(T.origin + (j - a.deb_prefix[t]));
    a.rcs[i] = compute_debris_rcs(a.pos[i], a.ori[i], T.re, T.im, T.rcs, __float_as_uint(a.sim[5]));
}

/* ====================== pulse formation ====================== */

struct PulseArgs {
    const float4 *pos, *rcs;
    float4 *aux, *sig;
    unsigned long long n;
    const float *aw;
    float awd[4];
    const float *rw;
    float rwd[4];
    const float *rk;     /* gate origins: FP32 running sum (plain), FP64 head (compensated) */
    const float *rk_lo;  /* FP64 tail (compensated) */
    const double *rk64;  /* FP64 (F64 mode) */
    unsigned G;
    float sim[16];
    float rs, inv_delta, win_lo, win_hi;
    int dense;
    int materialize;
    void *partials;      /* gridDim.x * G * 4 accumulators (x2 for double-float) */
    unsigned *counter;
    float4 *pulse;
    double *pulse64;
};

/* the pass-1 weight of one gate (rs.cl:1196-1209), bit-exact */
__device__ __forceinline__ float range_weight(const PulseArgs &P, float d) {
    float f0, f1;
    float dec0 = cl_fract(cl_clamp(fmaf(d, P.rwd[0], P.rwd[1] + 0.0f), 0.0f, P.rwd[2]), &f0);
    (void)cl_fract(cl_clamp(fmaf(d, P.rwd[0], P.rwd[1] + 1.0f), 0.0f, P.rwd[2]), &f1);
    return cl_mix(__ldg(P.rw + cl_f2u_rtz(f0)), __ldg(P.rw + cl_f2u_rtz(f1)), dec0);
}

/* the angular weight of scat_sig_aux (rs.cl:1066-1089) */
__device__ __forceinline__ float angular_weight(const PulseArgs &P, float angle) {
    float fi0, fi1;
    float raw0 = cl_clamp(fmaf(angle, P.awd[0], P.awd[1] + 0.0f), 0.0f, P.awd[2]);
    float raw1 = cl_clamp(fmaf(angle, P.awd[0], P.awd[1] + 1.0f), 0.0f, P.awd[2]);
    float dec0 = cl_fract(raw0, &fi0);
    (void)cl_fract(raw1, &fi1);
    return cl_mix(__ldg(P.aw + cl_f2u_rtz(fi0)), __ldg(P.aw + cl_f2u_rtz(fi1)), dec0);
}

/* error-free transformations */
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
    p = a * b;
    e = fmaf(a, b, -p);
}

/* accumulators: per-warp gate bins in shared memory */
struct AccF32 {
    typedef float bin_t;
    static constexpr int kWords = 1;
    float v[4];
    __device__ void set(float a, float b, float c, float d) { v[0] = a; v[1] = b; v[2] = c; v[3] = d; }
    __device__ void scale(float w, AccF32 &o) const { o.set(w * v[0], w * v[1], w * v[2], w * v[3]); }
    __device__ static void add_to(float *bin, const AccF32 &c) {
        bin[0] = bin[0] + c.v[0];
        bin[1] = bin[1] + c.v[1];
        bin[2] = bin[2] + c.v[2];
        bin[3] = bin[3] + c.v[3];
    }
};

/* double-float bin: 4 heads then 4 tails */
struct AccDF {
    typedef float bin_t;
    static constexpr int kWords = 2;
    float v[4];
    __device__ void set(float a, float b, float c, float d) { v[0] = a; v[1] = b; v[2] = c; v[3] = d; }
    __device__ void scale(float w, AccDF &o) const { o.set(w * v[0], w * v[1], w * v[2], w * v[3]); }
    __device__ static void add_to(float *bin, const AccDF &c) {
#pragma unroll
        for (int l = 0; l < 4; l++) {
            float s, e;
            two_sum(bin[l], c.v[l], s, e);
            bin[l] = s;
            bin[4 + l] = bin[4 + l] + e;
        }
    }
};

struct AccF64 {
    typedef double bin_t;
    static constexpr int kWords = 1;
    double v[4];
    __device__ void set(double a, double b, double c, double d) { v[0] = a; v[1] = b; v[2] = c; v[3] = d; }
    __device__ void scale(double w, AccF64 &o) const { o.set(w * v[0], w * v[1], w * v[2], w * v[3]); }
    __device__ static void add_to(double *bin, const AccF64 &c) {
        bin[0] = bin[0] + c.v[0];
        bin[1] = bin[1] + c.v[1];
        bin[2] = bin[2] + c.v[2];
        bin[3] = bin[3] + c.v[3];
    }
};

/* Add `c` to this warp's bin `gate`.  Lanes of the warp that address the same
 * gate are serialised in lane order (__match_any_sync), so every bin sees its
 * additions in a fixed order and the pulse is bit-reproducible run to run. */
template <class Acc>
__device__ __forceinline__ void bin_add(typename Acc::bin_t *wbins, unsigned active, bool valid, int gate,
                                        const Acc &c) {
    unsigned vmask = __ballot_sync(active, valid);
    if (!valid) return;
    const unsigned lane = threadIdx.x & 31u;
    unsigned peers = __match_any_sync(vmask, gate);
    int rank = __popc(peers & ((1u << lane) - 1u));
    int size = __popc(peers);
    typename Acc::bin_t *bin = wbins + (size_t)gate * 4 * Acc::kWords;
    for (int t = 0; t < size; t++) {
        if (t == rank) Acc::add_to(bin, c);
        __syncwarp(peers);
    }
}

/* warp-wide sum of one contribution per lane (fixed shuffle tree), added by
 * lane 0 to a bin of this warp */
template <class Acc>
__device__ __forceinline__ void warp_sum_into(typename Acc::bin_t *bin, Acc c) {
    if constexpr (Acc::kWords == 2) {
        float lo[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
            for (int l = 0; l < 4; l++) {
                float oh = __shfl_down_sync(0xffffffffu, c.v[l], off);
                float ol = __shfl_down_sync(0xffffffffu, lo[l], off);
                float s, e;
                two_sum(c.v[l], oh, s, e);
                c.v[l] = s;
                lo[l] = lo[l] + (e + ol);
            }
        }
        if ((threadIdx.x & 31u) == 0) {
#pragma unroll
            for (int l = 0; l < 4; l++) {
                float s, e;
                two_sum(bin[l], c.v[l], s, e);
                bin[l] = s;
                bin[4 + l] = bin[4 + l] + (e + lo[l]);
            }
        }
    } else {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
            for (int l = 0; l < 4; l++) c.v[l] = c.v[l] + __shfl_down_sync(0xffffffffu, c.v[l], off);
        }
        if ((threadIdx.x & 31u) == 0) Acc::add_to(bin, c);
    }
}

/* per-scatterer signal in the three precisions; returns false for a
 * scatterer whose signal or range is not finite (handled on the dense path) */
struct Sig32 {
    float r, g;          /* range and fractional gate position */
    float r_lo;          /* compensated: tail of the range */
    AccF32 s;            /* sig * angular weight */
    float sig[4];        /* sig before the angular weight (for aux/sig output) */
    float wang;
};

__device__ __forceinline__ void signal_plain(const PulseArgs &P, float4 p, float4 x, Sig32 &o) {
    const float *sd = P.sim;
    float l = len3(p.x, p.y, p.z);
    float nx = p.x / l, ny = p.y / l, nz = p.z / l;
    float angle = rsm_acosf(sd[0] * nx + sd[1] * ny + sd[2] * nz);
    o.wang = angular_weight(P, angle);
    float r = len3(p.x, p.y, p.z);
    float atten = 1.0f / (r * r);
    float phase = r * sd[4];
    float ss, cc;
    rsm_sincosf(phase, &ss, &cc);
    float ms = -ss;
    o.sig[0] = (x.x * cc - x.y * ms) * atten;
    o.sig[1] = (x.y * cc + x.x * ms) * atten;
    o.sig[2] = (x.z * cc - x.w * ms) * atten;
    o.sig[3] = (x.w * cc + x.z * ms) * atten;
    o.s.set(o.sig[0] * o.wang, o.sig[1] * o.wang, o.sig[2] * o.wang, o.sig[3] * o.wang);
    o.r = r;
    o.r_lo = 0.0f;
}

/* compensated: range as a double-float from the FP32 position, angle from a
 * well-conditioned atan2(|b x p|, b . p), phase k r reduced by pi/2 with the
 * product k * r_hi split exactly (fmaf) and the tails added after reduction */
__device__ __forceinline__ void signal_comp(const PulseArgs &P, float4 p, float4 x, Sig32 &o) {
    const float *sd = P.sim;
    float ax, ex, ay, ey, az, ez;
    two_prod(p.x, p.x, ax, ex);
    two_prod(p.y, p.y, ay, ey);
    two_prod(p.z, p.z, az, ez);
    float s1, e1, s2, e2;
    two_sum(ax, ay, s1, e1);
    two_sum(s1, az, s2, e2);
    float lo = ((ex + ey) + ez) + (e1 + e2);
    float sh = s2 + lo;
    float sl = lo - (sh - s2);
    float rh = sqrtf(sh);
    float rl = (fmaf(-rh, rh, sh) + sl) / (2.0f * rh);
    float r = rh + rl;
    float r_lo = rl - (r - rh);
    /* b x p with each product difference computed with one rounding */
    const float bx = sd[0], by = sd[1], bz = sd[2];
    float t, e;
    two_prod(bz, p.y, t, e);
    float cx = fmaf(by, p.z, -t) - e;
    two_prod(bx, p.z, t, e);
    float cy = fmaf(bz, p.x, -t) - e;
    two_prod(by, p.x, t, e);
    float cz = fmaf(bx, p.y, -t) - e;
    float cn = sqrtf(cx * cx + cy * cy + cz * cz);
    float dt = fmaf(bx, p.x, fmaf(by, p.y, bz * p.z));
    float angle = rsm_atan2f(cn, dt);
    o.wang = angular_weight(P, angle);
    /* phase */
    float ph, pl;
    two_prod(sd[4], r, ph, pl);
    pl = fmaf(sd[4], r_lo, pl);
    float q;
    float red = rsm_reduce_pio2(ph, &q);
    red = red + pl;
    float ss, cc;
    rsm_sincos_reduced(red, q, &ss, &cc);
    float atten = 1.0f / (r * r);
    float ms = -ss;
    o.sig[0] = (x.x * cc - x.y * ms) * atten;
    o.sig[1] = (x.y * cc + x.x * ms) * atten;
    o.sig[2] = (x.z * cc - x.w * ms) * atten;
    o.sig[3] = (x.w * cc + x.z * ms) * atten;
    o.s.set(o.sig[0] * o.wang, o.sig[1] * o.wang, o.sig[2] * o.wang, o.sig[3] * o.wang);
    o.r = r;
    o.r_lo = r_lo;
}

__device__ __forceinline__ bool finite4(const float *v) {
    return fabsf(v[0]) < INFINITY && fabsf(v[1]) < INFINITY && fabsf(v[2]) < INFINITY && fabsf(v[3]) < INFINITY;
}

/* lerp of a float table at a double index (FP64 oracle) */
__device__ __forceinline__ double lerp64(const float *W, const float *desc, double x) {
    double f = (double)desc[0] * x + (double)desc[1];
    double m = (double)desc[2];
    f = fmin(fmax(f, 0.0), m);
    double fl = floor(f);
    double a = f - fl;
    int i0 = (int)fl;
    int i1 = (fl + 1.0 > m) ? (int)m : i0 + 1;
    double w0 = (double)__ldg(W + i0), w1 = (double)__ldg(W + i1);
    return w0 + (w1 - w0) * a;
}

template <int MODE>  /* RSC_PULSE_PLAIN, RSC_PULSE_COMPENSATED, RSC_PULSE_F64 */
struct PulseTraits;
template <> struct PulseTraits<0> { typedef AccF32 Acc; };
template <> struct PulseTraits<1> { typedef AccDF Acc; };
template <> struct PulseTraits<2> { typedef AccF64 Acc; };

template <int MODE>
__global__ void __launch_bounds__(512) k_pulse(const PulseArgs P) {
    typedef typename PulseTraits<MODE>::Acc Acc;
    typedef typename Acc::bin_t bin_t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned G = P.G;
    const unsigned words = G * 4 * Acc::kWords;          /* bin_t per warp */
    const unsigned nwarps = blockDim.x >> 5;
    const unsigned warp = threadIdx.x >> 5;
    const unsigned lane = threadIdx.x & 31u;
    bin_t *bins = reinterpret_cast<bin_t *>(smem_raw);
    float *rk_s = reinterpret_cast<float *>(bins + (size_t)nwarps * words);
    float *rkl_s = rk_s + G;
    for (unsigned t = threadIdx.x; t < nwarps * words; t += blockDim.x) bins[t] = (bin_t)0;
    for (unsigned t = threadIdx.x; t < G; t += blockDim.x) {
        rk_s[t] = P.rk[t];
        rkl_s[t] = (MODE == 1) ? P.rk_lo[t] : 0.0f;
    }
    __syncthreads();
    bin_t *wbins = bins + (size_t)warp * words;

    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long n = P.n;
    /* every lane of a warp runs the same number of iterations so the warp
     * collectives below see the full warp */
    const unsigned long long base0 = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
    for (unsigned long long base = base0; base < n; base += stride) {
        const unsigned long long i = base + lane;
        const bool in = i < n;
        Acc c;
        float r = 0.0f, r_lo = 0.0f;
        double r64 = 0.0;
        bool finite = false;
        if (in) {
            float4 p = __ldg(P.pos + i);
            float4 x = __ldg(P.rcs + i);
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
        if (!P.dense) {
            /* candidate gates: only those the range weight can reach */
            int k_lo = 0, k_hi = -1;
            if (in && finite) {
                float g = (r - P.rs) * P.inv_delta;
                k_lo = max(0, (int)ceilf(fminf(fmaxf(g - P.win_hi, -1.0f), (float)G)));
                k_hi = min((int)G - 1, (int)floorf(fminf(g - P.win_lo, (float)G)));
            }
            const int maxc = min(kMaxCandidates, (int)__reduce_max_sync(0xffffffffu, (unsigned)max(k_hi - k_lo + 1, 0)));
            for (int j = 0; j < maxc; j++) {
                const int gate = k_lo + j;
                bool valid = gate <= k_hi;
                Acc cw;
                if (valid) {
                    if constexpr (MODE == 2) {
                        double w = lerp64(P.rw, P.rwd, r64 - P.rk64[gate]);
                        c.scale(w, cw);
                        valid = (w != 0.0);
                    } else {
                        float d = (MODE == 1) ? (r - rk_s[gate]) + (r_lo - rkl_s[gate]) : r - rk_s[gate];
                        float w = range_weight(P, d);
                        c.scale(w, cw);
                        valid = (w != 0.0f);
                    }
                }
                bin_add<Acc>(wbins, 0xffffffffu, valid, gate, cw);
            }
            /* a non-finite signal meets every gate (0 * inf = NaN in pass 1) */
            if (__any_sync(0xffffffffu, in && !finite)) {
                for (unsigned k = 0; k < G; k++) {
                    bool valid = in && !finite;
                    Acc cw;
                    if (valid) {
                        if constexpr (MODE == 2) {
                            c.scale(lerp64(P.rw, P.rwd, r64 - P.rk64[k]), cw);
                        } else {
                            c.scale(range_weight(P, r - rk_s[k]), cw);
                        }
                    }
                    bin_add<Acc>(wbins, 0xffffffffu, valid, (int)k, cw);
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
                    } else {
                        float d = (MODE == 1) ? (r - rk_s[k]) + (r_lo - rkl_s[k]) : r - rk_s[k];
                        c.scale(range_weight(P, d), cw);
                    }
                }
                warp_sum_into<Acc>(wbins + (size_t)k * 4 * Acc::kWords, cw);
            }
        }
    }
    __syncthreads();

    /* block partial: warp bins summed in warp order */
    const unsigned outs = G * 4;
    bin_t *part = reinterpret_cast<bin_t *>(P.partials) + (size_t)blockIdx.x * outs * Acc::kWords;
    for (unsigned o = threadIdx.x; o < outs; o += blockDim.x) {
        const unsigned k = o >> 2, l = o & 3u;
        if (Acc::kWords == 2) {
            float hi = 0.0f, lo = 0.0f;
            for (unsigned wv = 0; wv < nwarps; wv++) {
                const float *b = reinterpret_cast<const float *>(bins) + (size_t)wv * words + k * 8;
                float s, e;
                two_sum(hi, b[l], s, e);
                hi = s;
                lo = lo + (e + b[4 + l]);
            }
            reinterpret_cast<float *>(part)[o] = hi;
            reinterpret_cast<float *>(part)[outs + o] = lo;
        } else {
            bin_t acc = (bin_t)0;
            for (unsigned wv = 0; wv < nwarps; wv++) acc = acc + bins[(size_t)wv * words + o];
            part[o] = acc;
        }
    }
    __threadfence();
    __syncthreads();
    __shared__ bool s_last;
    if (threadIdx.x == 0) {
        unsigned ticket = atomicAdd(P.counter, 1u);
        s_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    /* last block: sum the block partials in block order; warp w takes
     * outputs w, w + nwarps, ...; lanes stride over blocks, then a fixed
     * shuffle tree */
    const unsigned nb = gridDim.x;
    for (unsigned o = warp; o < outs; o += nwarps) {
        if (Acc::kWords == 2) {
            const float *pf = reinterpret_cast<const float *>(P.partials);
            float hi = 0.0f, lo = 0.0f;
            for (unsigned b = lane; b < nb; b += 32) {
                const float *pb = pf + (size_t)b * outs * 2;
                float s, e;
                two_sum(hi, __ldcg(pb + o), s, e);
                hi = s;
                lo = lo + (e + __ldcg(pb + outs + o));
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                float ohi = __shfl_down_sync(0xffffffffu, hi, off);
                float olo = __shfl_down_sync(0xffffffffu, lo, off);
                float s, e;
                two_sum(hi, ohi, s, e);
                hi = s;
                lo = lo + (e + olo);
            }
            if (lane == 0) reinterpret_cast<float *>(P.pulse)[o] = hi + lo;
        } else {
            const bin_t *pf = reinterpret_cast<const bin_t *>(P.partials);
            bin_t acc = (bin_t)0;
            for (unsigned b = lane; b < nb; b += 32) acc = acc + __ldcg(pf + (size_t)b * outs + o);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) acc = acc + __shfl_down_sync(0xffffffffu, acc, off);
            if (lane == 0) {
                reinterpret_cast<float *>(P.pulse)[o] = (float)acc;
                if (MODE == 2) P.pulse64[o] = (double)acc;
            }
        }
    }
    if (threadIdx.x == 0) *P.counter = 0u;
}

/* scat_sig_aux (rs.cl:1050-1110) for RS_download */
__global__ void __launch_bounds__(256) k_sig_aux(const PulseArgs P) {
    unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    Sig32 sg;
    signal_plain(P, P.pos[i], P.rcs[i], sg);
    float4 ax = P.aux[i];
    ax.x = sg.r;
    ax.y = ax.y + P.sim[15];
    ax.w = sg.wang;
    P.aux[i] = ax;
    P.sig[i] = make_float4(sg.sig[0], sg.sig[1], sg.sig[2], sg.sig[3]);
}

/* diagnostics */
__global__ void k_eval_math(int fn, const float *a, const float *b, float *out, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
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
        default: out[i] = 0.0f; break;
    }
}

}  // namespace rsc

#endif
