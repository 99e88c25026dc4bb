/*
 * rsc_kernels.cuh -- the sm_103a kernels of the emulation loop.
 *
 *   k_advance_rain    one time step of the background range: el_atts /
 *                     bg_atts / fp_atts (rs.cl:533-739), one thread per
 *                     scatterer, float4 loads, the kernel chosen by concept.
 *   k_advance_debris  db_atts on every debris range (rs.cl:744-907) in one
 *                     launch, run beside the background kernel.
 *   k_db_rcs      debris RCS refresh after a beam move (rs.cl:909-919).
 *   k_sig_aux     forms aux / sig for RS_download when the pulse kernel did
 *                 not write them.
 *   k_les_remap   scales an LES frame's raw planes into a uvwt / cpxx slot.
 *   k_les_pairs   puts a uvwt volume into the slot's x-pair layout.
 * plus the pieces the pulse kernel (rsc_pulse.cuh) is built from: the
 * pass-1 weights, the per-scatterer signal and the per-warp gate bins.
 */
#ifndef SIMRADAR_GB300_RSC_KERNELS_CUH
#define SIMRADAR_GB300_RSC_KERNELS_CUH

#include "rsc_physics.cuh"

namespace rsc {

constexpr int kAdvanceThreads = 128;
constexpr int kMaxCandidates = 8;

struct DebrisType {
    unsigned long long origin, count;
    Image cd, cm, re, im;
    float adm[16];
    float rcs[16];
};

struct AdvanceArgs {
    /* pos and rcs are read from pos_in / rcs_in and written to pos / rcs:
     * the same arrays in place, or the worker's second pair so that the
     * pulse of the same step can read the first pair meanwhile */
    const float4 *pos_in, *rcs_in;
    float4 *pos, *vel, *ori, *tum, *rcs;
    uint4 *rnd;
    PairImage uvwt;
    Image cpxx;
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

/* What one background step makes of a scatterer, formed before anything is
 * stored, so that a thread can carry two scatterers' dependent load chains
 * (state, then LES texels) at once.  On a respawn `rcs` is the stored
 * backscatter, which the step keeps. */
struct RainNext {
    float4 pos, vel, rcs;
    uint4 seed;
    bool respawn;
};

__device__ __forceinline__ void rain_store(const AdvanceArgs &a, size_t i, const RainNext &o) {
    a.pos[i] = o.pos;
    a.vel[i] = o.vel;
    if (o.respawn) {
        /* the only time the seed is written; rcs keeps its previous value */
        a.rnd[i] = o.seed;
        if (a.rcs != a.rcs_in) a.rcs[i] = o.rcs;
    } else {
        a.rcs[i] = o.rcs;
    }
}

/* respawn (rs.cl:546-556, rs.cl:668-678): the only time the seed is read */
template <bool FMA>
__device__ __forceinline__ void rain_respawn(const AdvanceArgs &a, size_t i, const float *sd, RainNext &o) {
    uint4 seed = a.rnd[i];
    float4 r = cl_rand(&seed);
    if (FMA) {
        o.pos.x = fmaf(r.x, sd[12], sd[8]);
        o.pos.y = fmaf(r.y, sd[13], sd[9]);
        o.pos.z = fmaf(r.z, sd[14], sd[10]);
    } else {
        o.pos.x = r.x * sd[12] + sd[8];
        o.pos.y = r.y * sd[13] + sd[9];
        o.pos.z = r.z * sd[14] + sd[10];
    }
    o.vel = f4(0.0f, 0.0f, 0.0f, 0.0f);
    o.seed = seed;
    o.rcs = a.rcs_in[i];
    o.respawn = true;
}

/* ---- el_atts (rs.cl:653-739) ---- */
template <int SP = -1>
__device__ __forceinline__ void rain_el_next(const AdvanceArgs &a, size_t i, RainNext &o) {
    const float *sd = a.sim;
    const float dt = sd[11];
    const uint32_t concept = __float_as_uint(sd[5]);
    const float rho_air = 1.225f;
    const float rho_over_mu_air = 6.7308e4f;
    float4 pos = a.pos_in[i];
    float4 vel = a.vel[i];
    pos.x = fmaf(vel.x, dt, pos.x);
    pos.y = fmaf(vel.y, dt, pos.y);
    pos.z = fmaf(vel.z, dt, pos.z);
    pos.w = fmaf(vel.w, 0.0f, pos.w);
    const float area_over_mass_particle = 0.003006012f / pos.w;
    o.pos = pos;
    if (is_outside(pos, sd)) {
        rain_respawn<true>(a, i, sd, o);
        return;
    }
    float4 bg_vel = compute_bg_vel<SP>(pos, a.uvwt, a.wind, sd);
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
        if ((concept & kConceptBounded) && len4_exceeds_bound(vel, bg_vel)) {
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
    o.vel = vel;
    o.rcs = compute_ellipsoid_rcs(pos, a.drop, a.drop_desc);
    o.respawn = false;
}

/* ---- bg_atts (rs.cl:533-580) ---- */
template <int SP = -1>
__device__ __forceinline__ void rain_bg_next(const AdvanceArgs &a, size_t i, RainNext &o) {
    const float *sd = a.sim;
    const float dt = sd[11];
    float4 pos = a.pos_in[i];
    float4 vel = a.vel[i];
    pos.x = pos.x + vel.x * dt;
    pos.y = pos.y + vel.y * dt;
    pos.z = pos.z + vel.z * dt;
    pos.w = pos.w + vel.w * 0.0f;
    o.pos = pos;
    if (is_outside(pos, sd)) {
        rain_respawn<false>(a, i, sd, o);
        return;
    }
    o.vel = compute_bg_vel<SP>(pos, a.uvwt, a.wind, sd);
    o.rcs = compute_ellipsoid_rcs(pos, a.drop, a.drop_desc);
    o.respawn = false;
}

/* The background step of scatterer i, stored; its new position and
 * backscatter returned (xk false on a respawn, where xo is the kept one). */
template <int SP = -1>
__device__ __forceinline__ void rain_el(const AdvanceArgs &a, size_t i, float4 &po, float4 &xo, bool &xk) {
    RainNext o;
    rain_el_next<SP>(a, i, o);
    rain_store(a, i, o);
    po = o.pos;
    xo = o.rcs;
    xk = !o.respawn;
}

template <int SP = -1>
__device__ __forceinline__ void rain_bg(const AdvanceArgs &a, size_t i, float4 &po, float4 &xo, bool &xk) {
    RainNext o;
    rain_bg_next<SP>(a, i, o);
    rain_store(a, i, o);
    po = o.pos;
    xo = o.rcs;
    xk = !o.respawn;
}

/* ---- fp_atts (rs.cl:590-648) ---- */
__device__ __forceinline__ void rain_fp(const AdvanceArgs &a, size_t i, float4 &po, float4 &xo, bool &xk) {
    const float *sd = a.sim;
    const float wav_num = sd[4];
    const float dt = sd[11];
    float4 pos = a.pos_in[i];
    float4 vel = a.vel[i];
    float4 rcs = a.rcs_in[i];
    float c3[3];
    wind_table_index(c3, pos, a.wind, sd);
    float4 uv = read_pair_image3d(a.uvwt, c3[0], c3[1], c3[2]);
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
    if (a.pos != a.pos_in) a.pos[i] = pos;   /* fp_atts leaves the position */
    po = pos;
    xo = rcs;
    xk = true;
}

/* ---- db_atts (rs.cl:744-907) ---- */
__device__ __forceinline__ void debris_step(const AdvanceArgs &a, const DebrisType &T, size_t i, float4 &po, float4 &xo, bool &xk) {
    const float *sd = a.sim;
    const uint32_t concept = __float_as_uint(sd[5]);
    const float dt = sd[11];
    float4 pos = a.pos_in[i];
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
        po = pos;
        xo = f4(0.0f, 0.0f, 0.0f, 0.0f);
        xk = true;
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
    po = pos;
    xo = rcs;
    xk = true;
}

__device__ __forceinline__ int debris_type_of(const AdvanceArgs &a, unsigned long long j) {
    int t = 0;
#pragma unroll
    for (int k = 1; k < RSC_MAX_TYPES - 1; k++) {
        if (k < a.ntypes && j >= a.deb_prefix[k]) t = k;
    }
    return t;
}

/* One scatterer of block b of a time step (blocks [0, rain_blocks) take the
 * background, the rest the debris types in order): advanced in memory, and
 * its new position and backscatter returned for a pulse formed in the same
 * pass.  False when the thread has no scatterer. */
template <int RAIN_MODE>   /* 0 bg_atts, 1 el_atts, 2 fp_atts, -1 chosen by a.rain_mode */
__device__ __forceinline__ bool advance_one_t(const AdvanceArgs &a, unsigned b, unsigned long long &i_out,
                                              float4 &pos, float4 &rcs) {
    bool known = true;
    if (b < a.rain_blocks) {
        unsigned long long j = (unsigned long long)b * kAdvanceThreads + threadIdx.x;
        if (j >= a.rain_count) return false;
        size_t i = (size_t)(a.rain_origin + j);
        const int mode = RAIN_MODE >= 0 ? RAIN_MODE : a.rain_mode;
        if (mode == 1) {
            rain_el(a, i, pos, rcs, known);
        } else if (mode == 0) {
            rain_bg(a, i, pos, rcs, known);
        } else {
            rain_fp(a, i, pos, rcs, known);
        }
        i_out = i;
        return true;
    }
    unsigned long long j = (unsigned long long)(b - a.rain_blocks) * kAdvanceThreads + threadIdx.x;
    if (a.ntypes == 0 || j >= a.deb_prefix[a.ntypes]) return false;
    int t = debris_type_of(a, j);
    const DebrisType &T = a.types[t];
    size_t i = (size_t)(T.origin + (j - a.deb_prefix[t]));
    debris_step(a, T, i, pos, rcs, known);
    i_out = i;
    return true;
}

__device__ __forceinline__ bool advance_one(const AdvanceArgs &a, unsigned b, unsigned long long &i_out, float4 &pos,
                                            float4 &rcs) {
    return advance_one_t<-1>(a, b, i_out, pos, rcs);
}

/* One time step as two kernels: the background kernel holds only its own
 * (short) path, which the debris path's code slows by about a tenth when both
 * share one kernel; the host runs the debris kernel beside it on a second,
 * high-priority stream.  16 blocks of 128 per SM (32 registers, a few bytes
 * spilled in el_atts): the step is a chain of dependent loads (state, then
 * the LES texel pairs), so resident warps are what hides the latency (2.4%
 * faster per step than 6 blocks of 256 at 40 registers), and blocks of 128
 * fill the SM slots the pulse of the same step leaves another 2.3% faster
 * than blocks of 256.  The fused step kernel takes both paths through
 * advance_one. */
template <int RAIN_MODE, int SP = -1>   /* SP: the LES spacing code, when known (7 stretched) */
__global__ void __launch_bounds__(kAdvanceThreads, 2048 / kAdvanceThreads) k_advance_rain(const AdvanceArgs a) {
    const unsigned long long j = (unsigned long long)blockIdx.x * kAdvanceThreads + threadIdx.x;
    if (j >= a.rain_count) return;
    const size_t i = (size_t)(a.rain_origin + j);
    float4 pos, rcs;
    bool known;
    if (RAIN_MODE == 1) {
        rain_el<SP>(a, i, pos, rcs, known);
    } else if (RAIN_MODE == 0) {
        rain_bg<SP>(a, i, pos, rcs, known);
    } else {
        rain_fp(a, i, pos, rcs, known);
    }
}

/* The same step with two scatterers per thread (j and j + 128 of a block of
 * 256 scatterers): both are formed before either is stored, so the loads of
 * the two dependent chains overlap in one thread.  el_atts / bg_atts only. */
template <int RAIN_MODE, int SP = -1>
__global__ void __launch_bounds__(kAdvanceThreads, 1024 / kAdvanceThreads) k_advance_rain2(const AdvanceArgs a) {
    static_assert(RAIN_MODE == 0 || RAIN_MODE == 1, "el_atts / bg_atts");
    const unsigned long long j0 = (unsigned long long)blockIdx.x * (2 * kAdvanceThreads) + threadIdx.x;
    RainNext o[2];
    bool in[2];
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const unsigned long long j = j0 + (unsigned long long)q * kAdvanceThreads;
        in[q] = j < a.rain_count;
        if (in[q]) {
            if (RAIN_MODE == 1) {
                rain_el_next<SP>(a, (size_t)(a.rain_origin + j), o[q]);
            } else {
                rain_bg_next<SP>(a, (size_t)(a.rain_origin + j), o[q]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 2; q++) {
        if (in[q]) rain_store(a, (size_t)(a.rain_origin + j0 + (unsigned long long)q * kAdvanceThreads), o[q]);
    }
}

__global__ void __launch_bounds__(kAdvanceThreads) k_advance_debris(const AdvanceArgs a) {
    const unsigned long long j = (unsigned long long)blockIdx.x * kAdvanceThreads + threadIdx.x;
    if (a.ntypes == 0 || j >= a.deb_prefix[a.ntypes]) return;
    const int t = debris_type_of(a, j);
    const DebrisType &T = a.types[t];
    float4 pos, rcs;
    bool known;
    debris_step(a, T, (size_t)(T.origin + (j - a.deb_prefix[t])), pos, rcs, known);
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
    float bn_hi, bn_lo;  /* |beam| of sim[0..2] as a double-float (compensated form) */
    float rs, inv_delta, win_lo, win_hi;
    float rdelta;        /* gate spacing: the running sum's increment */
    unsigned rw_n;       /* range weight table length; <= 4 is kept in rwv */
    float rwv[4];
    int rw_tri;          /* the table is the triangle {0, 1, 0} with origin 1 and max 2 */
    int dense;
    int coherent_span;   /* warp-coherent gate path when a warp spans fewer gates */
    int materialize;
    int mom_n;           /* compensated form on the triangle whose support is mom_n gate spacings: terms
                          * summed per range interval as moments (PulseBins::add_k), 0 otherwise */
    double *acc64;       /* G * 4 FP64 accumulators, zero between launches */
    unsigned *counter;
    unsigned long long *runs;   /* the grouped compensated pulse's run counter, zero between launches (or null) */
    float4 *pulse;
    double *pulse64;
};

/* The norm of the beam vector sim[0..2] as a double-float, formed once per
 * pulse in double (the compensated signal divides by |b| |p|). */
__host__ __device__ inline void beam_norm_df(const float *sim, float &hi, float &lo) {
    const double x = sim[0], y = sim[1], z = sim[2];
    const double n = sqrt(x * x + y * y + z * z);
    hi = (float)n;
    lo = (float)(n - (double)hi);
}

/* the pass-1 weight of one gate (rs.cl:1196-1209), bit-exact.  The clamp
 * leaves an integer-valued floor in [0, max] (a NaN index clamps to 0), so
 * the conversion needs no range check. */
__device__ __forceinline__ float range_weight(const PulseArgs &P, float d) {
    float f0, f1;
    float dec0 = cl_fract(cl_clamp(fmaf(d, P.rwd[0], P.rwd[1] + 0.0f), 0.0f, P.rwd[2]), &f0);
    (void)cl_fract(cl_clamp(fmaf(d, P.rwd[0], P.rwd[1] + 1.0f), 0.0f, P.rwd[2]), &f1);
    return cl_mix(__ldg(P.rw + (uint32_t)f0), __ldg(P.rw + (uint32_t)f1), dec0);
}

/* The weight of the triangle table {0, 1, 0} with origin 1 and max 2 (what
 * RS_set_range_weight_to_triangle sets, rs.c:2620-2623), bit for bit the
 * value range_weight's two clamped indices, table picks and mix give on it:
 * on the rising side (index x0 in [0, 1)) the mix is 0 + (1 - 0) x0 = x0,
 * unless the second index has already rounded up to the last entry (x1 = 2,
 * a rounding corner within 2^-24 of the peak), where both picks are 0; on
 * the falling side (x0 in [1, 2)) it is 1 + (0 - 1)(x0 - 1) = 1 - (x0 - 1),
 * which is exact there; at x0 = 2 it is 0.  The GPU test of rsc_eval_math function
 * 8 compares it with the oracle's table lerp around every breakpoint. */
__device__ __forceinline__ float range_weight_tri(const float *rwd, float d) {
    /* t0, t1: the two raw indices; their clamps to [0, 2] are not formed.
     * On the rising side (t0 < 1) x0 = clamp(t0) is max(t0, 0) and x1 < 2
     * is t1 < 2; on the falling side x0 < 2 is t0 < 2, where x0 = t0.  A NaN
     * index gives 0, as the clamped form does. */
    const float t0 = fmaf(d, rwd[0], rwd[1] + 0.0f);
    const float t1 = fmaf(d, rwd[0], rwd[1] + 1.0f);
    const float up = t1 < 2.0f ? fmaxf(t0, 0.0f) : 0.0f;
    /* on [1, 2) both t0 - 1 and 1 - (t0 - 1) are exact (Sterbenz; a
     * multiple of 2^-23 in (0, 1]), so the falling side is 2 - t0, and
     * max(2 - t0, 0) gives the 0 at and beyond 2 (NaN: 0) */
    const float down = fmaxf(2.0f - t0, 0.0f);
    return t0 < 1.0f ? up : down;
}

/* the same weight with a table of at most 4 entries held in the kernel
 * parameters (the triangle of RS_set_range_weight_to_triangle has 3) */
__device__ __forceinline__ float range_weight_reg(const PulseArgs &P, float d) {
    if (P.rw_tri) return range_weight_tri(P.rwd, d);
    if (P.rw_n > 4) return range_weight(P, d);
    float f0, f1;
    float dec0 = cl_fract(cl_clamp(fmaf(d, P.rwd[0], P.rwd[1] + 0.0f), 0.0f, P.rwd[2]), &f0);
    (void)cl_fract(cl_clamp(fmaf(d, P.rwd[0], P.rwd[1] + 1.0f), 0.0f, P.rwd[2]), &f1);
    const uint32_t i0 = (uint32_t)f0, i1 = (uint32_t)f1;
    const float w0 = i0 == 0 ? P.rwv[0] : (i0 == 1 ? P.rwv[1] : (i0 == 2 ? P.rwv[2] : P.rwv[3]));
    const float w1 = i1 == 0 ? P.rwv[0] : (i1 == 1 ? P.rwv[1] : (i1 == 2 ? P.rwv[2] : P.rwv[3]));
    return cl_mix(w0, w1, dec0);
}

/* the angular weight of scat_sig_aux (rs.cl:1066-1089) */
__device__ __forceinline__ float angular_weight(const PulseArgs &P, float angle) {
    float fi0, fi1;
    float raw0 = cl_clamp(fmaf(angle, P.awd[0], P.awd[1] + 0.0f), 0.0f, P.awd[2]);
    float raw1 = cl_clamp(fmaf(angle, P.awd[0], P.awd[1] + 1.0f), 0.0f, P.awd[2]);
    float dec0 = cl_fract(raw0, &fi0);
    (void)cl_fract(raw1, &fi1);
    return cl_mix(__ldg(P.aw + (uint32_t)fi0), __ldg(P.aw + (uint32_t)fi1), dec0);
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
/* a + b = s + e exactly, for |a| >= |b| (or a == 0) */
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    e = b - (s - a);
}
/* (ah + al)(bh + bl) as a double-float pair (unnormalised), dropping al bl */
__device__ __forceinline__ void df_mul_pair(float ah, float al, float bh, float bl, float &h, float &l) {
    h = ah * bh;
    l = fmaf(ah, bl, fmaf(al, bh, fmaf(ah, bh, -h)));
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
/* double-float contributions: heads v, tails u */
struct AccDF {
    typedef float bin_t;
    static constexpr int kWords = 2;
    float v[4], u[4];
    __device__ void set(float a, float b, float c, float d) {
        v[0] = a; v[1] = b; v[2] = c; v[3] = d;
        u[0] = u[1] = u[2] = u[3] = 0.0f;
    }
    __device__ void set_lo(const float *t) { u[0] = t[0]; u[1] = t[1]; u[2] = t[2]; u[3] = t[3]; }
    __device__ void scale(float w, AccDF &o) const { scale_df(w, 0.0f, o); }
    __device__ void scale_df(float wh, float wl, AccDF &o) const {
#pragma unroll
        for (int l = 0; l < 4; l++) df_mul_pair(v[l], u[l], wh, wl, o.v[l], o.u[l]);
    }
    __device__ static void add_to(float *bin, const AccDF &c) {
#pragma unroll
        for (int l = 0; l < 4; l++) {
            float s, e;
            two_sum(bin[l], c.v[l], s, e);
            bin[l] = s;
            bin[4 + l] = bin[4 + l] + (e + c.u[l]);
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
        float lo[4] = {c.u[0], c.u[1], c.u[2], c.u[3]};
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
    float s_lo[4];       /* compensated: the tails of s (s + s_lo as double-floats) */
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

/* Launch shape of the LES layout kernels: blockIdx.x * 128 + threadIdx.x =
 * pair q in [0, nx + 2), rows (j, k) of the volume from blockIdx.y in steps
 * of gridDim.y. */
constexpr int kLesThreads = 128;

/* The remap of an LES frame (les.c:388-406): the file's u, v, w, p, t
 * planes (nn floats each) scaled into uvwt = (u v0, v v0, w v0, t t0), stored
 * in x-pair layout, and cpxx = (0, p p0, 0, 0), or (p p0, 0, 0, 0) when p is
 * the cn2 of the flat configuration. */
__global__ void __launch_bounds__(kLesThreads) k_les_remap(const float *__restrict__ raw, int nx, size_t rows,
                                                           float v0, float p0, float t0, int p_for_cn2,
                                                           float4 *__restrict__ uvwt, float4 *__restrict__ cpxx) {
    const int q = blockIdx.x * kLesThreads + threadIdx.x;
    if (q >= nx + 2) return;
    const size_t nn = rows * nx;
    for (size_t row = blockIdx.y; row < rows; row += gridDim.y) {
        const size_t k0 = row * nx + (size_t)min(max(q - 1, 0), nx - 1), k1 = row * nx + (size_t)min(q, nx - 1);
        const float4 a = make_float4(__ldg(raw + k0) * v0, __ldg(raw + nn + k0) * v0, __ldg(raw + 2 * nn + k0) * v0,
                                     __ldg(raw + 4 * nn + k0) * t0);
        const float4 b = make_float4(__ldg(raw + k1) * v0, __ldg(raw + nn + k1) * v0, __ldg(raw + 2 * nn + k1) * v0,
                                     __ldg(raw + 4 * nn + k1) * t0);
        float4 *o = uvwt + 2 * (row * (size_t)(nx + 2) + q);
        o[0] = a;
        o[1] = b;
        if (q >= 1 && q <= nx) {
            const size_t k = row * nx + (q - 1);
            const float pp = __ldg(raw + 3 * nn + k) * p0;
            cpxx[k] = p_for_cn2 ? make_float4(pp, 0.0f, 0.0f, 0.0f) : make_float4(0.0f, pp, 0.0f, 0.0f);
        }
    }
}

/* uvwt (rows * nx float4, x fastest) into the x-pair layout */
__global__ void __launch_bounds__(kLesThreads) k_les_pairs(const float4 *__restrict__ src, int nx, size_t rows,
                                                           float4 *__restrict__ uvwt) {
    const int q = blockIdx.x * kLesThreads + threadIdx.x;
    if (q >= nx + 2) return;
    for (size_t row = blockIdx.y; row < rows; row += gridDim.y) {
        float4 *o = uvwt + 2 * (row * (size_t)(nx + 2) + q);
        o[0] = __ldg(src + row * nx + min(max(q - 1, 0), nx - 1));
        o[1] = __ldg(src + row * nx + min(q, nx - 1));
    }
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
        case 8: {   /* the triangle range weight of d = a[i], scale b[i] */
            const float rwd[4] = {b[i], 1.0f, 2.0f, 0.0f};
            out[i] = range_weight_tri(rwd, a[i]);
            break;
        }
        default: out[i] = 0.0f; break;
    }
}

}  // namespace rsc

#endif
