/*
 * rsc_batch.cuh -- many emulation instances per launch.
 *
 * An instance is one worker: its own scatterer arrays, tables, gates, pulse
 * accumulator and counter.  One time step of every instance is three
 * launches: k_pulse_batch forms every instance's pulse on the batch's
 * stream while k_advance_batch_rain advances every instance's background
 * range on the advance stream (into the instance's other pos / rcs pair) and
 * k_advance_batch_debris, beside it on a high-priority stream, every
 * instance's debris.  Blocks are assigned to instances in proportion to
 * their work through a prefix table; each block copies its instance's launch
 * descriptor into shared memory, takes the step's beam / time / LES slot from
 * the per-step table, and runs the same block bodies as the one-instance
 * kernels (so every instance's state evolves bit for bit as it would alone).
 * A run of K steps is 3 K launches whose arguments differ only in the step
 * index, which is what lets the host capture it once in a CUDA graph.
 */
#ifndef SIMRADAR_GB300_RSC_BATCH_CUH
#define SIMRADAR_GB300_RSC_BATCH_CUH

#include "rsc_step.cuh"

namespace rsc {

/* per instance per step: the simulation descriptor, the LES slot, and the
 * pos / rcs pair the step's pulse and advance read and the pair the advance
 * writes (the instance's two pairs alternate from step to step, so the
 * pulse of a step runs beside its advance) */
struct BatchStep {
    float sim[16];
    int les_id;
    int pad[3];
    const float4 *pos_r, *rcs_r;
    float4 *pos_w, *rcs_w;
};

/* per instance, fixed for the batch: the advance descriptor plus both LES /
 * debris-flux-field slots (the step picks one) */
struct BatchAdvance {
    AdvanceArgs a;
    PairImage uvwt[2];
    Image cpxx[2];
    const float *dff[2];
};

/* the instance owning block b: the last i with prefix[i] <= b */
__device__ __forceinline__ int batch_instance(const unsigned *prefix, int n, unsigned b) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(prefix + mid) <= b) {
            lo = mid;
        } else {
            hi = mid - 1;
        }
    }
    return lo;
}

/* copy `bytes` (a multiple of 4) from global to shared memory, whole block */
__device__ __forceinline__ void block_copy(void *dst, const void *src, unsigned bytes) {
    const unsigned *s = static_cast<const unsigned *>(src);
    unsigned *d = static_cast<unsigned *>(dst);
    for (unsigned k = threadIdx.x; k < bytes / 4; k += blockDim.x) d[k] = __ldg(s + k);
}

/* The instance of this block and its advance descriptor for the step, in
 * shared memory; returns the instance. */
__device__ __forceinline__ int batch_advance_args(AdvanceArgs &sa, int &s_i, const BatchAdvance *inst,
                                                  const BatchStep *steps, const unsigned *prefix, int ninst) {
    if (threadIdx.x == 0) s_i = batch_instance(prefix, ninst, blockIdx.x);
    __syncthreads();
    const int i = s_i;
    block_copy(&sa, &inst[i].a, sizeof(AdvanceArgs));
    __syncthreads();
    if (threadIdx.x < 16) sa.sim[threadIdx.x] = steps[i].sim[threadIdx.x];
    if (threadIdx.x == 0) {
        const int les = steps[i].les_id & 1;
        sa.uvwt = inst[i].uvwt[les];
        sa.cpxx = inst[i].cpxx[les];
        sa.dff = inst[i].dff[les];
        sa.pos_in = steps[i].pos_r;
        sa.rcs_in = steps[i].rcs_r;
        sa.pos = steps[i].pos_w;
        sa.rcs = steps[i].rcs_w;
    }
    __syncthreads();
    return i;
}

/* The background range of every instance (prefix over their background
 * blocks of T threads); the rain body chosen per instance by its concept.
 * A full SM of resident threads (32 registers) measured 6% faster per
 * batched step than 6 blocks of 256 (40 registers), which had been faster
 * than 5: resident warps hide the texel loads' latency.  T (64, 128, 256)
 * and the resident blocks per SM (limited through dynamic shared memory)
 * are the batch's advance shape, which rsc_batch_autotune times. */
template <int T>
__global__ void __launch_bounds__(T, 2048 / T)
k_advance_batch_rain(const BatchAdvance *inst, const BatchStep *steps, const unsigned *prefix, int ninst) {
    __shared__ __align__(16) AdvanceArgs sa;
    __shared__ int s_i;
    const int i = batch_advance_args(sa, s_i, inst, steps, prefix, ninst);
    const unsigned long long j = (unsigned long long)(blockIdx.x - __ldg(prefix + i)) * T + threadIdx.x;
    if (j >= sa.rain_count) return;
    const size_t x = (size_t)(sa.rain_origin + j);
    float4 pos, rcs;
    bool known;
    if (sa.rain_mode == 1) {
        rain_el(sa, x, pos, rcs, known);
    } else if (sa.rain_mode == 0) {
        rain_bg(sa, x, pos, rcs, known);
    } else {
        rain_fp(sa, x, pos, rcs, known);
    }
}

/* The debris ranges of every instance (prefix over their debris blocks), run
 * beside k_advance_batch_rain on a high-priority stream. */
__global__ void __launch_bounds__(kAdvanceThreads)
k_advance_batch_debris(const BatchAdvance *inst, const BatchStep *steps, const unsigned *prefix, int ninst) {
    __shared__ __align__(16) AdvanceArgs sa;
    __shared__ int s_i;
    const int i = batch_advance_args(sa, s_i, inst, steps, prefix, ninst);
    const unsigned long long j = (unsigned long long)(blockIdx.x - __ldg(prefix + i)) * kAdvanceThreads + threadIdx.x;
    if (sa.ntypes == 0 || j >= sa.deb_prefix[sa.ntypes]) return;
    const int t = debris_type_of(sa, j);
    const DebrisType &T = sa.types[t];
    float4 pos, rcs;
    bool known;
    debris_step(sa, T, (size_t)(T.origin + (j - sa.deb_prefix[t])), pos, rcs, known);
}

/* TRI 1: every instance's range table is the triangle (compiled in) */
template <int MODE, int TRI = -1>
__global__ void __launch_bounds__(512)
k_pulse_batch(const PulseArgs *inst, const BatchStep *steps, const unsigned *prefix, int ninst, float4 *out,
              unsigned out_stride) {
    __shared__ __align__(16) PulseArgs sp;
    __shared__ int s_i;
    if (threadIdx.x == 0) s_i = batch_instance(prefix, ninst, blockIdx.x);
    __syncthreads();
    const int i = s_i;
    block_copy(&sp, &inst[i], sizeof(PulseArgs));
    __syncthreads();
    if (threadIdx.x < 16) sp.sim[threadIdx.x] = steps[i].sim[threadIdx.x];
    if (threadIdx.x == 0) {
        sp.pulse = out + (size_t)i * out_stride;
        sp.pos = steps[i].pos_r;
        sp.rcs = steps[i].rcs_r;
        beam_norm_df(steps[i].sim, sp.bn_hi, sp.bn_lo);
    }
    __syncthreads();
    const unsigned b0 = __ldg(prefix + i);
    /* an instance whose state is in spatial order takes two scatterers per
     * lane, as the one-instance kernel does */
    if (MODE != 2 && sp.coherent_span > 0 && !sp.materialize) {
        pulse_body_group<MODE == 2 ? 0 : MODE, 2, TRI>(sp, blockIdx.x - b0, __ldg(prefix + i + 1) - b0);
    } else {
        pulse_body<MODE>(sp, blockIdx.x - b0, __ldg(prefix + i + 1) - b0);
    }
}

/* ---- every step of a run in one launch (the persistent form) ----
 * Each block owns a fixed list of segments -- contiguous index ranges of an
 * instance, cut by the host so that every block carries the same cost --
 * and runs every step of the run on them: the segment's share of the
 * instance's pulse (its bins summed into that step's accumulator of the
 * instance, the last of the instance's blocks converting it), then the
 * advance of the same scatterers into the step's other pos / rcs pair.  The
 * pulse of step k + 1 reads only what this block's advance of step k wrote
 * and the advance of step k + 1 overwrites only what this block's pulse of
 * step k read, so no block ever waits for another: the pulses of different
 * steps use different accumulators and tickets ([step][instance]).  State is
 * read by the pulse with L2 loads (ld.global.cg): the arrays change during
 * the launch, so the read-only (non-coherent) path may not serve them. */
struct PersistSeg {
    unsigned long long start, end;   /* [start, end) of instance `inst` */
    int inst;
    int pad;
};

struct PersistArgs {
    const BatchAdvance *adv;
    const PulseArgs *pulse;
    const BatchStep *steps;          /* [k][instance] */
    const PersistSeg *seg;           /* the segments of block b: seg[seg_off[b] .. seg_off[b + 1]) */
    const unsigned *seg_off;
    const unsigned *nblk;            /* per instance: the blocks whose segments cover it */
    double *acc;                     /* [k][instance][Gmax][4], zero at launch */
    unsigned *tick;                  /* [k][instance], zero at launch */
    float4 *out;                     /* [k][instance][out_stride] */
    unsigned out_stride, Gmax;
    int steps_n, ninst;
};

constexpr int kPersistThreads = 256;

/* The pulse share of [start, end): runs of 64 neighbours per warp, two per
 * lane (PulseBins::add_k), then the block's sums into the accumulator. */
template <int MODE, int TRI>
__device__ __forceinline__ void persist_pulse(const PulseArgs &P, unsigned long long start, unsigned long long end,
                                              unsigned nblk) {
    PulseBins<MODE, 1> B;
    B.init(P);
    const unsigned long long stride = 64ull * (blockDim.x >> 5);
    for (unsigned long long base = start + 64ull * B.warp; base < end; base += stride) {
        bool in[2];
        unsigned long long idx[2];
        float4 pp[2], xx[2];
#pragma unroll
        for (int q = 0; q < 2; q++) {
            idx[q] = base + 32u * q + B.lane;
            in[q] = idx[q] < end;
            pp[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            xx[q] = pp[q];
            if (in[q]) {
                pp[q] = __ldcg(P.pos + idx[q]);
                xx[q] = __ldcg(P.rcs + idx[q]);
            }
        }
        B.template add_k<2, TRI>(P, in, idx, pp, xx);
    }
    B.finish(P, nblk);
}

/* The advance of [start, end): the background body of the instance's
 * concept inside the background range, db_atts inside a debris range. */
__device__ __forceinline__ void persist_advance(const AdvanceArgs &a, unsigned long long start, unsigned long long end) {
    const unsigned long long r0 = a.rain_origin, r1 = a.rain_origin + a.rain_count;
    for (unsigned long long x = start + threadIdx.x; x < end; x += blockDim.x) {
        float4 pos, rcs;
        bool known;
        if (x >= r0 && x < r1) {
            if (a.rain_mode == 1) {
                rain_el(a, (size_t)x, pos, rcs, known);
            } else if (a.rain_mode == 0) {
                rain_bg(a, (size_t)x, pos, rcs, known);
            } else {
                rain_fp(a, (size_t)x, pos, rcs, known);
            }
            continue;
        }
        for (int t = 0; t < a.ntypes; t++) {
            const DebrisType &T = a.types[t];
            if (x >= T.origin && x < T.origin + T.count) {
                debris_step(a, T, (size_t)x, pos, rcs, known);
                break;
            }
        }
    }
}

template <int MODE, int TRI = -1>
__global__ void __launch_bounds__(kPersistThreads, 4) k_batch_persist(const PersistArgs A) {
    __shared__ __align__(16) PulseArgs sp;
    __shared__ __align__(16) AdvanceArgs sa;
    const unsigned s0 = __ldg(A.seg_off + blockIdx.x), s1 = __ldg(A.seg_off + blockIdx.x + 1);
    for (int k = 0; k < A.steps_n; k++) {
        for (unsigned sg = s0; sg < s1; sg++) {
            const int i = A.seg[sg].inst;
            const unsigned long long start = A.seg[sg].start, end = A.seg[sg].end;
            const size_t slot = (size_t)k * A.ninst + i;
            const BatchStep *st = A.steps + slot;
            /* the pulse of step k on this segment */
            block_copy(&sp, &A.pulse[i], sizeof(PulseArgs));
            __syncthreads();
            if (threadIdx.x < 16) sp.sim[threadIdx.x] = st->sim[threadIdx.x];
            if (threadIdx.x == 0) {
                sp.pulse = A.out + slot * A.out_stride;
                sp.acc64 = A.acc + slot * A.Gmax * 4;
                sp.counter = A.tick + slot;
                sp.pos = st->pos_r;
                sp.rcs = st->rcs_r;
                beam_norm_df(st->sim, sp.bn_hi, sp.bn_lo);
            }
            __syncthreads();
            persist_pulse<MODE, TRI>(sp, start, end, __ldg(A.nblk + i));
            __syncthreads();
            /* then its advance into the step's other pair */
            block_copy(&sa, &A.adv[i].a, sizeof(AdvanceArgs));
            __syncthreads();
            if (threadIdx.x < 16) sa.sim[threadIdx.x] = st->sim[threadIdx.x];
            if (threadIdx.x == 0) {
                const int les = st->les_id & 1;
                sa.uvwt = A.adv[i].uvwt[les];
                sa.cpxx = A.adv[i].cpxx[les];
                sa.dff = A.adv[i].dff[les];
                sa.pos_in = st->pos_r;
                sa.rcs_in = st->rcs_r;
                sa.pos = st->pos_w;
                sa.rcs = st->rcs_w;
            }
            __syncthreads();
            persist_advance(sa, start, end);
            __syncthreads();
        }
    }
}

}  // namespace rsc

#endif
