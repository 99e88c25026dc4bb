/*
 * rsc.cu -- host side of the GB300 backend: the C ABI declared in
 * include/rsc.h.  Device memory, table uploads, launch geometry and the
 * lazily formed aux / sig arrays live here; the kernels are in
 * rsc_kernels.cuh.  Compiled with -fmad=false (see rsmath.h).
 */
#include <cuda_runtime.h>

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <tuple>
#include <mutex>
#include <vector>

#include "../../include/rsc.h"
#include "rsc_batch.cuh"
#include "rsc_sort.cuh"
#include "rsc_les.h"
#include "rsc_populate.h"

using rsc::AdvanceArgs;
using rsc::DebrisType;
using rsc::Image;
using rsc::PulseArgs;

namespace {

thread_local char g_err[512] = "";

int fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

/* A failed CUDA call: the runtime also keeps the error as its "last error",
 * which a later cudaGetLastError() after a good launch would report again;
 * it is read (cleared) here.  An error that leaves the context unusable
 * stays, as it must. */
int cuda_fail(int code, const char *fmt, ...) {
    (void)cudaGetLastError();
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

#define RSC_CUDA(call)                                                                          \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            return cuda_fail(e_ == cudaErrorMemoryAllocation ? RSC_ERR_NOMEM : RSC_ERR_CUDA,    \
                             "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
        }                                                                                       \
    } while (0)

struct Table2D {
    float4 *a = nullptr, *b = nullptr;
    uint32_t nx = 0, ny = 0;
    float desc[16] = {0};
};

}  // namespace

struct rsc_worker {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    /* attribute arrays */
    size_t num_scats = 0, numel = 0;
    float4 *pos = nullptr, *vel = nullptr, *ori = nullptr, *tum = nullptr;
    float4 *aux = nullptr, *rcs = nullptr, *sig = nullptr;
    uint4 *rnd = nullptr;
    /* pulse */
    uint32_t G = 0;
    float range_start = 0.0f, range_delta = 0.0f;
    float4 *pulse = nullptr;
    double *pulse64 = nullptr;
    float *rk = nullptr, *rk_hi = nullptr, *rk_lo = nullptr;
    double *rk64 = nullptr;
    double *acc64 = nullptr;      /* the pulse kernel's FP64 grid accumulator */
    unsigned *counter = nullptr;
    unsigned long long *runs = nullptr;   /* the compensated pulse's run counter */
    /* tables */
    float *range_weight = nullptr;
    uint32_t range_n = 0;
    float range_desc[4] = {0};
    float range_weight_host0 = 1.0f, range_weight_hostm = 1.0f; /* edge values W[0], W[xm] */
    float range_weight_small[4] = {0.0f, 0.0f, 0.0f, 0.0f};   /* the first 4 entries, for tables of <= 4 */
    float *angular_weight = nullptr;
    uint32_t angular_n = 0;
    float angular_desc[4] = {0};
    float4 *ellipsoid = nullptr;
    uint32_t ellipsoid_n = 0;
    float ellipsoid_desc[4] = {0};
    float4 *les_uvwt[2] = {nullptr, nullptr}, *les_cpxx[2] = {nullptr, nullptr};
    uint32_t les_nx = 0, les_ny = 0, les_nz = 0;
    float les_desc[16] = {0};
    /* LES frames from an rsc_les_source: raw planes copied on les_copy into
     * les_raw and remapped into a slot; les_ready[slot] marks the slot
     * written, les_wait[slot] that no advance has waited for it yet */
    cudaStream_t les_copy = nullptr;
    cudaEvent_t les_mark = nullptr, les_ready[2] = {nullptr, nullptr};
    bool les_wait[2] = {false, false};
    float *les_raw = nullptr;
    size_t les_raw_n = 0;
    /* uvwt of rsc_set_les on its way into a slot's x-pair layout */
    float4 *les_stage = nullptr;
    size_t les_stage_n = 0;
    Table2D adm[RSC_MAX_TYPES];
    Table2D rcs_tab[RSC_MAX_TYPES];
    float *dff[2] = {nullptr, nullptr};
    uint32_t dff_n = 0;
    float dff_desc[16] = {0};
    /* modes and bookkeeping */
    int precision = RSC_PULSE_PLAIN;
    int materialize = 0;
    int moments = 1;          /* rsc_set_pulse_moments */
    bool sig_aux_stale = false;
    bool have_pulse_desc = false;
    /* the pos / rcs pair the latest pulse read: its aux / sig, when the pulse
     * kernel did not write them, are formed from this pair */
    const float4 *sa_pos = nullptr, *sa_rcs = nullptr;
    float last_sim[16] = {0};
    uint64_t launches = 0;
    /* pulse launch shape chosen by rsc_autotune (0: default) */
    int tune_warps = 0, tune_per_sm = 0;
    int adv_per_thread = 1;   /* background scatterers per advance thread (rsc_set_advance_shape) */
    /* spatial order of the background range (rsc_sort.cuh): perm[slot] is the
     * caller's index, inv[index] the slot; NULL perm = caller's order */
    int sort_interval = 128;
    uint64_t since_sort = 0;
    bool sort_due = true;
    unsigned *perm = nullptr, *perm_alt = nullptr, *inv = nullptr;
    unsigned *sort_key = nullptr, *sort_order = nullptr, *sort_hist = nullptr, *sort_blocks = nullptr;
    uint4 *alt[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    uint64_t sorts = 0;
    /* fused step: rsc_advance_time records the advance, and the next
     * rsc_make_pulse runs it together with the pulse (k_step); any other call
     * that reads or changes the state or the tables runs it alone first */
    int fuse = 0;
    cudaStream_t side = nullptr;             /* debris kernel beside the background kernel */
    /* The advance of a step runs on `adv` beside the pulse of the same step on
     * `stream`: it reads the current pos / rcs pair (which the pulse reads)
     * and writes the other pair, which then becomes current.  ev_read /
     * ev_read_next follow the pairs: recorded after the last pulse that read
     * them, the advance waits for the one of the pair it overwrites.  Work on
     * `stream` that reads or changes the state or the advance's tables first
     * waits for `adv` (flush_pending) and then has the next advance wait for
     * it (release_main). */
    float4 *pos_next = nullptr, *rcs_next = nullptr;
    cudaStream_t adv = nullptr;
    cudaEvent_t ev_read = nullptr, ev_read_next = nullptr, ev_adv = nullptr, ev_main = nullptr;
    bool read_pending = false, read_next_pending = false, main_pending = false;
    uint64_t adv_seq = 0, adv_joined = 0;   /* work queued on adv / covered by the last join */
    /* the last pulse launch shape: mode, path, gates, tuning -> grid, threads, smem */
    int geo_key[5] = {-1, -1, -1, -1, -1};
    int geo_grid = 0, geo_threads = 0;
    size_t geo_smem = 0;
    /* rsc_download_pulse_async: the pulse goes to the host on its own stream,
     * so the next advance does not wait for the copy; the next pulse kernel
     * (which rewrites the pulse) waits for d2h_done */
    cudaStream_t d2h = nullptr;
    cudaEvent_t pulse_ev = nullptr, d2h_done = nullptr;
    bool d2h_pending = false;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    bool pend = false;
    AdvanceArgs pend_a;
    unsigned pend_blocks = 0;
    rsc_population pend_pop;
    float pend_sim[16] = {0};
};

namespace {
int flush_pending(rsc_worker *w);

/* The worker's stream waits for everything queued on the advance stream. */
int join_adv(rsc_worker *w) {
    if (w->adv_joined == w->adv_seq) return RSC_OK;   /* nothing queued there since */
    w->adv_joined = w->adv_seq;
    cudaError_t e = cudaEventRecord(w->ev_adv, w->adv);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(w->stream, w->ev_adv, 0);
    if (e != cudaSuccess) return cuda_fail(RSC_ERR_CUDA, "stream ordering: %s", cudaGetErrorString(e));
    return RSC_OK;
}

/* The next advance waits for the work queued on the worker's stream so far
 * (after work there that changed the state or a table the advance reads). */
int release_main(rsc_worker *w) {
    cudaError_t e = cudaEventRecord(w->ev_main, w->stream);
    if (e != cudaSuccess) return cuda_fail(RSC_ERR_CUDA, "stream ordering: %s", cudaGetErrorString(e));
    w->main_pending = true;
    return RSC_OK;
}

/* After a launch on the worker's stream that reads the current pos / rcs
 * pair: the advance that overwrites the pair waits for it. */
int mark_read(rsc_worker *w) {
    cudaError_t e = cudaEventRecord(w->ev_read, w->stream);
    if (e != cudaSuccess) return cuda_fail(RSC_ERR_CUDA, "stream ordering: %s", cudaGetErrorString(e));
    w->read_pending = true;
    return RSC_OK;
}
}

namespace {

int check_worker(rsc_worker *w) {
    if (w == nullptr) return fail(RSC_ERR_ARG, "worker is NULL");
    cudaError_t e = cudaSetDevice(w->device);
    if (e != cudaSuccess) return cuda_fail(RSC_ERR_CUDA, "cudaSetDevice(%d): %s", w->device, cudaGetErrorString(e));
    return RSC_OK;
}

int check_alloc(rsc_worker *w) {
    int s = check_worker(w);
    if (s) return s;
    if (w->pos == nullptr) return fail(RSC_ERR_STATE, "rsc_worker_malloc has not been called");
    return RSC_OK;
}

void free_ptr(void *p) {
    if (p) cudaFree(p);
}

void free_sort(rsc_worker *w) {
    unsigned **u[] = {&w->perm, &w->perm_alt, &w->inv, &w->sort_key, &w->sort_order, &w->sort_hist, &w->sort_blocks};
    for (unsigned **q : u) {
        free_ptr(*q);
        *q = nullptr;
    }
    for (uint4 *&a : w->alt) {
        free_ptr(a);
        a = nullptr;
    }
    w->sort_due = true;
    w->since_sort = 0;
}

/* The eight attribute arrays as 16-byte elements, in a fixed order. */
void attribute_arrays(rsc_worker *w, uint4 **out[8]) {
    out[0] = reinterpret_cast<uint4 **>(&w->pos);
    out[1] = reinterpret_cast<uint4 **>(&w->vel);
    out[2] = reinterpret_cast<uint4 **>(&w->ori);
    out[3] = reinterpret_cast<uint4 **>(&w->tum);
    out[4] = reinterpret_cast<uint4 **>(&w->aux);
    out[5] = reinterpret_cast<uint4 **>(&w->rcs);
    out[6] = reinterpret_cast<uint4 **>(&w->sig);
    out[7] = &w->rnd;
}

void free_arrays(rsc_worker *w) {
    if (w->d2h) cudaStreamSynchronize(w->d2h);
    if (w->adv) cudaStreamSynchronize(w->adv);
    w->d2h_pending = false;
    w->read_pending = w->read_next_pending = w->main_pending = false;
    free_ptr(w->pos_next);
    free_ptr(w->rcs_next);
    w->pos_next = w->rcs_next = nullptr;
    free_ptr(w->pos);
    free_ptr(w->vel);
    free_ptr(w->ori);
    free_ptr(w->tum);
    free_ptr(w->aux);
    free_ptr(w->rcs);
    free_ptr(w->sig);
    free_ptr(w->rnd);
    free_ptr(w->pulse);
    free_ptr(w->pulse64);
    free_ptr(w->rk);
    free_ptr(w->rk_hi);
    free_ptr(w->rk_lo);
    free_ptr(w->rk64);
    free_ptr(w->acc64);
    free_ptr(w->counter);
    free_ptr(w->runs);
    free_sort(w);
    w->pos = w->vel = w->ori = w->tum = w->aux = w->rcs = w->sig = w->pulse = nullptr;
    w->rnd = nullptr;
    w->pulse64 = nullptr;
    w->rk = w->rk_hi = w->rk_lo = nullptr;
    w->rk64 = nullptr;
    w->acc64 = nullptr;
    w->counter = nullptr;
    w->runs = nullptr;
    w->num_scats = w->numel = 0;
}

int upload_floats(float **dst, const float *src, size_t n) {
    free_ptr(*dst);
    *dst = nullptr;
    RSC_CUDA(cudaMalloc((void **)dst, n * sizeof(float)));
    RSC_CUDA(cudaMemcpy(*dst, src, n * sizeof(float), cudaMemcpyHostToDevice));
    return RSC_OK;
}

int upload_float4(float4 **dst, const float *src4, size_t n) {
    free_ptr(*dst);
    *dst = nullptr;
    RSC_CUDA(cudaMalloc((void **)dst, n * sizeof(float4)));
    RSC_CUDA(cudaMemcpy(*dst, src4, n * sizeof(float4), cudaMemcpyHostToDevice));
    return RSC_OK;
}

Image make_image(const float4 *d, uint32_t nx, uint32_t ny, uint32_t nz) {
    Image im;
    im.data = d;
    im.nx = (int)nx;
    im.ny = (int)ny;
    im.nz = (int)nz;
    return im;
}

/* The range weight table is RS_set_range_weight_to_triangle's {0, 1, 0}
 * (entries compared bit for bit: a -0 would change the mix) with origin 1
 * and max 2, which the pulse kernel evaluates by range_weight_tri. */
bool is_triangle(uint32_t n, const float *w4, const float *desc) {
    static const float tri[3] = {0.0f, 1.0f, 0.0f};
    return n == 3 && memcmp(w4, tri, sizeof(tri)) == 0 && desc[1] == 1.0f && desc[2] == 2.0f;
}

rsc::PairImage make_pair_image(const float4 *d, uint32_t nx, uint32_t ny, uint32_t nz) {
    rsc::PairImage im;
    im.data = d;
    im.nx = (int)nx;
    im.ny = (int)ny;
    im.nz = (int)nz;
    return im;
}

/* float4 count of an LES uvwt slot in x-pair layout */
size_t les_pair_float4s(uint32_t nx, uint32_t ny, uint32_t nz) { return 2 * ((size_t)nx + 2) * ny * nz; }

/* Grid of the LES layout kernels for nx x rows. */
dim3 les_grid(uint32_t nx, size_t rows) {
    return dim3((unsigned)((nx + 2 + rsc::kLesThreads - 1) / rsc::kLesThreads), (unsigned)std::min<size_t>(rows, 65535));
}

/* A device array of at least n elements (contents not kept). */
template <typename T>
int ensure_buffer(T **p, size_t *cap, size_t n, cudaStream_t wait_stream) {
    if (*cap >= n) return RSC_OK;
    if (wait_stream) cudaStreamSynchronize(wait_stream);
    free_ptr(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(RSC_ERR_NOMEM, "%zu MB of LES staging: %s", (n * sizeof(T)) >> 20, cudaGetErrorString(e));
    *cap = n;
    return RSC_OK;
}

/* Debris launch description shared by the advance kernels and k_db_rcs. */
int fill_debris(rsc_worker *w, const rsc_population *pop, AdvanceArgs &a, unsigned long long *total) {
    a.ntypes = 0;
    unsigned long long acc = 0;
    for (int k = 1; k < RSC_MAX_TYPES; k++) {
        if (pop->counts[k] == 0) continue;
        if (pop->origins[k] + pop->counts[k] > w->num_scats) {
            return fail(RSC_ERR_ARG, "debris type %d range [%llu, %llu) exceeds %zu scatterers", k,
                        (unsigned long long)pop->origins[k], (unsigned long long)(pop->origins[k] + pop->counts[k]),
                        w->num_scats);
        }
        int ai = pop->adm_index[k], ri = pop->rcs_index[k];
        if (ai < 0 || ai >= RSC_MAX_TYPES || w->adm[ai].a == nullptr) {
            return fail(RSC_ERR_STATE, "debris type %d: ADM table %d not set", k, ai);
        }
        if (ri < 0 || ri >= RSC_MAX_TYPES || w->rcs_tab[ri].a == nullptr) {
            return fail(RSC_ERR_STATE, "debris type %d: RCS table %d not set", k, ri);
        }
        DebrisType &T = a.types[a.ntypes];
        T.origin = pop->origins[k];
        T.count = pop->counts[k];
        T.cd = make_image(w->adm[ai].a, w->adm[ai].nx, w->adm[ai].ny, 1);
        T.cm = make_image(w->adm[ai].b, w->adm[ai].nx, w->adm[ai].ny, 1);
        T.re = make_image(w->rcs_tab[ri].a, w->rcs_tab[ri].nx, w->rcs_tab[ri].ny, 1);
        T.im = make_image(w->rcs_tab[ri].b, w->rcs_tab[ri].nx, w->rcs_tab[ri].ny, 1);
        memcpy(T.adm, w->adm[ai].desc, sizeof(T.adm));
        memcpy(T.rcs, w->rcs_tab[ri].desc, sizeof(T.rcs));
        a.deb_prefix[a.ntypes] = acc;
        acc += pop->counts[k];
        a.ntypes++;
    }
    a.deb_prefix[a.ntypes] = acc;
    *total = acc;
    return RSC_OK;
}

/* Gate origins: the FP32 running sum of make_pulse_pass_1 (rs.cl:1214) and
 * the FP64 values range_start + k * range_delta (head and tail). */
int set_gates(rsc_worker *w) {
    const uint32_t G = w->G;
    std::vector<float> rk(G), hi(G), lo(G);
    std::vector<double> r64(G);
    float r = w->range_start;
    for (uint32_t k = 0; k < G; k++) {
        rk[k] = r;
        r = r + w->range_delta;
        double e = (double)w->range_start + (double)k * (double)w->range_delta;
        r64[k] = e;
        hi[k] = (float)e;
        lo[k] = (float)(e - (double)hi[k]);
    }
    RSC_CUDA(cudaMemcpy(w->rk, rk.data(), G * sizeof(float), cudaMemcpyHostToDevice));
    RSC_CUDA(cudaMemcpy(w->rk_hi, hi.data(), G * sizeof(float), cudaMemcpyHostToDevice));
    RSC_CUDA(cudaMemcpy(w->rk_lo, lo.data(), G * sizeof(float), cudaMemcpyHostToDevice));
    RSC_CUDA(cudaMemcpy(w->rk64, r64.data(), G * sizeof(double), cudaMemcpyHostToDevice));
    return RSC_OK;
}

/* Resident blocks per SM of a kernel at a launch shape.  The kernel's
 * dynamic shared memory limit is raised to the device's opt-in maximum, so
 * a shape computed once stays launchable whatever other workers set. */
template <typename K>
cudaError_t kernel_occupancy(K kern, int threads, size_t smem, int *per_sm) {
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kern);
    const int max_dynamic = optin - (int)fa.sharedSizeBytes;   /* the static part counts against the limit */
    if (e == cudaSuccess && (max_dynamic < 0 || (size_t)max_dynamic < smem)) e = cudaErrorInvalidValue;
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, kern, threads, smem);
    return e;
}

/* Scatterers per lane of the grouped plain pulse kernel: 2 measured fastest
 * (51.7 us against 54.7 for 3 and 62.0 for 4 at README scale: more
 * registers per lane, fewer resident warps). */
constexpr int kPulseGroup = 2;

typedef void (*PulseKernel)(const PulseArgs);

/* The one-instance pulse kernel for a mode and a gate path (0 atomics, 1
 * coherent warps, 2 every gate).  The plain form is compiled once per path
 * (1.5% faster on a 2M-scatterer step); the compensated and FP64 forms choose
 * the path at run time (one compensated kernel per path measured 7% slower). */
PulseKernel pulse_kernel(int mode, int path) {
    if (mode == RSC_PULSE_PLAIN) {
        if (path == 4) return rsc::k_pulse_group<0, kPulseGroup, 1>;
        if (path == 3) return rsc::k_pulse_group<0, kPulseGroup>;
        return path == 2 ? rsc::k_pulse<0, 2> : (path == 1 ? rsc::k_pulse<0, 1> : rsc::k_pulse<0, 0>);
    }
    if (mode == RSC_PULSE_COMPENSATED) {
        if (path == 4) return rsc::k_pulse_group<1, kPulseGroup, 1>;
        return path == 3 ? rsc::k_pulse_group<1, kPulseGroup> : rsc::k_pulse<1, -1>;
    }
    return rsc::k_pulse<2, -1>;
}

/* 0 atomics, 1 coherent warps, 2 every gate, 3 coherent warps with
 * kPulseGroup scatterers per lane (the compensated form, and the plain form
 * when it does not write aux / sig), 4 the same with the triangle range
 * table compiled in */
int pulse_path(const PulseArgs &P, int mode) {
    if (P.dense) return 2;
    if (P.coherent_span <= 0) return 0;
    if ((mode == RSC_PULSE_PLAIN && !P.materialize) || mode == RSC_PULSE_COMPENSATED) return P.rw_tri ? 4 : 3;
    return 1;
}

/* Launch shape of the pulse kernel (one-instance or batched form) for G
 * gates: warps per block as many as fit 200 KB of bins (at most 16, at most
 * want_warps when that is > 0), resident blocks per SM from the occupancy
 * calculator (at most 4, at most want_per_sm when that is > 0). */
int pulse_shape(int mode, bool batch, uint32_t G, int want_warps, int want_per_sm, int *per_sm_out, int *threads,
                size_t *smem, int path = 0) {
    size_t per_warp = rsc::pulse_warp_bytes(mode, G);
    size_t budget = 200 * 1024;
    int warps = (int)(budget / per_warp);
    if (warps > 16) warps = 16;
    if (warps < 1) return fail(RSC_ERR_UNSUPPORTED, "%u gates do not fit the pulse kernel's shared memory", G);
    if (want_warps > 0 && want_warps < warps) warps = want_warps;
    *threads = warps * 32;
    *smem = (size_t)warps * per_warp + 2 * G * sizeof(float);
    int per_sm = 1;
    cudaError_t e;
    if (!batch) {
        e = kernel_occupancy(pulse_kernel(mode, path), *threads, *smem, &per_sm);
    } else if (mode == RSC_PULSE_PLAIN || mode == RSC_PULSE_COMPENSATED) {
        /* both forms of the batched kernel (range table tested per gate, and
         * the triangle compiled in) get the shared-memory limit raised; the
         * shape is the one both fit */
        int per_sm_tri = 1;
        if (mode == RSC_PULSE_PLAIN) {
            e = kernel_occupancy(rsc::k_pulse_batch<0>, *threads, *smem, &per_sm);
            if (e == cudaSuccess) e = kernel_occupancy(rsc::k_pulse_batch<0, 1>, *threads, *smem, &per_sm_tri);
        } else {
            e = kernel_occupancy(rsc::k_pulse_batch<1>, *threads, *smem, &per_sm);
            if (e == cudaSuccess) e = kernel_occupancy(rsc::k_pulse_batch<1, 1>, *threads, *smem, &per_sm_tri);
        }
        if (per_sm_tri < per_sm) per_sm = per_sm_tri;
    } else {
        e = kernel_occupancy(rsc::k_pulse_batch<2>, *threads, *smem, &per_sm);
    }
    if (e != cudaSuccess) return cuda_fail(RSC_ERR_CUDA, "pulse kernel configuration: %s", cudaGetErrorString(e));
    if (per_sm < 1) per_sm = 1;
    if (per_sm > 4) per_sm = 4;
    if (want_per_sm > 0 && want_per_sm < per_sm) per_sm = want_per_sm;
    *per_sm_out = per_sm;
    return RSC_OK;
}

int pulse_geometry(rsc_worker *w, int mode, int path, int *grid, int *threads, size_t *smem) {
    const int key[5] = {mode, path, (int)w->G, w->tune_warps, w->tune_per_sm};
    if (memcmp(key, w->geo_key, sizeof(key)) == 0) {
        /* same shape as the last launch: no occupancy query per pulse */
        *grid = w->geo_grid;
        *threads = w->geo_threads;
        *smem = w->geo_smem;
        return RSC_OK;
    }
    int per_sm = 1;
    int s = pulse_shape(mode, false, w->G, w->tune_warps, w->tune_per_sm, &per_sm, threads, smem, path);
    if (s) return s;
    *grid = w->num_sms * per_sm;
    memcpy(w->geo_key, key, sizeof(key));
    w->geo_grid = *grid;
    w->geo_threads = *threads;
    w->geo_smem = *smem;
    return RSC_OK;
}

/* One time step: the background kernel (its mode chosen at compile time) on
 * the worker's stream and the debris kernel beside it on the side stream,
 * joined back before anything later on the worker's stream.  Returns the
 * number of launches. */
cudaError_t launch_advance(rsc_worker *w, const AdvanceArgs &a, unsigned blocks, int *launched, cudaStream_t st) {
    const unsigned deb_blocks = blocks - a.rain_blocks;
    cudaError_t e = cudaSuccess;
    *launched = 0;
    if (deb_blocks) {
        e = cudaEventRecord(w->fork_ev, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(w->side, w->fork_ev, 0);
        if (e != cudaSuccess) return e;
        rsc::k_advance_debris<<<deb_blocks, rsc::kAdvanceThreads, 0, w->side>>>(a);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(w->join_ev, w->side);
        if (e != cudaSuccess) return e;
        (*launched)++;
    }
    if (a.rain_blocks) {
        const bool stretched = rsm_f2u(a.wind[7]) == 7u;   /* the LES index form, fixed per LES */
        const unsigned pair_blocks = (unsigned)((a.rain_count + 2 * rsc::kAdvanceThreads - 1) / (2 * rsc::kAdvanceThreads));
        if (w->adv_per_thread == 2 && a.rain_mode != 2) {
            if (a.rain_mode == 1 && stretched) {
                rsc::k_advance_rain2<1, 7><<<pair_blocks, rsc::kAdvanceThreads, 0, st>>>(a);
            } else if (a.rain_mode == 1) {
                rsc::k_advance_rain2<1><<<pair_blocks, rsc::kAdvanceThreads, 0, st>>>(a);
            } else if (stretched) {
                rsc::k_advance_rain2<0, 7><<<pair_blocks, rsc::kAdvanceThreads, 0, st>>>(a);
            } else {
                rsc::k_advance_rain2<0><<<pair_blocks, rsc::kAdvanceThreads, 0, st>>>(a);
            }
        } else if (a.rain_mode == 1 && stretched) {
            rsc::k_advance_rain<1, 7><<<a.rain_blocks, rsc::kAdvanceThreads, 0, st>>>(a);
        } else if (a.rain_mode == 1) {
            rsc::k_advance_rain<1><<<a.rain_blocks, rsc::kAdvanceThreads, 0, st>>>(a);
        } else if (a.rain_mode == 0 && stretched) {
            rsc::k_advance_rain<0, 7><<<a.rain_blocks, rsc::kAdvanceThreads, 0, st>>>(a);
        } else if (a.rain_mode == 0) {
            rsc::k_advance_rain<0><<<a.rain_blocks, rsc::kAdvanceThreads, 0, st>>>(a);
        } else {
            rsc::k_advance_rain<2><<<a.rain_blocks, rsc::kAdvanceThreads, 0, st>>>(a);
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        (*launched)++;
    }
    if (deb_blocks) e = cudaStreamWaitEvent(st, w->join_ev, 0);
    return e;
}

void launch_pulse(int mode, const PulseArgs &P, int grid, int threads, size_t smem, cudaStream_t st) {
    pulse_kernel(mode, pulse_path(P, mode))<<<grid, threads, smem, st>>>(P);
}

/* The compensated form's interval moments (PulseArgs::mom_n): on the
 * triangle range table whose support, 1 / scale, is a whole number of gate
 * spacings (up to rsc::kMomMaxN), taken by the grouped pulse path. */
int moment_span(const PulseArgs &P) {
    if (!P.rw_tri || P.dense || !(P.rdelta > 0.0f) || !(P.rwd[0] > 0.0f)) return 0;
    const double x = 1.0 / ((double)P.rwd[0] * (double)P.rdelta);
    const double n = floor(x + 0.5);
    if (n < 1.0 || n > (double)rsc::kMomMaxN || fabs(x - n) > 1.0e-6 * n) return 0;
    return (int)n;
}

/* The margin, in gates, by which the sparse path widens the exact support
 * d_lo .. d_hi (metres) of the range weight: the measured drift of the FP32
 * running-sum gate origins from exact spacing; two ulps of the largest range
 * a window can reach (the rounding of r - r0 and of the gate origins there);
 * and a few FP32 roundings of g = (r - r0) / delta, of the window bounds and
 * of the weight's raw index, relative to the gate span, with a floor of 1e-4
 * gate.  A gate outside the widened window gets an exactly zero weight. */
double window_margin(double drift, float range_start, float range_delta, uint32_t G, double d_lo, double d_hi) {
    const double delta = (double)range_delta;
    const double span = (double)G + (fabs(d_lo) + fabs(d_hi)) / delta + 2.0;
    const double r_max = fabs((double)range_start) + delta * span;
    const double ulp_r = ldexp(1.0, ilogb(r_max) - 23);
    return (drift + 2.0 * ulp_r) / delta + 8.0 * ldexp(1.0, -23) * span + 1.0e-4;
}

void fill_pulse_args(rsc_worker *w, PulseArgs &P, const float *sim) {
    memset(&P, 0, sizeof(P));
    P.pos = w->pos;
    P.rcs = w->rcs;
    P.aux = w->aux;
    P.sig = w->sig;
    P.n = w->num_scats;
    P.aw = w->angular_weight;
    memcpy(P.awd, w->angular_desc, sizeof(P.awd));
    P.rw = w->range_weight;
    memcpy(P.rwd, w->range_desc, sizeof(P.rwd));
    P.rk = w->rk;
    P.rk_lo = w->rk_lo;
    P.rk64 = w->rk64;
    P.G = w->G;
    memcpy(P.sim, sim, sizeof(P.sim));
    rsc::beam_norm_df(P.sim, P.bn_hi, P.bn_lo);
    P.rs = w->range_start;
    P.inv_delta = w->range_delta != 0.0f ? 1.0f / w->range_delta : 0.0f;
    P.rdelta = w->range_delta;
    P.rw_n = w->range_n;
    memcpy(P.rwv, w->range_weight_small, sizeof(P.rwv));
    P.rw_tri = is_triangle(w->range_n, w->range_weight_small, w->range_desc) ? 1 : 0;
    P.acc64 = w->acc64;
    P.counter = w->counter;
    P.coherent_span = w->perm != nullptr ? (int)w->G + 1 : 0;
    P.pulse = w->pulse;
    P.pulse64 = w->pulse64;
    /* Candidate window of the sparse path.  The weight is W[0] or W[xm] when
     * the table index clamps, so when both edge values are 0 only gates with
     * 0 < (r - r_k) * xs + x0 < xm can receive a non-zero weight; the window is
     * that interval in gate units plus a margin for the FP32 running sum of
     * the gate origins and the rounding of the window arithmetic. */
    P.dense = 1;
    const float xs = w->range_desc[0], x0 = w->range_desc[1], xm = w->range_desc[2];
    if (w->range_delta > 0.0f && xs > 0.0f && xm >= 0.0f && w->range_n > 0) {
        uint32_t im = (uint32_t)xm;
        if (im < w->range_n && w->range_weight_host0 == 0.0f && w->range_weight_hostm == 0.0f) {
            double d_lo = -(double)x0 / (double)xs;
            double d_hi = ((double)xm - (double)x0) / (double)xs;
            double drift = 0.0, r = w->range_start;
            float rf = w->range_start;
            for (uint32_t k = 0; k < w->G; k++) {
                drift = fmax(drift, fabs((double)rf - r));
                rf = rf + w->range_delta;
                r += (double)w->range_delta;
            }
            const double margin = window_margin(drift, w->range_start, w->range_delta, w->G, d_lo, d_hi);
            double lo = d_lo / (double)w->range_delta - margin;
            double hi = d_hi / (double)w->range_delta + margin;
            if (hi - lo + 1.0 < (double)rsc::kMaxCandidates) {
                P.dense = 0;
                P.win_lo = (float)lo;
                P.win_hi = (float)hi;
            }
        }
    }
}

}  // namespace

extern "C" {

const char *rsc_last_error(void) { return g_err; }

int rsc_device_count(int *count) {
    if (count == nullptr) return fail(RSC_ERR_ARG, "count is NULL");
    int n = 0;
    RSC_CUDA(cudaGetDeviceCount(&n));
    *count = n;
    return RSC_OK;
}

int rsc_worker_create(int device, rsc_worker **out) {
    if (out == nullptr) return fail(RSC_ERR_ARG, "out is NULL");
    *out = nullptr;
    int n = 0;
    RSC_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(RSC_ERR_ARG, "device %d of %d", device, n);
    RSC_CUDA(cudaSetDevice(device));
    rsc_worker *w = new rsc_worker();
    w->device = device;
    cudaError_t e = cudaDeviceGetAttribute(&w->num_sms, cudaDevAttrMultiProcessorCount, device);
    /* Priorities: the debris kernel's few blocks take SM slots ahead of the
     * background kernel's queued blocks, so they run beside it rather than
     * after it; the pulse (worker's stream) is dispatched ahead of the
     * background advance of the same step, which fills the slots it leaves
     * (a free-running loop measured 77 against 90 us per step with equal
     * priorities, when the advance's blocks could take every slot first). */
    int prio_least = 0, prio_greatest = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    const int prio_main = prio_greatest < prio_least ? prio_greatest + 1 : prio_greatest;
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&w->stream, cudaStreamNonBlocking, prio_main);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&w->side, cudaStreamNonBlocking, prio_greatest);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->fork_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->join_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&w->adv, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->ev_read, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->ev_read_next, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->ev_adv, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->ev_main, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        delete w;
        return cuda_fail(RSC_ERR_CUDA, "worker creation: %s", cudaGetErrorString(e));
    }
    *out = w;
    return RSC_OK;
}

int rsc_worker_free(rsc_worker *w) {
    if (w == nullptr) return RSC_OK;
    cudaSetDevice(w->device);
    if (w->adv) cudaStreamSynchronize(w->adv);
    if (w->stream) cudaStreamSynchronize(w->stream);
    if (w->les_copy) cudaStreamSynchronize(w->les_copy);
    free_arrays(w);
    free_ptr(w->range_weight);
    free_ptr(w->angular_weight);
    free_ptr(w->ellipsoid);
    for (int s = 0; s < 2; s++) {
        free_ptr(w->les_uvwt[s]);
        free_ptr(w->les_cpxx[s]);
        free_ptr(w->dff[s]);
    }
    for (int t = 0; t < RSC_MAX_TYPES; t++) {
        free_ptr(w->adm[t].a);
        free_ptr(w->adm[t].b);
        free_ptr(w->rcs_tab[t].a);
        free_ptr(w->rcs_tab[t].b);
    }
    if (w->les_copy) {
        cudaStreamSynchronize(w->les_copy);
        cudaStreamDestroy(w->les_copy);
    }
    free_ptr(w->les_raw);
    free_ptr(w->les_stage);
    if (w->les_mark) cudaEventDestroy(w->les_mark);
    for (int s = 0; s < 2; s++) {
        if (w->les_ready[s]) cudaEventDestroy(w->les_ready[s]);
    }
    if (w->side) {
        cudaStreamSynchronize(w->side);
        cudaStreamDestroy(w->side);
    }
    if (w->d2h) {
        cudaStreamSynchronize(w->d2h);
        cudaStreamDestroy(w->d2h);
    }
    if (w->pulse_ev) cudaEventDestroy(w->pulse_ev);
    if (w->d2h_done) cudaEventDestroy(w->d2h_done);
    if (w->adv) cudaStreamDestroy(w->adv);
    cudaEvent_t evs[] = {w->ev_read, w->ev_read_next, w->ev_adv, w->ev_main};
    for (cudaEvent_t e : evs) {
        if (e) cudaEventDestroy(e);
    }
    if (w->fork_ev) cudaEventDestroy(w->fork_ev);
    if (w->join_ev) cudaEventDestroy(w->join_ev);
    if (w->stream) cudaStreamDestroy(w->stream);
    delete w;
    return RSC_OK;
}

int rsc_worker_malloc(rsc_worker *w, size_t num_scats, float range_start, float range_delta, uint32_t range_count) {
    int s = check_worker(w);
    if (s) return s;
    if (num_scats == 0) return fail(RSC_ERR_ARG, "num_scats is 0");
    if (range_count == 0 || range_count > RSC_MAX_GATES) {
        return fail(RSC_ERR_ARG, "range_count %u outside [1, %d]", range_count, RSC_MAX_GATES);
    }
    if (!(fabsf(range_start) < INFINITY) || !(fabsf(range_delta) < INFINITY)) {
        return fail(RSC_ERR_ARG, "range_start / range_delta not finite");
    }
    cudaStreamSynchronize(w->adv);
    cudaStreamSynchronize(w->stream);
    w->pend = false;
    free_arrays(w);
    const size_t numel = (num_scats + 63) / 64 * 64;
    const size_t b4 = numel * sizeof(float4);
    w->num_scats = num_scats;
    w->numel = numel;
    w->G = range_count;
    w->range_start = range_start;
    w->range_delta = range_delta;
    float4 **arrays[] = {&w->pos, &w->vel, &w->ori, &w->tum, &w->aux, &w->rcs, &w->sig, &w->pos_next, &w->rcs_next};
    for (float4 **a : arrays) {
        cudaError_t e = cudaMalloc((void **)a, b4);
        if (e != cudaSuccess) {
            free_arrays(w);
            return cuda_fail(RSC_ERR_NOMEM, "cudaMalloc of %zu B: %s", b4, cudaGetErrorString(e));
        }
        RSC_CUDA(cudaMemsetAsync(*a, 0, b4, w->stream));
    }
    RSC_CUDA(cudaMalloc((void **)&w->rnd, numel * sizeof(uint4)));
    RSC_CUDA(cudaMemsetAsync(w->rnd, 0, numel * sizeof(uint4), w->stream));
    RSC_CUDA(cudaMalloc((void **)&w->pulse, range_count * sizeof(float4)));
    RSC_CUDA(cudaMemsetAsync(w->pulse, 0, range_count * sizeof(float4), w->stream));
    RSC_CUDA(cudaMalloc((void **)&w->pulse64, range_count * 4 * sizeof(double)));
    RSC_CUDA(cudaMalloc((void **)&w->rk, range_count * sizeof(float)));
    RSC_CUDA(cudaMalloc((void **)&w->rk_hi, range_count * sizeof(float)));
    RSC_CUDA(cudaMalloc((void **)&w->rk_lo, range_count * sizeof(float)));
    RSC_CUDA(cudaMalloc((void **)&w->rk64, range_count * sizeof(double)));
    /* the pulse kernel's FP64 accumulator; each launch leaves it at zero */
    RSC_CUDA(cudaMalloc((void **)&w->acc64, range_count * 4 * sizeof(double)));
    RSC_CUDA(cudaMemsetAsync(w->acc64, 0, range_count * 4 * sizeof(double), w->stream));
    RSC_CUDA(cudaMalloc((void **)&w->counter, sizeof(unsigned)));
    RSC_CUDA(cudaMemsetAsync(w->counter, 0, sizeof(unsigned), w->stream));
    RSC_CUDA(cudaMalloc((void **)&w->runs, sizeof(unsigned long long)));
    RSC_CUDA(cudaMemsetAsync(w->runs, 0, sizeof(unsigned long long), w->stream));
    s = set_gates(w);
    if (s) return s;
    RSC_CUDA(cudaStreamSynchronize(w->stream));
    w->sig_aux_stale = false;
    w->have_pulse_desc = false;
    return RSC_OK;
}

int rsc_set_range_weight(rsc_worker *w, const float *table, uint32_t n, const float desc[4]) {
    int s = check_worker(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    if (table == nullptr || desc == nullptr || n == 0) return fail(RSC_ERR_ARG, "range weight table");
    if (!(desc[2] >= 0.0f) || (uint32_t)desc[2] >= n) return fail(RSC_ERR_ARG, "range weight max index %g >= %u", desc[2], n);
    cudaStreamSynchronize(w->stream);
    s = upload_floats(&w->range_weight, table, n);
    if (s) return s;
    w->range_n = n;
    memcpy(w->range_desc, desc, sizeof(w->range_desc));
    w->range_weight_host0 = table[0];
    w->range_weight_hostm = table[(uint32_t)desc[2]];
    for (uint32_t k = 0; k < 4; k++) w->range_weight_small[k] = k < n ? table[k] : 0.0f;
    return RSC_OK;
}

int rsc_set_angular_weight(rsc_worker *w, const float *table, uint32_t n, const float desc[4]) {
    int s = check_worker(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    if (table == nullptr || desc == nullptr || n == 0) return fail(RSC_ERR_ARG, "angular weight table");
    if (!(desc[2] >= 0.0f) || (uint32_t)desc[2] >= n) return fail(RSC_ERR_ARG, "angular weight max index %g >= %u", desc[2], n);
    cudaStreamSynchronize(w->stream);
    s = upload_floats(&w->angular_weight, table, n);
    if (s) return s;
    w->angular_n = n;
    memcpy(w->angular_desc, desc, sizeof(w->angular_desc));
    return RSC_OK;
}

int rsc_set_rcs_ellipsoid(rsc_worker *w, const float *table4, uint32_t n, const float desc[4]) {
    int s = check_worker(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    if (table4 == nullptr || desc == nullptr || n == 0) return fail(RSC_ERR_ARG, "ellipsoid RCS table");
    if (!(desc[2] >= 0.0f) || (uint32_t)desc[2] >= n) return fail(RSC_ERR_ARG, "ellipsoid max index %g >= %u", desc[2], n);
    cudaStreamSynchronize(w->stream);
    s = upload_float4(&w->ellipsoid, table4, n);
    if (s) return s;
    w->ellipsoid_n = n;
    memcpy(w->ellipsoid_desc, desc, sizeof(w->ellipsoid_desc));
    return release_main(w);
}

/* The worker's stream waits for an asynchronous pulse copy before the pulse
 * is rewritten. */
static int pulse_d2h_wait(rsc_worker *w) {
    if (!w->d2h_pending) return RSC_OK;
    RSC_CUDA(cudaStreamWaitEvent(w->stream, w->d2h_done, 0));
    w->d2h_pending = false;
    return RSC_OK;
}

/* Make the worker's stream wait for a pending remap into LES slot `slot`. */
static int les_slot_wait(rsc_worker *w, int slot, cudaStream_t st) {
    if (!w->les_wait[slot]) return RSC_OK;
    RSC_CUDA(cudaStreamWaitEvent(st, w->les_ready[slot], 0));
    w->les_wait[slot] = false;
    return RSC_OK;
}

/* Both LES slots allocated for nx x ny x nz texels. */
static int ensure_les_slots(rsc_worker *w, uint32_t nx, uint32_t ny, uint32_t nz) {
    const size_t nn = (size_t)nx * ny * nz;
    if (((size_t)nx + 2) * ny * nz >= (1ull << 31)) {
        return fail(RSC_ERR_UNSUPPORTED, "LES of %zu texels (the kernels index below 2^31)", nn);
    }
    if (w->les_uvwt[0] != nullptr && (nx != w->les_nx || ny != w->les_ny || nz != w->les_nz)) {
        /* new dimensions: reallocate both slots (rs.c:3000-3016 releases them) */
        cudaStreamSynchronize(w->stream);
        if (w->les_copy) cudaStreamSynchronize(w->les_copy);
        w->les_wait[0] = w->les_wait[1] = false;
        for (int k = 0; k < 2; k++) {
            free_ptr(w->les_uvwt[k]);
            free_ptr(w->les_cpxx[k]);
            w->les_uvwt[k] = w->les_cpxx[k] = nullptr;
        }
    }
    if (w->les_uvwt[0] == nullptr) {
        for (int k = 0; k < 2; k++) {
            RSC_CUDA(cudaMalloc((void **)&w->les_uvwt[k], les_pair_float4s(nx, ny, nz) * sizeof(float4)));
            RSC_CUDA(cudaMalloc((void **)&w->les_cpxx[k], nn * sizeof(float4)));
            RSC_CUDA(cudaMemsetAsync(w->les_cpxx[k], 0, nn * sizeof(float4), w->stream));
        }
        w->les_nx = nx;
        w->les_ny = ny;
        w->les_nz = nz;
    }
    return RSC_OK;
}

static int set_les_impl(rsc_worker *w, int slot, const float *uvwt4, const float *cpxx4, uint32_t nx, uint32_t ny,
                        uint32_t nz, const float desc[16], bool async) {
    int s = check_worker(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    if (slot < 0 || slot > 1) return fail(RSC_ERR_ARG, "LES slot %d", slot);
    if (uvwt4 == nullptr || desc == nullptr || nx == 0 || ny == 0 || nz == 0) return fail(RSC_ERR_ARG, "LES table");
    s = ensure_les_slots(w, nx, ny, nz);
    if (s) return s;
    s = les_slot_wait(w, slot, w->stream);
    if (s) return s;
    const size_t nn = (size_t)nx * ny * nz;
    s = ensure_buffer(&w->les_stage, &w->les_stage_n, nn, w->stream);
    if (s) return s;
    RSC_CUDA(cudaMemcpyAsync(w->les_stage, uvwt4, nn * sizeof(float4), cudaMemcpyHostToDevice, w->stream));
    rsc::k_les_pairs<<<les_grid(nx, (size_t)ny * nz), rsc::kLesThreads, 0, w->stream>>>(w->les_stage, (int)nx,
                                                                                      (size_t)ny * nz, w->les_uvwt[slot]);
    RSC_CUDA(cudaGetLastError());
    w->launches++;
    if (cpxx4) {
        RSC_CUDA(cudaMemcpyAsync(w->les_cpxx[slot], cpxx4, nn * sizeof(float4), cudaMemcpyHostToDevice, w->stream));
    }
    memcpy(w->les_desc, desc, sizeof(w->les_desc));
    if (!async) RSC_CUDA(cudaStreamSynchronize(w->stream));
    return release_main(w);
}

int rsc_set_les(rsc_worker *w, int slot, const float *uvwt4, const float *cpxx4, uint32_t nx, uint32_t ny, uint32_t nz,
                const float desc[16]) {
    return set_les_impl(w, slot, uvwt4, cpxx4, nx, ny, nz, desc, false);
}

int rsc_set_les_async(rsc_worker *w, int slot, const float *uvwt4, const float *cpxx4, uint32_t nx, uint32_t ny,
                      uint32_t nz, const float desc[16]) {
    return set_les_impl(w, slot, uvwt4, cpxx4, nx, ny, nz, desc, true);
}

int rsc_les_upload_async(rsc_worker *w, rsc_les_source *src, int slot, uint32_t frame, float *time) {
    int s = check_worker(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    if (src == nullptr) return fail(RSC_ERR_ARG, "LES source is NULL");
    if (slot < 0 || slot > 1) return fail(RSC_ERR_ARG, "LES slot %d", slot);
    const rsc_les_info &I = rscles::info(src);
    if (frame >= I.frames) return fail(RSC_ERR_ARG, "LES frame %u of %u", frame, I.frames);
    s = ensure_les_slots(w, I.nx, I.ny, I.nz);
    if (s) return s;
    const size_t nn = (size_t)I.nx * I.ny * I.nz;
    if (w->les_copy == nullptr) {
        RSC_CUDA(cudaStreamCreateWithFlags(&w->les_copy, cudaStreamNonBlocking));
        RSC_CUDA(cudaEventCreateWithFlags(&w->les_mark, cudaEventDisableTiming));
        for (int k = 0; k < 2; k++) RSC_CUDA(cudaEventCreateWithFlags(&w->les_ready[k], cudaEventDisableTiming));
    }
    /* the staging buffer is reused in copy-stream order */
    s = ensure_buffer(&w->les_raw, &w->les_raw_n, 5 * nn, w->les_copy);
    if (s) return s;
    rscles::Held h;
    const char *why = "";
    s = rscles::acquire(src, frame, &h, &why);
    if (s) return fail(s, "LES frame %u: %s", frame, why);
    if (rscles::pin(src, h, &why) != RSC_OK) {
        /* pageable: the copy is staged by the driver, still correct */
    }
    cudaError_t e = cudaMemcpyAsync(w->les_raw, h.planes, 5 * nn * sizeof(float), cudaMemcpyHostToDevice, w->les_copy);
    rscles::release(src, h, e == cudaSuccess ? w->les_copy : nullptr);
    if (e != cudaSuccess) return cuda_fail(RSC_ERR_CUDA, "LES frame copy: %s", cudaGetErrorString(e));
    /* the slot is rewritten after the work queued on the worker so far (its
     * advance stream included: flush_pending made the worker's stream wait
     * for it) */
    RSC_CUDA(cudaEventRecord(w->les_mark, w->stream));
    RSC_CUDA(cudaStreamWaitEvent(w->les_copy, w->les_mark, 0));
    const size_t rows = (size_t)I.ny * I.nz;
    rsc::k_les_remap<<<les_grid(I.nx, rows), rsc::kLesThreads, 0, w->les_copy>>>(
        w->les_raw, (int)I.nx, rows, I.v0, I.p0, I.t0, I.p_for_cn2, w->les_uvwt[slot], w->les_cpxx[slot]);
    RSC_CUDA(cudaGetLastError());
    RSC_CUDA(cudaEventRecord(w->les_ready[slot], w->les_copy));
    w->les_wait[slot] = true;
    w->launches++;
    rsc_les_descriptor(&I, w->les_desc);
    if (time) *time = h.time;
    return RSC_OK;
}

static int set_table2d(rsc_worker *w, Table2D *t, const float *a4, const float *b4, uint32_t nx, uint32_t ny,
                       const float desc[16]) {
    int s0 = flush_pending(w);
    if (s0) return s0;
    if (a4 == nullptr || b4 == nullptr || desc == nullptr || nx == 0 || ny == 0) return fail(RSC_ERR_ARG, "2-D table");
    cudaStreamSynchronize(w->stream);
    const size_t nn = (size_t)nx * ny;
    if (nn >= (1ull << 31)) return fail(RSC_ERR_UNSUPPORTED, "2-D table of %zu texels (the kernels index below 2^31)", nn);
    int s = upload_float4(&t->a, a4, nn);
    if (s) return s;
    s = upload_float4(&t->b, b4, nn);
    if (s) return s;
    t->nx = nx;
    t->ny = ny;
    memcpy(t->desc, desc, sizeof(t->desc));
    return release_main(w);
}

int rsc_set_adm(rsc_worker *w, int index, const float *cd4, const float *cm4, uint32_t nx, uint32_t ny,
                const float desc[16]) {
    int s = check_worker(w);
    if (s) return s;
    if (index < 0 || index >= RSC_MAX_TYPES) return fail(RSC_ERR_ARG, "ADM index %d", index);
    return set_table2d(w, &w->adm[index], cd4, cm4, nx, ny, desc);
}

int rsc_set_rcs(rsc_worker *w, int index, const float *real4, const float *imag4, uint32_t nx, uint32_t ny,
                const float desc[16]) {
    int s = check_worker(w);
    if (s) return s;
    if (index < 0 || index >= RSC_MAX_TYPES) return fail(RSC_ERR_ARG, "RCS index %d", index);
    return set_table2d(w, &w->rcs_tab[index], real4, imag4, nx, ny, desc);
}

int rsc_set_dff(rsc_worker *w, int slot, const float *icdf, uint32_t n, const float desc[16]) {
    int s = check_worker(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    if (slot < 0 || slot > 1 || icdf == nullptr || desc == nullptr || n == 0) return fail(RSC_ERR_ARG, "DFF table");
    /* db_atts reads icdf[floor(clamp(r * sf + {0, 1}, 0, sf))] (rs.cl:799-805) */
    if (!(desc[15] >= 0.0f && desc[15] < (float)n)) return fail(RSC_ERR_ARG, "DFF max index %g >= %u", desc[15], n);
    cudaStreamSynchronize(w->stream);
    s = upload_floats(&w->dff[slot], icdf, n);
    if (s) return s;
    w->dff_n = n;
    memcpy(w->dff_desc, desc, sizeof(w->dff_desc));
    return release_main(w);
}

static unsigned grid_of(unsigned long long n, unsigned threads) { return (unsigned)((n + threads - 1) / threads); }

/* Counting sort of the background range into spatial order: range shells
 * of a quarter gate, then Morton order of direction, over the scan box
 * (sim_desc s8-s10 origin, s12-s14 size): rsc_sort.cuh.  Every
 * attribute array and perm move to the second buffer set, which then becomes
 * the current one. */
static int sort_worker(rsc_worker *w, const rsc_population *pop, const float *sim, cudaStream_t st) {
    const unsigned long long origin = pop->origins[0], count = pop->counts[0];
    w->sort_due = false;
    w->since_sort = 0;
    if (count < 256 || origin + count > w->num_scats) return RSC_OK;
    const unsigned long long numel = w->numel;
    if (w->perm == nullptr) {
        const size_t u4 = numel * sizeof(unsigned);
        cudaError_t e = cudaMalloc((void **)&w->perm, u4);
        if (e == cudaSuccess) e = cudaMalloc((void **)&w->perm_alt, u4);
        if (e == cudaSuccess) e = cudaMalloc((void **)&w->inv, u4);
        if (e == cudaSuccess) e = cudaMalloc((void **)&w->sort_key, u4);
        if (e == cudaSuccess) e = cudaMalloc((void **)&w->sort_order, u4);
        if (e == cudaSuccess) e = cudaMalloc((void **)&w->sort_hist, sizeof(unsigned) * rsc::kMaxSortCells);
        if (e == cudaSuccess) e = cudaMalloc((void **)&w->sort_blocks, sizeof(unsigned) * rsc::kScanBlock);
        for (int k = 0; k < 8 && e == cudaSuccess; k++) e = cudaMalloc((void **)&w->alt[k], numel * sizeof(uint4));
        if (e != cudaSuccess) {
            free_sort(w);
            w->sort_due = false;
            return cuda_fail(RSC_ERR_NOMEM, "spatial-order buffers for %llu scatterers: %s", numel, cudaGetErrorString(e));
        }
        rsc::k_iota<<<grid_of(numel, rsc::kSortThreads), rsc::kSortThreads, 0, st>>>(w->perm, numel);
        rsc::k_iota<<<grid_of(numel, rsc::kSortThreads), rsc::kSortThreads, 0, st>>>(w->inv, numel);
        w->launches += 2;
    }
    /* range shells of a quarter gate over the box's range, direction cells
     * over its direction cosines, about one scatterer per cell, at most
     * kMaxSortCells cells */
    double r_lo = INFINITY, r_hi = 0.0, u_lo = INFINITY, u_hi = -INFINITY, v_lo = INFINITY, v_hi = -INFINITY;
    for (int c = 0; c < 8; c++) {
        const double x = (double)sim[8] + ((c & 1) ? (double)sim[12] : 0.0);
        const double y = (double)sim[9] + ((c & 2) ? (double)sim[13] : 0.0);
        const double z = (double)sim[10] + ((c & 4) ? (double)sim[14] : 0.0);
        const double r = sqrt(x * x + y * y + z * z);
        if (!(r > 0.0)) continue;
        r_lo = fmin(r_lo, r);
        r_hi = fmax(r_hi, r);
        u_lo = fmin(u_lo, x / r);
        u_hi = fmax(u_hi, x / r);
        v_lo = fmin(v_lo, z / r);
        v_hi = fmax(v_hi, z / r);
    }
    if (!(r_hi > r_lo) || !(u_hi > u_lo) || !(v_hi > v_lo)) {
        r_lo = 0.0, r_hi = 1.0, u_lo = -1.0, u_hi = 1.0, v_lo = -1.0, v_hi = 1.0;
    }
    double shell = fabs((double)w->range_delta) * 0.25;
    if (!(shell > 0.0)) shell = (r_hi - r_lo) / 64.0;
    double shells_d = ceil((r_hi - r_lo) / shell);
    if (shells_d < 1.0) shells_d = 1.0;
    if (shells_d > (double)(rsc::kMaxSortCells / 4)) shells_d = (double)(rsc::kMaxSortCells / 4);
    const unsigned shells = (unsigned)shells_d;
    unsigned bits = (unsigned)lrint(0.5 * log2(fmax((double)count / shells, 1.0)));
    if (bits > 12) bits = 12;
    while (bits > 0 && ((unsigned long long)shells << (2 * bits)) > rsc::kMaxSortCells) bits--;
    const unsigned H = shells << (2 * bits);
    RSC_CUDA(cudaMemsetAsync(w->sort_hist, 0, H * sizeof(unsigned), st));
    rsc::SortArgs a;
    a.pos = w->pos;
    a.origin = origin;
    a.count = count;
    a.r0 = (float)r_lo;
    a.ir = (float)(1.0 / (shells * shell));
    a.u0 = (float)u_lo;
    a.iu = (float)(1.0 / (u_hi - u_lo));
    a.v0 = (float)v_lo;
    a.iv = (float)(1.0 / (v_hi - v_lo));
    a.shells = shells;
    a.bits = bits;
    a.key = w->sort_key;
    a.hist = w->sort_hist;
    rsc::k_sort_key<<<grid_of(count, rsc::kSortThreads), rsc::kSortThreads, 0, st>>>(a);
    const unsigned nb = (H + rsc::kScanBlock - 1) / rsc::kScanBlock;
    rsc::k_scan_blocks<<<nb, rsc::kScanThreads, 0, st>>>(w->sort_hist, H, w->sort_blocks);
    rsc::k_scan_top<<<1, rsc::kScanThreads, 0, st>>>(w->sort_blocks, nb);
    rsc::k_scan_add<<<nb, rsc::kScanThreads, 0, st>>>(w->sort_hist, H, w->sort_blocks);
    rsc::k_sort_scatter<<<grid_of(count, rsc::kSortThreads), rsc::kSortThreads, 0, st>>>(w->sort_key, count,
                                                                                        w->sort_hist, w->sort_order);
    uint4 **arr[8];
    attribute_arrays(w, arr);
    rsc::PermuteArgs p;
    for (int k = 0; k < 8; k++) {
        p.src[k] = *arr[k];
        p.dst[k] = w->alt[k];
    }
    p.perm_src = w->perm;
    p.perm_dst = w->perm_alt;
    p.origin = origin;
    p.count = count;
    p.numel = numel;
    p.order = w->sort_order;
    rsc::k_sort_permute<<<grid_of(numel, rsc::kSortThreads), rsc::kSortThreads, 0, st>>>(p);
    for (int k = 0; k < 8; k++) {
        uint4 *t = *arr[k];
        *arr[k] = w->alt[k];
        w->alt[k] = t;
    }
    unsigned *t = w->perm;
    w->perm = w->perm_alt;
    w->perm_alt = t;
    rsc::k_sort_inverse<<<grid_of(numel, rsc::kSortThreads), rsc::kSortThreads, 0, st>>>(w->perm, w->inv, numel);
    RSC_CUDA(cudaGetLastError());
    w->launches += 8;
    w->sorts++;
    return RSC_OK;
}

/* aux / sig of the latest pulse (scat_sig_aux, rs.cl:1050-1110) when the
 * pulse kernel did not write them: formed on `st` from the pos / rcs pair
 * that pulse read and its descriptor.  rs.c's RS_download returns what the
 * last scat_sig_aux launch wrote, so they are formed before anything
 * overwrites or reorders that pair (a second advance, a sort, an upload, a
 * batch run), or on download. */
static int settle_sig_aux(rsc_worker *w, cudaStream_t st) {
    if (!w->sig_aux_stale || !w->have_pulse_desc) return RSC_OK;
    PulseArgs P;
    fill_pulse_args(w, P, w->last_sim);
    if (w->sa_pos != nullptr) {
        P.pos = w->sa_pos;
        P.rcs = w->sa_rcs;
    }
    const unsigned blocks = (unsigned)((w->num_scats + 255) / 256);
    rsc::k_sig_aux<<<blocks, 256, 0, st>>>(P);
    RSC_CUDA(cudaGetLastError());
    w->launches++;
    w->sig_aux_stale = false;
    return RSC_OK;
}

/* Sort when the interval has passed or the state was replaced. */
static int maybe_sort(rsc_worker *w, const rsc_population *pop, const float *sim, cudaStream_t st) {
    if (w->sort_interval <= 0) return RSC_OK;
    if (!w->sort_due && w->since_sort < (uint64_t)w->sort_interval) return RSC_OK;
    /* the arrays move: after the advance stream, before its next advance */
    int s = join_adv(w);
    if (s) return s;
    s = settle_sig_aux(w, st);
    if (s) return s;
    s = sort_worker(w, pop, sim, st);
    if (s) return s;
    return release_main(w);
}

}  // extern "C"

namespace {

/* Run a recorded advance on its own and do its bookkeeping. */
int flush_pending(rsc_worker *w) {
    int s = join_adv(w);
    if (s) return s;
    if (!w->pend) return RSC_OK;
    w->pend = false;
    if (w->pend_blocks) {
        /* the fused form's advance, in place on the worker's stream */
        int n = 0;
        RSC_CUDA(launch_advance(w, w->pend_a, w->pend_blocks, &n, w->stream));
        w->launches += n;
        s = release_main(w);
        if (s) return s;
    }
    w->since_sort++;
    return maybe_sort(w, &w->pend_pop, w->pend_sim, w->stream);
}

/* Launch shape of the step kernel: 256 threads (the advance's blocks), the
 * pulse bins of its 8 warps, as many resident blocks as fit (at most 8). */
int step_shape(int mode, rsc_worker *w, int *grid, size_t *smem) {
    *smem = (size_t)(rsc::kAdvanceThreads / 32) * rsc::pulse_warp_bytes(mode, w->G) + 2 * w->G * sizeof(float);
    int per_sm = 1;
    cudaError_t e = mode == RSC_PULSE_PLAIN
                        ? kernel_occupancy(rsc::k_step<0>, rsc::kAdvanceThreads, *smem, &per_sm)
                        : kernel_occupancy(rsc::k_step<1>, rsc::kAdvanceThreads, *smem, &per_sm);
    if (e != cudaSuccess) return cuda_fail(RSC_ERR_CUDA, "step kernel configuration: %s", cudaGetErrorString(e));
    if (per_sm < 1) per_sm = 1;
    if (per_sm > 8) per_sm = 8;
    *grid = w->num_sms * per_sm;
    return RSC_OK;
}

}  // namespace

extern "C" {

}  // extern "C"

namespace rsc {
/* the constant part of RS_populate's state (rs.c:4672-4744): zero velocity,
 * the attitude facing the beam, no tumbling, unit RCS, no signal; slots past
 * the populated ones zero */
__global__ void __launch_bounds__(256) k_fill_population(float4 *vel, float4 *ori, float4 *tum, float4 *rcs,
                                                         float4 *sig, unsigned long long used,
                                                         unsigned long long numel) {
    const unsigned long long i = (unsigned long long)blockIdx.x * 256 + threadIdx.x;
    if (i >= numel) return;
    const bool u = i < used;
    const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    vel[i] = z;
    sig[i] = z;
    ori[i] = u ? make_float4(0.5f, -0.5f, -0.5f, 0.5f) : z;
    tum[i] = u ? make_float4(0.0f, 0.0f, 0.0f, 1.0f) : z;
    rcs[i] = u ? make_float4(1.0f, 0.0f, 1.0f, 0.0f) : z;
}
}  // namespace rsc

extern "C" {

int rsc_populate_upload(rsc_worker *w, const rsc_populate_args *args, uint32_t *dsd_pop) {
    int s = check_alloc(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    if (args == nullptr) return fail(RSC_ERR_ARG, "args is NULL");
    rscpop::Generator g;
    const char *why = "";
    s = g.init(args, &why);
    if (s) return fail(s, "%s", why);
    if (g.total > w->num_scats) return fail(RSC_ERR_ARG, "the type ranges exceed the %zu scatterers", w->num_scats);
    if (dsd_pop && args->dsd_count) memset(dsd_pop, 0, args->dsd_count * sizeof(uint32_t));
    RSC_CUDA(cudaStreamSynchronize(w->stream));
    free_sort(w);   /* the state is replaced: slots in the caller's order again */
    const size_t chunk = (size_t)1 << 20;
    float *hp[2] = {nullptr, nullptr}, *ha[2] = {nullptr, nullptr};
    uint32_t *hr[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t e = cudaSuccess;
    for (int b = 0; b < 2 && e == cudaSuccess; b++) {
        e = cudaMallocHost((void **)&hp[b], chunk * 16);
        if (e == cudaSuccess) e = cudaMallocHost((void **)&ha[b], chunk * 16);
        if (e == cudaSuccess) e = cudaMallocHost((void **)&hr[b], chunk * 16);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming);
    }
    bool used[2] = {false, false};
    for (size_t c = 0; e == cudaSuccess && c < g.total; c += chunk) {
        const int b = (int)((c / chunk) & 1);
        if (used[b]) e = cudaEventSynchronize(ev[b]);   /* the copies out of this buffer are done */
        if (e != cudaSuccess) break;
        const size_t n = g.total - c < chunk ? g.total - c : chunk;
        g.fill(n, hp[b], ha[b], hr[b], dsd_pop);   /* overlaps the copies of the other buffer */
        e = cudaMemcpyAsync(w->pos + c, hp[b], n * 16, cudaMemcpyHostToDevice, w->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(w->aux + c, ha[b], n * 16, cudaMemcpyHostToDevice, w->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(w->rnd + c, hr[b], n * 16, cudaMemcpyHostToDevice, w->stream);
        if (e == cudaSuccess) e = cudaEventRecord(ev[b], w->stream);
        used[b] = true;
    }
    const size_t tail = w->numel - g.total;
    if (e == cudaSuccess && tail) e = cudaMemsetAsync(w->pos + g.total, 0, tail * 16, w->stream);
    if (e == cudaSuccess && tail) e = cudaMemsetAsync(w->aux + g.total, 0, tail * 16, w->stream);
    if (e == cudaSuccess && tail) e = cudaMemsetAsync(w->rnd + g.total, 0, tail * 16, w->stream);
    if (e == cudaSuccess) {
        rsc::k_fill_population<<<(unsigned)((w->numel + 255) / 256), 256, 0, w->stream>>>(
            w->vel, w->ori, w->tum, w->rcs, w->sig, g.total, w->numel);
        e = cudaGetLastError();
        w->launches++;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(w->stream);
    for (int b = 0; b < 2; b++) {
        if (hp[b]) cudaFreeHost(hp[b]);
        if (ha[b]) cudaFreeHost(ha[b]);
        if (hr[b]) cudaFreeHost(hr[b]);
        if (ev[b]) cudaEventDestroy(ev[b]);
    }
    if (e != cudaSuccess) return cuda_fail(RSC_ERR_CUDA, "populate: %s", cudaGetErrorString(e));
    w->sig_aux_stale = false;
    w->have_pulse_desc = false;
    w->sort_due = true;
    return release_main(w);
}

int rsc_set_fused_step(rsc_worker *w, int enable) {
    int s = check_worker(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    w->fuse = enable ? 1 : 0;
    return RSC_OK;
}

int rsc_upload(rsc_worker *w, size_t offset, size_t count, const float *pos4, const float *vel4, const float *ori4,
               const float *tum4, const float *aux4, const float *rcs4, const float *sig4, const uint32_t *rnd4) {
    int s = check_alloc(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    s = settle_sig_aux(w, w->stream);
    if (s) return s;
    if (offset + count > w->num_scats) return fail(RSC_ERR_ARG, "upload [%zu, %zu) beyond %zu", offset, offset + count, w->num_scats);
    const size_t b = count * 16;
    uint4 **arr[8];
    attribute_arrays(w, arr);
    const void *src[8] = {pos4, vel4, ori4, tum4, aux4, rcs4, sig4, rnd4};
    for (int k = 0; k < 8; k++) {
        if (src[k] == nullptr || count == 0) continue;
        if (w->perm == nullptr) {
            RSC_CUDA(cudaMemcpyAsync(*arr[k] + offset, src[k], b, cudaMemcpyHostToDevice, w->stream));
        } else {
            /* caller's order -> slots, through the idle second buffer */
            RSC_CUDA(cudaMemcpyAsync(w->alt[0], src[k], b, cudaMemcpyHostToDevice, w->stream));
            rsc::k_scatter16<<<grid_of(count, rsc::kSortThreads), rsc::kSortThreads, 0, w->stream>>>(
                *arr[k], w->alt[0], w->inv, offset, count);
            RSC_CUDA(cudaGetLastError());
            w->launches++;
        }
    }
    RSC_CUDA(cudaStreamSynchronize(w->stream));
    if (aux4 || sig4) w->sig_aux_stale = false;
    if (pos4) w->sort_due = true;
    return release_main(w);
}

int rsc_set_sort_interval(rsc_worker *w, int steps) {
    int s = check_worker(w);
    if (s) return s;
    if (steps < 0) return fail(RSC_ERR_ARG, "sort interval %d", steps);
    w->sort_interval = steps;
    return RSC_OK;
}

int rsc_sort_count(rsc_worker *w, uint64_t *count) {
    if (w == nullptr || count == nullptr) return fail(RSC_ERR_ARG, "NULL argument");
    *count = w->sorts;
    return RSC_OK;
}

int rsc_download(rsc_worker *w, size_t offset, size_t count, float *pos4, float *vel4, float *ori4, float *tum4,
                 float *aux4, float *rcs4, float *sig4, uint32_t *rnd4) {
    int s = check_alloc(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    if (offset + count > w->num_scats) return fail(RSC_ERR_ARG, "download [%zu, %zu) beyond %zu", offset, offset + count, w->num_scats);
    if (aux4 || sig4) {
        s = settle_sig_aux(w, w->stream);
        if (s) return s;
    }
    const size_t b = count * 16;
    uint4 **arr[8];
    attribute_arrays(w, arr);
    void *dst[8] = {pos4, vel4, ori4, tum4, aux4, rcs4, sig4, rnd4};
    for (int k = 0; k < 8; k++) {
        if (dst[k] == nullptr || count == 0) continue;
        if (w->perm == nullptr) {
            RSC_CUDA(cudaMemcpyAsync(dst[k], *arr[k] + offset, b, cudaMemcpyDeviceToHost, w->stream));
        } else {
            /* slots -> caller's order, through the idle second buffer */
            rsc::k_gather16<<<grid_of(count, rsc::kSortThreads), rsc::kSortThreads, 0, w->stream>>>(
                w->alt[0], *arr[k], w->inv, offset, count);
            RSC_CUDA(cudaGetLastError());
            w->launches++;
            RSC_CUDA(cudaMemcpyAsync(dst[k], w->alt[0], b, cudaMemcpyDeviceToHost, w->stream));
        }
    }
    RSC_CUDA(cudaStreamSynchronize(w->stream));
    return RSC_OK;
}

/* Scatterers outside every population range keep their pos / rcs: copied
 * into the pair an advance writes (nothing to copy when the ranges cover
 * the arrays, the usual case). */
static int copy_unadvanced(rsc_worker *w, const rsc_population *pop, cudaStream_t st) {
    std::vector<std::pair<unsigned long long, unsigned long long>> r;
    for (int k = 0; k < RSC_MAX_TYPES; k++) {
        if (pop->counts[k]) r.emplace_back(pop->origins[k], pop->origins[k] + pop->counts[k]);
    }
    std::sort(r.begin(), r.end());
    unsigned long long at = 0;
    r.emplace_back(w->num_scats, w->num_scats);
    for (const auto &q : r) {
        const unsigned long long lo = at, hi = std::min<unsigned long long>(q.first, w->num_scats);
        if (hi > lo) {
            RSC_CUDA(cudaMemcpyAsync(w->pos_next + lo, w->pos + lo, (hi - lo) * sizeof(float4), cudaMemcpyDeviceToDevice, st));
            RSC_CUDA(cudaMemcpyAsync(w->rcs_next + lo, w->rcs + lo, (hi - lo) * sizeof(float4), cudaMemcpyDeviceToDevice, st));
        }
        at = std::max(at, q.second);
    }
    return RSC_OK;
}

/* The advance launch of one worker: descriptor and block count. */
static int fill_advance_args(rsc_worker *w, const rsc_population *pop, int les_id, const float *sim_desc,
                             AdvanceArgs &a, unsigned *blocks_out) {
    if (pop == nullptr || sim_desc == nullptr) return fail(RSC_ERR_ARG, "population / sim_desc is NULL");
    if (les_id < 0 || les_id > 1 || w->les_uvwt[les_id] == nullptr) return fail(RSC_ERR_STATE, "LES slot %d not set", les_id);
    if (pop->origins[0] + pop->counts[0] > w->num_scats) return fail(RSC_ERR_ARG, "background range beyond the arrays");
    const uint32_t concept = rsm_f2u(sim_desc[5]);
    int s;
    memset(&a, 0, sizeof(a));
    a.pos_in = w->pos;
    a.rcs_in = w->rcs;
    a.pos = w->pos;
    a.vel = w->vel;
    a.ori = w->ori;
    a.tum = w->tum;
    a.rcs = w->rcs;
    a.rnd = w->rnd;
    a.uvwt = make_pair_image(w->les_uvwt[les_id], w->les_nx, w->les_ny, w->les_nz);
    a.cpxx = make_image(w->les_cpxx[les_id], w->les_nx, w->les_ny, w->les_nz);
    memcpy(a.wind, w->les_desc, sizeof(a.wind));
    memcpy(a.sim, sim_desc, sizeof(a.sim));
    a.drop = w->ellipsoid;
    memcpy(a.drop_desc, w->ellipsoid_desc, sizeof(a.drop_desc));
    a.dff = w->dff[les_id];
    memcpy(a.dff_desc, w->dff_desc, sizeof(a.dff_desc));
    a.rain_origin = pop->origins[0];
    a.rain_count = pop->counts[0];
    /* kernel selection of rs.c:5339-5349 */
    if (concept & rsc::kConceptDragged) {
        a.rain_mode = 1;
    } else if (concept & rsc::kConceptFixedPos) {
        a.rain_mode = 2;
    } else {
        a.rain_mode = 0;
    }
    if (a.rain_count && a.rain_mode != 2 && w->ellipsoid == nullptr) {
        return fail(RSC_ERR_STATE, "ellipsoid RCS table not set");
    }
    a.rain_blocks = (unsigned)((a.rain_count + rsc::kAdvanceThreads - 1) / rsc::kAdvanceThreads);
    unsigned long long deb = 0;
    s = fill_debris(w, pop, a, &deb);
    if (s) return s;
    if ((concept & rsc::kConceptDFF) && deb && a.dff == nullptr) return fail(RSC_ERR_STATE, "debris flux field not set");
    *blocks_out = a.rain_blocks + (unsigned)((deb + rsc::kAdvanceThreads - 1) / rsc::kAdvanceThreads);
    return RSC_OK;
}

int rsc_advance_time(rsc_worker *w, const rsc_population *pop, int les_id, const float sim_desc[16]) {
    int s = check_alloc(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    AdvanceArgs a;
    unsigned blocks = 0;
    s = fill_advance_args(w, pop, les_id, sim_desc, a, &blocks);
    if (s) return s;
    if (blocks == 0) return RSC_OK;
    if (w->fuse && w->precision != RSC_PULSE_F64) {
        /* run with the next pulse, or alone by the next call that needs it,
         * in place on the worker's stream */
        s = les_slot_wait(w, les_id, w->stream);
        if (s) return s;
        s = settle_sig_aux(w, w->stream);   /* the recorded advance runs in place */
        if (s) return s;
        w->pend = true;
        w->pend_a = a;
        w->pend_blocks = blocks;
        w->pend_pop = *pop;
        memcpy(w->pend_sim, sim_desc, sizeof(w->pend_sim));
        w->sig_aux_stale = true;
        return RSC_OK;
    }
    /* on the advance stream, beside the pulse of this step: read the current
     * pos / rcs pair, write the other one once the last pulse that read it
     * and the state or table changes queued since are done */
    a.pos = w->pos_next;
    a.rcs = w->rcs_next;
    w->adv_seq++;   /* a later join waits for what follows */
    if (w->read_next_pending) {
        RSC_CUDA(cudaStreamWaitEvent(w->adv, w->ev_read_next, 0));
        w->read_next_pending = false;
    }
    if (w->main_pending) {
        RSC_CUDA(cudaStreamWaitEvent(w->adv, w->ev_main, 0));
        w->main_pending = false;
    }
    s = les_slot_wait(w, les_id, w->adv);
    if (s) return s;
    if (w->sig_aux_stale && w->sa_pos == w->pos_next) {
        /* a second advance since the pulse overwrites the pair it read */
        s = settle_sig_aux(w, w->adv);
        if (s) return s;
    }
    s = copy_unadvanced(w, pop, w->adv);
    if (s) return s;
    int n = 0;
    RSC_CUDA(launch_advance(w, a, blocks, &n, w->adv));
    w->launches += n;
    std::swap(w->pos, w->pos_next);
    std::swap(w->rcs, w->rcs_next);
    std::swap(w->ev_read, w->ev_read_next);
    std::swap(w->read_pending, w->read_next_pending);
    w->sig_aux_stale = true;
    w->since_sort++;
    return maybe_sort(w, pop, sim_desc, w->stream);
}

int rsc_update_debris_rcs(rsc_worker *w, const rsc_population *pop, const float sim_desc[16]) {
    int s = check_alloc(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    if (pop == nullptr || sim_desc == nullptr) return fail(RSC_ERR_ARG, "population / sim_desc is NULL");
    AdvanceArgs a;
    memset(&a, 0, sizeof(a));
    a.pos_in = a.pos = w->pos;
    a.ori = w->ori;
    a.rcs_in = a.rcs = w->rcs;
    memcpy(a.sim, sim_desc, sizeof(a.sim));
    unsigned long long deb = 0;
    s = fill_debris(w, pop, a, &deb);
    if (s) return s;
    if (deb == 0) return RSC_OK;
    unsigned blocks = (unsigned)((deb + rsc::kAdvanceThreads - 1) / rsc::kAdvanceThreads);
    rsc::k_db_rcs<<<blocks, rsc::kAdvanceThreads, 0, w->stream>>>(a);
    RSC_CUDA(cudaGetLastError());
    w->launches++;
    return release_main(w);
}

int rsc_make_pulse(rsc_worker *w, const float sim_desc[16]) {
    int s = check_alloc(w);
    if (s) return s;
    if (sim_desc == nullptr) return fail(RSC_ERR_ARG, "sim_desc is NULL");
    if (w->range_weight == nullptr || w->angular_weight == nullptr) {
        return fail(RSC_ERR_STATE, "range / angular weight tables not set");
    }
    const int mode = w->precision;
    PulseArgs P;
    fill_pulse_args(w, P, sim_desc);
    if (mode == RSC_PULSE_COMPENSATED) {
        P.rk = w->rk_hi;
        /* the error-free warp sums need the grouped path, whatever the order */
        P.coherent_span = (int)w->G + 1;
        P.mom_n = w->moments ? moment_span(P) : 0;
        P.runs = w->runs;
    }
    const bool mat = (mode == RSC_PULSE_PLAIN) && (w->materialize || sim_desc[15] != 0.0f);
    P.materialize = mat ? 1 : 0;
    int grid = 0, threads = 0;
    size_t smem = 0;
    s = pulse_geometry(w, mode, pulse_path(P, mode), &grid, &threads, &smem);
    if (s) return s;
    s = pulse_d2h_wait(w);
    if (s) return s;
    if (w->pend && mode != RSC_PULSE_F64) {
        /* the recorded advance and this pulse in one pass over the state */
        int sgrid = 0;
        size_t ssmem = 0;
        s = step_shape(mode, w, &sgrid, &ssmem);
        if (s) return s;
        P.mom_n = 0;   /* the fused kernel sums per gate */
        if (mode == RSC_PULSE_PLAIN) {
            rsc::k_step<0><<<sgrid, rsc::kAdvanceThreads, ssmem, w->stream>>>(w->pend_a, P, w->pend_blocks);
        } else {
            rsc::k_step<1><<<sgrid, rsc::kAdvanceThreads, ssmem, w->stream>>>(w->pend_a, P, w->pend_blocks);
        }
        RSC_CUDA(cudaGetLastError());
        w->pend = false;
        w->launches++;
        s = mark_read(w);
        if (s == RSC_OK) s = release_main(w);   /* the state changed in place */
        if (s) return s;
        memcpy(w->last_sim, sim_desc, sizeof(w->last_sim));
        w->have_pulse_desc = true;
        w->sig_aux_stale = !mat;
        w->sa_pos = w->pos;
        w->sa_rcs = w->rcs;
        w->since_sort++;
        return maybe_sort(w, &w->pend_pop, w->pend_sim, w->stream);
    }
    s = flush_pending(w);
    if (s) return s;
    launch_pulse(mode, P, grid, threads, smem, w->stream);
    RSC_CUDA(cudaGetLastError());
    w->launches++;
    s = mark_read(w);
    if (s) return s;
    memcpy(w->last_sim, sim_desc, sizeof(w->last_sim));
    w->have_pulse_desc = true;
    w->sig_aux_stale = !mat;
    w->sa_pos = P.pos;
    w->sa_rcs = P.rcs;
    return RSC_OK;
}

int rsc_download_pulse(rsc_worker *w, float *pulse4, float gain) {
    int s = check_alloc(w);
    if (s) return s;
    if (pulse4 == nullptr) return fail(RSC_ERR_ARG, "pulse4 is NULL");
    RSC_CUDA(cudaMemcpyAsync(pulse4, w->pulse, w->G * sizeof(float4), cudaMemcpyDeviceToHost, w->stream));
    RSC_CUDA(cudaStreamSynchronize(w->stream));
    for (uint32_t k = 0; k < 4 * w->G; k++) pulse4[k] = pulse4[k] * gain;
    return RSC_OK;
}

int rsc_download_pulse_async(rsc_worker *w, float *pulse4) {
    int s = check_alloc(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    if (pulse4 == nullptr) return fail(RSC_ERR_ARG, "pulse4 is NULL");
    if (w->d2h == nullptr) {
        RSC_CUDA(cudaStreamCreateWithFlags(&w->d2h, cudaStreamNonBlocking));
        RSC_CUDA(cudaEventCreateWithFlags(&w->pulse_ev, cudaEventDisableTiming));
        RSC_CUDA(cudaEventCreateWithFlags(&w->d2h_done, cudaEventDisableTiming));
    }
    RSC_CUDA(cudaEventRecord(w->pulse_ev, w->stream));
    RSC_CUDA(cudaStreamWaitEvent(w->d2h, w->pulse_ev, 0));
    RSC_CUDA(cudaMemcpyAsync(pulse4, w->pulse, w->G * sizeof(float4), cudaMemcpyDeviceToHost, w->d2h));
    RSC_CUDA(cudaEventRecord(w->d2h_done, w->d2h));
    w->d2h_pending = true;
    return RSC_OK;
}


int rsc_synchronize(rsc_worker *w) {
    int s = check_worker(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    RSC_CUDA(cudaStreamSynchronize(w->stream));
    if (w->d2h) RSC_CUDA(cudaStreamSynchronize(w->d2h));
    w->d2h_pending = false;
    return RSC_OK;
}

int rsc_set_pulse_precision(rsc_worker *w, int mode) {
    int s = check_worker(w);
    if (s) return s;
    if (mode != RSC_PULSE_PLAIN && mode != RSC_PULSE_COMPENSATED && mode != RSC_PULSE_F64) {
        return fail(RSC_ERR_ARG, "precision mode %d", mode);
    }
    w->precision = mode;
    return RSC_OK;
}

int rsc_set_materialize_sig_aux(rsc_worker *w, int enable) {
    int s = check_worker(w);
    if (s) return s;
    w->materialize = enable ? 1 : 0;
    return RSC_OK;
}

int rsc_set_pulse_moments(rsc_worker *w, int enable) {
    int s = check_worker(w);
    if (s) return s;
    w->moments = enable ? 1 : 0;
    return RSC_OK;
}

int rsc_launch_count(rsc_worker *w, uint64_t *count) {
    if (w == nullptr || count == nullptr) return fail(RSC_ERR_ARG, "NULL argument");
    *count = w->launches;
    return RSC_OK;
}

int rsc_get_stream(rsc_worker *w, void **stream) {
    if (w == nullptr || stream == nullptr) return fail(RSC_ERR_ARG, "NULL argument");
    *stream = (void *)w->stream;
    return RSC_OK;
}

int rsc_get_advance_stream(rsc_worker *w, void **stream) {
    if (w == nullptr || stream == nullptr) return fail(RSC_ERR_ARG, "NULL argument");
    *stream = (void *)w->adv;
    return RSC_OK;
}

}  // extern "C"

/* ---- launch-shape autotuning and the batching form ------------------------- */

namespace {

struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    cudaError_t init() {
        cudaError_t e = cudaEventCreate(&a);
        if (e == cudaSuccess) e = cudaEventCreate(&b);
        return e;
    }
    ~EventPair() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

/* candidate shapes: warps per block x resident blocks per SM */
const int kTuneWarps[] = {16, 8, 4};
const int kTuneReps = 3;

}  // namespace

struct rsc_batch {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_join = nullptr, ev_h2d = nullptr, ev_done = nullptr;
    /* the debris kernel beside the background kernel (high priority) */
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, side_ev = nullptr;
    /* the advance stream (the pulse of a step runs on `stream` beside it):
     * ev_bp / ev_ba after the pulse / advance of the last two steps */
    cudaStream_t adv = nullptr;
    cudaEvent_t ev_bp[2] = {nullptr, nullptr}, ev_ba[2] = {nullptr, nullptr}, ev_afork = nullptr;
    std::vector<rsc_worker *> w;
    std::vector<rsc_population> pops;
    bool have_pops = false;
    int mode = RSC_PULSE_PLAIN;
    uint32_t Gmax = 0;
    int tune_warps = 0, tune_per_sm = 0;
    /* background advance shape: threads per block and the shared-memory
     * bytes each block asks for, which limits the resident blocks per SM
     * (0: as many as fit) */
    int adv_threads = rsc::kAdvanceThreads, adv_per_sm = 0;
    size_t adv_smem = 0;
    bool tri = false;   /* the pulse kernel with the triangle range weight compiled in */
    /* per-instance launch descriptors and block prefixes */
    std::vector<rsc::BatchAdvance> h_adv;
    std::vector<PulseArgs> h_pulse;
    std::vector<unsigned> h_rain_prefix, h_deb_prefix, h_pulse_prefix;
    std::vector<uint32_t> concept;
    rsc::BatchAdvance *d_adv = nullptr;
    PulseArgs *d_pulse = nullptr;
    unsigned *d_rain_prefix = nullptr, *d_deb_prefix = nullptr, *d_pulse_prefix = nullptr;
    unsigned rain_blocks = 0, deb_blocks = 0, pulse_blocks = 0;
    int pulse_threads = 0, pulse_per_sm = 0;
    size_t pulse_smem = 0;
    /* per-step descriptors (pinned on the host) and the pulses of a run */
    int cap_steps = 0;
    rsc::BatchStep *h_steps = nullptr;
    rsc::BatchStep *d_steps = nullptr;
    float4 *d_out = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    uint64_t launches = 0;
    /* LES refills on a copy stream: per instance and slot, the event of the
     * last run that read the slot, the event of the refill's completion and
     * whether a run still has to wait for it */
    cudaStream_t copy_stream = nullptr;
    float4 *les_stage = nullptr;   /* uvwt of rsc_batch_set_les_async before its pair layout */
    size_t les_stage_n = 0;
    std::vector<cudaEvent_t> slot_used, slot_ready;
    std::vector<char> slot_pending;
    /* the persistent form (rsc_batch_set_persistent): per-block segments,
     * per-instance block counts, per-step accumulators and tickets */
    bool persist = false;
    unsigned persist_blocks = 0;
    size_t persist_smem = 0;
    rsc::PersistSeg *d_pseg = nullptr;
    unsigned *d_pseg_off = nullptr, *d_pnblk = nullptr;
    size_t pseg_cap = 0;
    double *d_pacc = nullptr;
    unsigned *d_ptick = nullptr;
    size_t pacc_cap = 0;   /* step x instance slots */
};

namespace {

int check_batch(rsc_batch *b) {
    if (b == nullptr) return fail(RSC_ERR_ARG, "batch is NULL");
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return cuda_fail(RSC_ERR_CUDA, "cudaSetDevice(%d): %s", b->device, cudaGetErrorString(e));
    return RSC_OK;
}

void batch_drop_graph(rsc_batch *b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->graph_steps = 0;
}

/* Room for `steps` steps of per-step descriptors and pulses. */
int batch_reserve(rsc_batch *b, int steps) {
    if (steps <= b->cap_steps) return RSC_OK;
    RSC_CUDA(cudaStreamSynchronize(b->stream));
    batch_drop_graph(b);
    if (b->h_steps) cudaFreeHost(b->h_steps);
    free_ptr(b->d_steps);
    free_ptr(b->d_out);
    b->h_steps = nullptr;
    b->d_steps = nullptr;
    b->d_out = nullptr;
    b->cap_steps = 0;
    const size_t n = b->w.size();
    const size_t rows = (size_t)steps * n;
    cudaError_t e = cudaMallocHost((void **)&b->h_steps, rows * sizeof(rsc::BatchStep));
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_steps, rows * sizeof(rsc::BatchStep));
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_out, rows * b->Gmax * sizeof(float4));
    if (e != cudaSuccess) return cuda_fail(RSC_ERR_NOMEM, "batch buffers for %d steps: %s", steps, cudaGetErrorString(e));
    memset(b->h_steps, 0, rows * sizeof(rsc::BatchStep));
    RSC_CUDA(cudaMemsetAsync(b->d_out, 0, rows * b->Gmax * sizeof(float4), b->stream));
    b->cap_steps = steps;
    return RSC_OK;
}

/* Build every instance's descriptors for the beam / concept of `row` (one
 * BatchStep per instance) and the block prefixes; upload them.  A change of
 * grid or block shape retires the captured graph. */
int batch_prepare(rsc_batch *b, const rsc::BatchStep *row) {
    if (!b->have_pops) return fail(RSC_ERR_STATE, "rsc_batch_set_populations has not been called");
    const size_t n = b->w.size();
    int per_sm = 1, threads = 0;
    size_t smem = 0;
    int s = pulse_shape(b->mode, true, b->Gmax, b->tune_warps, b->tune_per_sm, &per_sm, &threads, &smem);
    if (s) return s;
    const double total = (double)b->num_sms * per_sm;
    double sum_n = 0.0;
    for (rsc_worker *x : b->w) sum_n += (double)x->num_scats;
    b->h_adv.assign(n, rsc::BatchAdvance());
    b->h_pulse.assign(n, PulseArgs());
    b->h_rain_prefix.assign(n + 1, 0u);
    b->h_deb_prefix.assign(n + 1, 0u);
    b->h_pulse_prefix.assign(n + 1, 0u);
    bool tri = true;   /* every instance's range table is the triangle */
    b->concept.assign(n, 0u);
    unsigned acc_r = 0, acc_d = 0, acc_p = 0;
    for (size_t i = 0; i < n; i++) {
        rsc_worker *x = b->w[i];
        if (x->pos == nullptr) return fail(RSC_ERR_STATE, "instance %zu is not allocated", i);
        if (x->G > b->Gmax) return fail(RSC_ERR_STATE, "instance %zu has more gates than when the batch was created", i);
        if (x->range_weight == nullptr || x->angular_weight == nullptr) {
            return fail(RSC_ERR_STATE, "instance %zu: range / angular weight tables not set", i);
        }
        rsc::BatchAdvance &A = b->h_adv[i];
        unsigned blocks = 0;
        s = fill_advance_args(x, &b->pops[i], row[i].les_id, row[i].sim, A.a, &blocks);
        if (s) {
            char why[sizeof(g_err)];
            snprintf(why, sizeof(why), "%s", g_err);
            return fail(s, "instance %zu: %s", i, why);
        }
        for (int slot = 0; slot < 2; slot++) {
            A.uvwt[slot] = make_pair_image(x->les_uvwt[slot], x->les_nx, x->les_ny, x->les_nz);
            A.cpxx[slot] = make_image(x->les_cpxx[slot], x->les_nx, x->les_ny, x->les_nz);
            A.dff[slot] = x->dff[slot];
        }
        b->h_rain_prefix[i] = acc_r;
        acc_r += (unsigned)((A.a.rain_count + (unsigned long long)b->adv_threads - 1) / (unsigned long long)b->adv_threads);
        b->h_deb_prefix[i] = acc_d;
        acc_d += blocks - A.a.rain_blocks;
        PulseArgs &P = b->h_pulse[i];
        fill_pulse_args(x, P, row[i].sim);
        if (b->mode == RSC_PULSE_COMPENSATED) {
            P.rk = x->rk_hi;
            P.coherent_span = (int)x->G + 1;
            P.mom_n = x->moments ? moment_span(P) : 0;
            P.runs = x->runs;
        }
        P.materialize = 0;
        tri = tri && P.rw_tri;
        /* pulse blocks in proportion to the scatterers, at least one, and no
         * block without a scatterer to start on */
        double share = sum_n > 0.0 ? total * (double)x->num_scats / sum_n : 1.0;
        unsigned bi = (unsigned)llround(share);
        unsigned cap = (unsigned)((x->num_scats + (size_t)threads - 1) / (size_t)threads);
        if (bi > cap) bi = cap;
        if (bi < 1) bi = 1;
        b->h_pulse_prefix[i] = acc_p;
        acc_p += bi;
        b->concept[i] = rsm_f2u(row[i].sim[5]);
    }
    b->h_rain_prefix[n] = acc_r;
    b->h_deb_prefix[n] = acc_d;
    b->h_pulse_prefix[n] = acc_p;
    if (acc_r != b->rain_blocks || acc_d != b->deb_blocks || acc_p != b->pulse_blocks || threads != b->pulse_threads ||
        smem != b->pulse_smem || tri != b->tri) {
        batch_drop_graph(b);
    }
    b->tri = tri;
    b->rain_blocks = acc_r;
    b->deb_blocks = acc_d;
    b->pulse_blocks = acc_p;
    b->pulse_threads = threads;
    b->pulse_smem = smem;
    b->pulse_per_sm = per_sm;
    /* pageable sources: each copy has taken its bytes when the call returns */
    RSC_CUDA(cudaMemcpyAsync(b->d_adv, b->h_adv.data(), n * sizeof(rsc::BatchAdvance), cudaMemcpyHostToDevice, b->stream));
    RSC_CUDA(cudaMemcpyAsync(b->d_pulse, b->h_pulse.data(), n * sizeof(PulseArgs), cudaMemcpyHostToDevice, b->stream));
    RSC_CUDA(cudaMemcpyAsync(b->d_rain_prefix, b->h_rain_prefix.data(), (n + 1) * sizeof(unsigned),
                             cudaMemcpyHostToDevice, b->stream));
    RSC_CUDA(cudaMemcpyAsync(b->d_deb_prefix, b->h_deb_prefix.data(), (n + 1) * sizeof(unsigned),
                             cudaMemcpyHostToDevice, b->stream));
    RSC_CUDA(cudaMemcpyAsync(b->d_pulse_prefix, b->h_pulse_prefix.data(), (n + 1) * sizeof(unsigned),
                             cudaMemcpyHostToDevice, b->stream));
    return RSC_OK;
}

cudaError_t batch_launch_pulse(rsc_batch *b, int k) {
    const int n = (int)b->w.size();
    const rsc::BatchStep *st = b->d_steps + (size_t)k * n;
    float4 *out = b->d_out + (size_t)k * n * b->Gmax;
    const unsigned g = b->pulse_blocks, t = (unsigned)b->pulse_threads;
    const size_t sm = b->pulse_smem;
    if (b->mode == RSC_PULSE_PLAIN && b->tri) {
        rsc::k_pulse_batch<0, 1><<<g, t, sm, b->stream>>>(b->d_pulse, st, b->d_pulse_prefix, n, out, b->Gmax);
    } else if (b->mode == RSC_PULSE_PLAIN) {
        rsc::k_pulse_batch<0><<<g, t, sm, b->stream>>>(b->d_pulse, st, b->d_pulse_prefix, n, out, b->Gmax);
    } else if (b->mode == RSC_PULSE_COMPENSATED && b->tri) {
        rsc::k_pulse_batch<1, 1><<<g, t, sm, b->stream>>>(b->d_pulse, st, b->d_pulse_prefix, n, out, b->Gmax);
    } else if (b->mode == RSC_PULSE_COMPENSATED) {
        rsc::k_pulse_batch<1><<<g, t, sm, b->stream>>>(b->d_pulse, st, b->d_pulse_prefix, n, out, b->Gmax);
    } else {
        rsc::k_pulse_batch<2><<<g, t, sm, b->stream>>>(b->d_pulse, st, b->d_pulse_prefix, n, out, b->Gmax);
    }
    return cudaGetLastError();
}

/* Steps 0..K-1: the pulse of every instance on the batch's stream and the
 * advance of every instance beside it on the advance stream (background
 * kernel, debris kernel on the side stream).  The pulse of step k waits for
 * the advance of step k - 1 (which wrote what it reads); the advance of step
 * k for the pulse of step k - 1 (which read the pair it overwrites).  The
 * advance stream starts after the work queued on the batch's stream and the
 * batch's stream ends after it. */
/* The background advance of one step of every instance at the batch's
 * advance shape. */
cudaError_t batch_launch_rain(rsc_batch *b, const rsc::BatchAdvance *adv, const rsc::BatchStep *st) {
    const int n = (int)b->w.size();
    const unsigned g = b->rain_blocks;
    const size_t sm = b->adv_smem;
    if (b->adv_threads == 64) {
        rsc::k_advance_batch_rain<64><<<g, 64, sm, b->adv>>>(adv, st, b->d_rain_prefix, n);
    } else if (b->adv_threads == 256) {
        rsc::k_advance_batch_rain<256><<<g, 256, sm, b->adv>>>(adv, st, b->d_rain_prefix, n);
    } else {
        rsc::k_advance_batch_rain<128><<<g, 128, sm, b->adv>>>(adv, st, b->d_rain_prefix, n);
    }
    return cudaGetLastError();
}

/* Dynamic shared memory that leaves at most per_sm blocks of the batched
 * background advance resident on an SM (0: no limit). */
int batch_advance_smem(rsc_batch *b, int threads, int per_sm, size_t *smem) {
    *smem = 0;
    if (per_sm <= 0) return RSC_OK;
    int dev = 0, sm_bytes = 0, optin = 0;
    RSC_CUDA(cudaGetDevice(&dev));
    RSC_CUDA(cudaDeviceGetAttribute(&sm_bytes, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    RSC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    size_t want = (size_t)sm_bytes / (size_t)per_sm + 1;
    want = (want + 127) & ~(size_t)127;
    if (want > (size_t)optin - 1024) want = (size_t)optin - 1024;
    void *k = threads == 64 ? reinterpret_cast<void *>(rsc::k_advance_batch_rain<64>)
                            : (threads == 256 ? reinterpret_cast<void *>(rsc::k_advance_batch_rain<256>)
                                              : reinterpret_cast<void *>(rsc::k_advance_batch_rain<128>));
    RSC_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want));
    *smem = want;
    (void)b;
    return RSC_OK;
}

cudaError_t batch_enqueue(rsc_batch *b, int steps) {
    const int n = (int)b->w.size();
    const bool advance = b->rain_blocks || b->deb_blocks;
    cudaError_t e = cudaSuccess;
    if (advance) {
        e = cudaEventRecord(b->ev_afork, b->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->adv, b->ev_afork, 0);
        if (e != cudaSuccess) return e;
    }
    for (int k = 0; k < steps; k++) {
        if (advance && k > 0) {
            e = cudaStreamWaitEvent(b->stream, b->ev_ba[(k - 1) & 1], 0);
            if (e != cudaSuccess) return e;
        }
        e = batch_launch_pulse(b, k);
        if (e == cudaSuccess && advance) e = cudaEventRecord(b->ev_bp[k & 1], b->stream);
        if (e != cudaSuccess) return e;
        if (!advance) continue;
        const rsc::BatchStep *st = b->d_steps + (size_t)k * n;
        if (k > 0) {
            e = cudaStreamWaitEvent(b->adv, b->ev_bp[(k - 1) & 1], 0);
            if (e != cudaSuccess) return e;
        }
        if (b->deb_blocks) {
            e = cudaEventRecord(b->fork_ev, b->adv);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(b->side, b->fork_ev, 0);
            if (e != cudaSuccess) return e;
            rsc::k_advance_batch_debris<<<b->deb_blocks, rsc::kAdvanceThreads, 0, b->side>>>(b->d_adv, st,
                                                                                            b->d_deb_prefix, n);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaEventRecord(b->side_ev, b->side);
            if (e != cudaSuccess) return e;
        }
        if (b->rain_blocks) {
            e = batch_launch_rain(b, b->d_adv, st);
            if (e != cudaSuccess) return e;
        }
        if (b->deb_blocks) {
            e = cudaStreamWaitEvent(b->adv, b->side_ev, 0);
            if (e != cudaSuccess) return e;
        }
        e = cudaEventRecord(b->ev_ba[k & 1], b->adv);
        if (e != cudaSuccess) return e;
    }
    if (advance) e = cudaStreamWaitEvent(b->stream, b->ev_ba[(steps - 1) & 1], 0);
    return e;
}

int batch_capture(rsc_batch *b, int steps) {
    batch_drop_graph(b);
    RSC_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = batch_enqueue(b, steps);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->graph = nullptr;
        return cuda_fail(RSC_ERR_CUDA, "graph capture of %d steps: %s", steps, cudaGetErrorString(e));
    }
    b->graph_steps = steps;
    return RSC_OK;
}

/* The pos / rcs pairs of every step: step k of a run reads the instance's
 * current pair when k is even, its other pair when k is odd, and the advance
 * writes the other one. */
void batch_fill_pairs(rsc_batch *b, int steps) {
    const size_t n = b->w.size();
    for (int k = 0; k < steps; k++) {
        for (size_t i = 0; i < n; i++) {
            rsc_worker *x = b->w[i];
            rsc::BatchStep &S = b->h_steps[(size_t)k * n + i];
            const bool odd = (k & 1) != 0;
            S.pos_r = odd ? x->pos_next : x->pos;
            S.rcs_r = odd ? x->rcs_next : x->rcs;
            S.pos_w = odd ? x->pos : x->pos_next;
            S.rcs_w = odd ? x->rcs : x->rcs_next;
        }
    }
}

/* After a run of `steps` steps: an odd count leaves each instance's state in
 * its other pair. */
void batch_swap_pairs(rsc_batch *b, int steps) {
    if ((steps & 1) == 0 || (b->rain_blocks == 0 && b->deb_blocks == 0)) return;
    for (rsc_worker *x : b->w) {
        std::swap(x->pos, x->pos_next);
        std::swap(x->rcs, x->rcs_next);
        std::swap(x->ev_read, x->ev_read_next);
        std::swap(x->read_pending, x->read_next_pending);
    }
}

/* Copy steps' descriptors into the pinned table, checking them. */
int batch_fill_steps(rsc_batch *b, int steps, const float *sim_descs, const int *les_ids) {
    const size_t n = b->w.size();
    RSC_CUDA(cudaEventSynchronize(b->ev_h2d));   /* the last run's copy of the table has been taken */
    for (int k = 0; k < steps; k++) {
        for (size_t i = 0; i < n; i++) {
            const size_t r = (size_t)k * n + i;
            const int les = les_ids ? les_ids[r] : 0;
            rsc_worker *x = b->w[i];
            if (les < 0 || les > 1 || x->les_uvwt[les] == nullptr) {
                return fail(RSC_ERR_STATE, "step %d instance %zu: LES slot %d not set", k, i, les);
            }
            const float *sim = sim_descs + r * 16;
            if (k > 0 && rsm_f2u(sim[5]) != rsm_f2u(sim_descs[i * 16 + 5])) {
                return fail(RSC_ERR_ARG, "step %d instance %zu: the concept changes within a run", k, i);
            }
            const rsc_population &p = b->pops[i];
            bool deb = false;
            for (int t = 1; t < RSC_MAX_TYPES; t++) deb = deb || p.counts[t] != 0;
            if ((rsm_f2u(sim[5]) & rsc::kConceptDFF) && deb && x->dff[les] == nullptr) {
                return fail(RSC_ERR_STATE, "step %d instance %zu: debris flux field of slot %d not set", k, i, les);
            }
            rsc::BatchStep &S = b->h_steps[r];
            memcpy(S.sim, sim, sizeof(S.sim));
            S.les_id = les;
        }
    }
    return RSC_OK;
}

/* Order the batch stream after every worker's queued work. */
int batch_join_workers(rsc_batch *b) {
    for (rsc_worker *x : b->w) {
        int s = flush_pending(x);
        if (s) return s;
        RSC_CUDA(cudaEventRecord(b->ev_join, x->stream));
        RSC_CUDA(cudaStreamWaitEvent(b->stream, b->ev_join, 0));
    }
    return RSC_OK;
}

}  // namespace

extern "C" {

int rsc_set_pulse_shape(rsc_worker *w, int warps, int blocks_per_sm) {
    int s = check_worker(w);
    if (s) return s;
    if (warps < 0 || warps > 16 || blocks_per_sm < 0 || blocks_per_sm > 4) {
        return fail(RSC_ERR_ARG, "pulse shape %d warps x %d blocks per SM", warps, blocks_per_sm);
    }
    w->tune_warps = warps;
    w->tune_per_sm = blocks_per_sm;
    return RSC_OK;
}

int rsc_set_advance_shape(rsc_worker *w, int scatterers_per_thread) {
    int s = check_worker(w);
    if (s) return s;
    if (scatterers_per_thread != 1 && scatterers_per_thread != 2) {
        return fail(RSC_ERR_ARG, "advance shape: %d scatterers per thread", scatterers_per_thread);
    }
    w->adv_per_thread = scatterers_per_thread;
    return RSC_OK;
}

int rsc_autotune(rsc_worker *w, const float sim_desc[16], int *warps_out, int *blocks_per_sm_out) {
    int s = check_alloc(w);
    if (s) return s;
    s = flush_pending(w);
    if (s) return s;
    if (sim_desc == nullptr) return fail(RSC_ERR_ARG, "sim_desc is NULL");
    if (w->range_weight == nullptr || w->angular_weight == nullptr) {
        return fail(RSC_ERR_STATE, "range / angular weight tables not set");
    }
    const int mode = w->precision;
    PulseArgs P;
    fill_pulse_args(w, P, sim_desc);
    if (mode == RSC_PULSE_COMPENSATED) {
        P.rk = w->rk_hi;
        P.coherent_span = (int)w->G + 1;
        P.mom_n = w->moments ? moment_span(P) : 0;
        P.runs = w->runs;
    }
    P.materialize = 0;
    s = pulse_d2h_wait(w);
    if (s) return s;
    EventPair ev;
    RSC_CUDA(ev.init());
    float best = INFINITY;
    int best_w = 0, best_p = 0;
    for (int warps : kTuneWarps) {
        for (int per_sm = 1; per_sm <= 4; per_sm++) {
            int got = 0, threads = 0;
            size_t smem = 0;
            s = pulse_shape(mode, false, w->G, warps, per_sm, &got, &threads, &smem, pulse_path(P, mode));
            if (s) return s;
            if (threads != warps * 32 || got != per_sm) continue;   /* shape not reachable */
            const int grid = w->num_sms * per_sm;
            launch_pulse(mode, P, grid, threads, smem, w->stream);
            RSC_CUDA(cudaEventRecord(ev.a, w->stream));
            for (int r = 0; r < kTuneReps; r++) launch_pulse(mode, P, grid, threads, smem, w->stream);
            RSC_CUDA(cudaEventRecord(ev.b, w->stream));
            RSC_CUDA(cudaGetLastError());
            RSC_CUDA(cudaEventSynchronize(ev.b));
            float ms = 0.0f;
            RSC_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
            w->launches += 1 + kTuneReps;
            if (ms < best) {
                best = ms;
                best_w = warps;
                best_p = per_sm;
            }
        }
    }
    s = mark_read(w);
    if (s) return s;
    w->tune_warps = best_w;
    w->tune_per_sm = best_p;
    memcpy(w->last_sim, sim_desc, sizeof(w->last_sim));
    w->have_pulse_desc = true;
    w->sig_aux_stale = true;
    if (warps_out) *warps_out = best_w;
    if (blocks_per_sm_out) *blocks_per_sm_out = best_p;
    return RSC_OK;
}

int rsc_batch_create(rsc_worker *const *workers, int count, rsc_batch **out) {
    if (out == nullptr || workers == nullptr) return fail(RSC_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (count < 1) return fail(RSC_ERR_ARG, "batch of %d instances", count);
    for (int i = 0; i < count; i++) {
        if (workers[i] == nullptr) return fail(RSC_ERR_ARG, "instance %d is NULL", i);
        if (workers[i]->pos == nullptr) return fail(RSC_ERR_STATE, "instance %d is not allocated", i);
        if (workers[i]->device != workers[0]->device) return fail(RSC_ERR_ARG, "instances on different devices");
        for (int j = 0; j < i; j++) {
            if (workers[j] == workers[i]) return fail(RSC_ERR_ARG, "instance %d repeats instance %d", i, j);
        }
    }
    rsc_batch *b = new rsc_batch();
    b->device = workers[0]->device;
    b->num_sms = workers[0]->num_sms;
    b->w.assign(workers, workers + count);
    b->pops.assign(count, rsc_population());
    for (rsc_worker *x : b->w) b->Gmax = x->G > b->Gmax ? x->G : b->Gmax;
    cudaError_t e = cudaSetDevice(b->device);
    /* priorities as a worker's: pulses ahead of the background advance,
     * debris ahead of both */
    int prio_least = 0, prio_greatest = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    const int prio_main = prio_greatest < prio_least ? prio_greatest + 1 : prio_greatest;
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&b->stream, cudaStreamNonBlocking, prio_main);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_h2d, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&b->side, cudaStreamNonBlocking, prio_greatest);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->side_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->adv, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; k++) {
        e = cudaEventCreateWithFlags(&b->ev_bp[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_ba[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_afork, cudaEventDisableTiming);
    b->slot_used.assign(2 * count, nullptr);
    b->slot_ready.assign(2 * count, nullptr);
    b->slot_pending.assign(2 * count, 0);
    for (int q = 0; q < 2 * count && e == cudaSuccess; q++) {
        e = cudaEventCreateWithFlags(&b->slot_used[q], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->slot_ready[q], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_adv, count * sizeof(rsc::BatchAdvance));
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_pulse, count * sizeof(PulseArgs));
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_rain_prefix, (count + 1) * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_deb_prefix, (count + 1) * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_pulse_prefix, (count + 1) * sizeof(unsigned));
    if (e != cudaSuccess) {
        rsc_batch_free(b);
        return cuda_fail(RSC_ERR_CUDA, "batch creation: %s", cudaGetErrorString(e));
    }
    *out = b;
    return RSC_OK;
}

int rsc_batch_free(rsc_batch *b) {
    if (b == nullptr) return RSC_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    batch_drop_graph(b);
    if (b->h_steps) cudaFreeHost(b->h_steps);
    free_ptr(b->d_steps);
    free_ptr(b->d_out);
    free_ptr(b->d_adv);
    free_ptr(b->d_pulse);
    free_ptr(b->d_rain_prefix);
    free_ptr(b->d_deb_prefix);
    free_ptr(b->d_pulse_prefix);
    free_ptr(b->d_pseg);
    free_ptr(b->d_pseg_off);
    free_ptr(b->d_pnblk);
    free_ptr(b->d_pacc);
    free_ptr(b->d_ptick);
    if (b->copy_stream) cudaStreamSynchronize(b->copy_stream);
    free_ptr(b->les_stage);
    for (cudaEvent_t ev : b->slot_used) {
        if (ev) cudaEventDestroy(ev);
    }
    for (cudaEvent_t ev : b->slot_ready) {
        if (ev) cudaEventDestroy(ev);
    }
    if (b->copy_stream) cudaStreamDestroy(b->copy_stream);
    if (b->side) {
        cudaStreamSynchronize(b->side);
        cudaStreamDestroy(b->side);
    }
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    if (b->side_ev) cudaEventDestroy(b->side_ev);
    if (b->adv) {
        cudaStreamSynchronize(b->adv);
        cudaStreamDestroy(b->adv);
    }
    for (int k = 0; k < 2; k++) {
        if (b->ev_bp[k]) cudaEventDestroy(b->ev_bp[k]);
        if (b->ev_ba[k]) cudaEventDestroy(b->ev_ba[k]);
    }
    if (b->ev_afork) cudaEventDestroy(b->ev_afork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    if (b->ev_h2d) cudaEventDestroy(b->ev_h2d);
    if (b->ev_done) cudaEventDestroy(b->ev_done);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return RSC_OK;
}

int rsc_batch_set_populations(rsc_batch *b, const rsc_population *pops) {
    int s = check_batch(b);
    if (s) return s;
    if (pops == nullptr) return fail(RSC_ERR_ARG, "pops is NULL");
    b->pops.assign(pops, pops + b->w.size());
    b->have_pops = true;
    return RSC_OK;
}

int rsc_batch_set_precision(rsc_batch *b, int mode) {
    int s = check_batch(b);
    if (s) return s;
    if (mode != RSC_PULSE_PLAIN && mode != RSC_PULSE_COMPENSATED && mode != RSC_PULSE_F64) {
        return fail(RSC_ERR_ARG, "precision mode %d", mode);
    }
    if (mode != b->mode) {
        RSC_CUDA(cudaStreamSynchronize(b->stream));
        batch_drop_graph(b);
    }
    b->mode = mode;
    return RSC_OK;
}

}  // extern "C"

namespace {

/* The batched background advance's shape, timed as one step beside the
 * batched pulse: threads per block 64 / 128 / 256, each with every block
 * that fits resident and with half of them (shared memory asked for per
 * block).  The advance writes the step's other pos / rcs pair, which the
 * next run overwrites, and the arrays it updates in place (vel, rnd) are
 * scratch copies here, so the state is not changed.  Without the memory for
 * the copies the shape stays as it was. */
int batch_tune_advance(rsc_batch *b) {
    const size_t n = b->w.size();
    if (b->rain_blocks == 0) return RSC_OK;
    std::vector<size_t> off(n);
    size_t total = 0;
    for (size_t i = 0; i < n; i++) {
        off[i] = total;
        total += b->w[i]->numel;
    }
    float4 *svel = nullptr;
    uint4 *srnd = nullptr;
    rsc::BatchAdvance *sadv = nullptr;
    cudaError_t e = cudaMalloc((void **)&svel, total * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc((void **)&srnd, total * sizeof(uint4));
    if (e == cudaSuccess) e = cudaMalloc((void **)&sadv, n * sizeof(rsc::BatchAdvance));
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        free_ptr(svel);
        free_ptr(srnd);
        return RSC_OK;
    }
    std::vector<rsc::BatchAdvance> adv(b->h_adv);
    int s = RSC_OK;
    for (size_t i = 0; i < n && s == RSC_OK; i++) {
        rsc_worker *x = b->w[i];
        adv[i].a.vel = svel + off[i];
        adv[i].a.rnd = srnd + off[i];
        if (cudaMemcpyAsync(svel + off[i], x->vel, x->numel * sizeof(float4), cudaMemcpyDeviceToDevice, b->stream) !=
                cudaSuccess ||
            cudaMemcpyAsync(srnd + off[i], x->rnd, x->numel * sizeof(uint4), cudaMemcpyDeviceToDevice, b->stream) !=
                cudaSuccess) {
            s = cuda_fail(RSC_ERR_CUDA, "advance tuning copies failed");
        }
    }
    if (s == RSC_OK && cudaMemcpyAsync(sadv, adv.data(), n * sizeof(rsc::BatchAdvance), cudaMemcpyHostToDevice,
                                       b->stream) != cudaSuccess) {
        s = cuda_fail(RSC_ERR_CUDA, "advance tuning arguments");
    }
    EventPair ev;
    if (s == RSC_OK && ev.init() != cudaSuccess) s = cuda_fail(RSC_ERR_CUDA, "advance tuning events");
    float best = INFINITY;
    int best_t = b->adv_threads, best_p = b->adv_per_sm;
    const int shapes[6][2] = {{128, 0}, {64, 0}, {256, 0}, {128, 8}, {64, 16}, {256, 4}};
    for (int c = 0; c < 6 && s == RSC_OK; c++) {
        b->adv_threads = shapes[c][0];
        b->adv_per_sm = shapes[c][1];
        s = batch_advance_smem(b, b->adv_threads, b->adv_per_sm, &b->adv_smem);
        if (s == RSC_OK) s = batch_prepare(b, b->h_steps);
        if (s) break;
        float ms = 0.0f;
        for (int r = 0; r <= kTuneReps && s == RSC_OK; r++) {
            cudaError_t q = cudaEventRecord(r == 1 ? ev.a : b->ev_afork, b->stream);
            if (r == 1 && q == cudaSuccess) q = cudaEventRecord(b->ev_afork, b->stream);
            if (q == cudaSuccess) q = cudaStreamWaitEvent(b->adv, b->ev_afork, 0);
            if (q == cudaSuccess) q = batch_launch_pulse(b, 0);
            if (q == cudaSuccess) q = batch_launch_rain(b, sadv, b->d_steps);
            if (q == cudaSuccess) q = cudaEventRecord(b->ev_ba[0], b->adv);
            if (q == cudaSuccess) q = cudaStreamWaitEvent(b->stream, b->ev_ba[0], 0);
            if (q != cudaSuccess) s = cuda_fail(RSC_ERR_CUDA, "advance tuning step: %s", cudaGetErrorString(q));
            b->launches += 2;
        }
        if (s) break;
        if (cudaEventRecord(ev.b, b->stream) != cudaSuccess || cudaEventSynchronize(ev.b) != cudaSuccess ||
            cudaEventElapsedTime(&ms, ev.a, ev.b) != cudaSuccess) {
            s = cuda_fail(RSC_ERR_CUDA, "advance tuning timing");
            break;
        }
        if (ms < best) {
            best = ms;
            best_t = shapes[c][0];
            best_p = shapes[c][1];
        }
    }
    (void)cudaStreamSynchronize(b->stream);
    free_ptr(svel);
    free_ptr(srnd);
    free_ptr(sadv);
    if (s) return s;
    b->adv_threads = best_t;
    b->adv_per_sm = best_p;
    s = batch_advance_smem(b, best_t, best_p, &b->adv_smem);
    if (s == RSC_OK) s = batch_prepare(b, b->h_steps);
    return s;
}

}  // namespace

extern "C" {

int rsc_batch_set_advance_shape(rsc_batch *b, int threads, int blocks_per_sm) {
    int s = check_batch(b);
    if (s) return s;
    if (threads != 64 && threads != 128 && threads != 256) return fail(RSC_ERR_ARG, "advance threads %d", threads);
    if (blocks_per_sm < 0 || blocks_per_sm * threads > 2048) {
        return fail(RSC_ERR_ARG, "advance blocks per SM %d at %d threads", blocks_per_sm, threads);
    }
    size_t smem = 0;
    s = batch_advance_smem(b, threads, blocks_per_sm, &smem);
    if (s) return s;
    b->adv_threads = threads;
    b->adv_per_sm = blocks_per_sm;
    b->adv_smem = smem;
    batch_drop_graph(b);
    return RSC_OK;
}

int rsc_batch_get_advance_shape(rsc_batch *b, int *threads, int *blocks_per_sm) {
    if (b == nullptr) return fail(RSC_ERR_ARG, "batch is NULL");
    if (threads) *threads = b->adv_threads;
    if (blocks_per_sm) *blocks_per_sm = b->adv_per_sm;
    return RSC_OK;
}

int rsc_batch_autotune(rsc_batch *b, const float *sim_descs) {
    int s = check_batch(b);
    if (s) return s;
    if (sim_descs == nullptr) return fail(RSC_ERR_ARG, "sim_descs is NULL");
    s = batch_reserve(b, 1);
    if (s) return s;
    s = batch_fill_steps(b, 1, sim_descs, nullptr);
    if (s) return s;
    s = batch_join_workers(b);
    if (s) return s;
    const size_t n = b->w.size();
    batch_fill_pairs(b, 1);
    RSC_CUDA(cudaMemcpyAsync(b->d_steps, b->h_steps, n * sizeof(rsc::BatchStep), cudaMemcpyHostToDevice, b->stream));
    RSC_CUDA(cudaEventRecord(b->ev_h2d, b->stream));
    EventPair ev;
    RSC_CUDA(ev.init());
    float best = INFINITY;
    int best_w = 0, best_p = 0;
    for (int warps : kTuneWarps) {
        for (int per_sm = 1; per_sm <= 4; per_sm++) {
            b->tune_warps = warps;
            b->tune_per_sm = per_sm;
            s = batch_prepare(b, b->h_steps);
            if (s) return s;
            if (b->pulse_threads != warps * 32 || b->pulse_per_sm != per_sm) continue;
            RSC_CUDA(batch_launch_pulse(b, 0));
            RSC_CUDA(cudaEventRecord(ev.a, b->stream));
            for (int r = 0; r < kTuneReps; r++) RSC_CUDA(batch_launch_pulse(b, 0));
            RSC_CUDA(cudaEventRecord(ev.b, b->stream));
            RSC_CUDA(cudaEventSynchronize(ev.b));
            float ms = 0.0f;
            RSC_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
            b->launches += 1 + kTuneReps;
            if (ms < best) {
                best = ms;
                best_w = warps;
                best_p = per_sm;
            }
        }
    }
    b->tune_warps = best_w;
    b->tune_per_sm = best_p;
    s = batch_prepare(b, b->h_steps);
    if (s == RSC_OK) s = batch_tune_advance(b);
    if (s) return s;
    batch_drop_graph(b);
    RSC_CUDA(cudaEventRecord(b->ev_done, b->stream));
    for (rsc_worker *x : b->w) RSC_CUDA(cudaStreamWaitEvent(x->stream, b->ev_done, 0));
    return RSC_OK;
}

}  // extern "C"

namespace {

/* Cost of one scatterer in the persistent form's partition, in units of a
 * pulse term: the pulse (1) plus its advance -- a background scatterer's
 * about one more, a debris scatterer's (attitude, ADM lookups, tumble,
 * debris RCS) about eight. */
constexpr double kPersistRainCost = 2.0, kPersistDebrisCost = 9.0, kPersistIdleCost = 1.0;

void *persist_kernel_for(int mode, bool tri) {
    if (mode == RSC_PULSE_PLAIN) {
        return tri ? reinterpret_cast<void *>(rsc::k_batch_persist<0, 1>)
                   : reinterpret_cast<void *>(rsc::k_batch_persist<0, -1>);
    }
    return tri ? reinterpret_cast<void *>(rsc::k_batch_persist<1, 1>) : reinterpret_cast<void *>(rsc::k_batch_persist<1, -1>);
}

/* Cut every instance into segments of equal cost per block (64-aligned
 * within the instance), one list per block, and size the accumulators for
 * `steps` steps. */
int batch_persist_prepare(rsc_batch *b, int steps) {
    const size_t n = b->w.size();
    const size_t threads = rsc::kPersistThreads;
    const size_t smem = (threads / 32) * rsc::pulse_warp_bytes(b->mode, b->Gmax) + 2 * b->Gmax * sizeof(float);
    void *kern = persist_kernel_for(b->mode, b->tri);
    if (smem > 48 * 1024) {
        RSC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    int per_sm = 0;
    RSC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (int)threads, smem));
    if (per_sm < 1) return fail(RSC_ERR_UNSUPPORTED, "the persistent batch kernel does not fit an SM (%zu B)", smem);
    if (per_sm > 4) per_sm = 4;
    const unsigned nb = (unsigned)(b->num_sms * per_sm);
    /* piecewise-constant cost over each instance's indices */
    struct Piece {
        int inst;
        unsigned long long lo, hi;
        double w;
    };
    std::vector<Piece> pieces;
    for (size_t i = 0; i < n; i++) {
        const rsc_worker *x = b->w[i];
        const rsc_population &pop = b->pops[i];
        std::vector<std::tuple<unsigned long long, unsigned long long, double>> r;
        for (int k = 0; k < RSC_MAX_TYPES; k++) {
            if (pop.counts[k] == 0) continue;
            r.emplace_back(pop.origins[k], pop.origins[k] + pop.counts[k], k == 0 ? kPersistRainCost : kPersistDebrisCost);
        }
        std::sort(r.begin(), r.end());
        unsigned long long at = 0;
        for (const auto &q : r) {
            const unsigned long long lo = std::min<unsigned long long>(std::get<0>(q), x->num_scats);
            const unsigned long long hi = std::min<unsigned long long>(std::get<1>(q), x->num_scats);
            if (lo > at) pieces.push_back({(int)i, at, lo, kPersistIdleCost});
            if (hi > std::max(lo, at)) pieces.push_back({(int)i, std::max(lo, at), hi, std::get<2>(q)});
            at = std::max(at, hi);
        }
        if (at < x->num_scats) pieces.push_back({(int)i, at, x->num_scats, kPersistIdleCost});
    }
    double total = 0.0;
    for (const Piece &p : pieces) total += (double)(p.hi - p.lo) * p.w;
    const double target = total / nb;
    std::vector<std::vector<rsc::PersistSeg>> per(nb);
    unsigned blk = 0;
    double cum = 0.0;
    for (const Piece &p : pieces) {
        unsigned long long cur = p.lo;
        while (cur < p.hi) {
            unsigned long long cut = p.hi;
            if (blk + 1 < nb) {
                const double room = target * (blk + 1) - cum;
                const unsigned long long take = room <= 0.0 ? 0 : (unsigned long long)ceil(room / p.w);
                const unsigned long long c = ((cur + take + 63) / 64) * 64;   /* 64-aligned in the instance */
                if (c < p.hi) cut = std::max(c, cur + 1);
            }
            auto &v = per[blk];
            if (!v.empty() && v.back().inst == p.inst && v.back().end == cur) {
                v.back().end = cut;
            } else {
                v.push_back({cur, cut, p.inst, 0});
            }
            cum += (double)(cut - cur) * p.w;
            cur = cut;
            if (blk + 1 < nb && cum >= target * (blk + 1) - 1e-9) blk++;
        }
    }
    std::vector<rsc::PersistSeg> seg;
    std::vector<unsigned> off(nb + 1, 0u), nblk(n, 0u);
    for (unsigned q = 0; q < nb; q++) {
        off[q] = (unsigned)seg.size();
        int last = -1;
        for (const auto &g : per[q]) {
            seg.push_back(g);
            if (g.inst != last) nblk[g.inst]++;
            last = g.inst;
        }
    }
    off[nb] = (unsigned)seg.size();
    for (size_t i = 0; i < n; i++) {
        if (nblk[i] == 0) return fail(RSC_ERR_STATE, "persistent partition left instance %zu without a block", i);
    }
    if (seg.size() > b->pseg_cap || b->d_pseg_off == nullptr) {
        free_ptr(b->d_pseg);
        free_ptr(b->d_pseg_off);
        free_ptr(b->d_pnblk);
        b->pseg_cap = 0;
        cudaError_t e = cudaMalloc((void **)&b->d_pseg, seg.size() * sizeof(rsc::PersistSeg));
        if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_pseg_off, (size_t)(4 * b->num_sms + 1) * sizeof(unsigned));
        if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_pnblk, n * sizeof(unsigned));
        if (e != cudaSuccess) return cuda_fail(RSC_ERR_NOMEM, "persistent segments: %s", cudaGetErrorString(e));
        b->pseg_cap = seg.size();
    }
    const size_t slots = (size_t)steps * n;
    if (slots > b->pacc_cap) {
        free_ptr(b->d_pacc);
        free_ptr(b->d_ptick);
        b->pacc_cap = 0;
        cudaError_t e = cudaMalloc((void **)&b->d_pacc, slots * b->Gmax * 4 * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_ptick, slots * sizeof(unsigned));
        if (e != cudaSuccess) return cuda_fail(RSC_ERR_NOMEM, "persistent accumulators: %s", cudaGetErrorString(e));
        b->pacc_cap = slots;
    }
    RSC_CUDA(cudaMemcpyAsync(b->d_pseg, seg.data(), seg.size() * sizeof(rsc::PersistSeg), cudaMemcpyHostToDevice,
                             b->stream));
    RSC_CUDA(cudaMemcpyAsync(b->d_pseg_off, off.data(), off.size() * sizeof(unsigned), cudaMemcpyHostToDevice,
                             b->stream));
    RSC_CUDA(cudaMemcpyAsync(b->d_pnblk, nblk.data(), n * sizeof(unsigned), cudaMemcpyHostToDevice, b->stream));
    /* the copies read host vectors of this call: wait before they go */
    RSC_CUDA(cudaStreamSynchronize(b->stream));
    b->persist_blocks = nb;
    b->persist_smem = smem;
    return RSC_OK;
}

/* Every step of the run in one launch (after zeroing its accumulators). */
int batch_persist_launch(rsc_batch *b, int steps) {
    const size_t n = b->w.size();
    const size_t slots = (size_t)steps * n;
    RSC_CUDA(cudaMemsetAsync(b->d_pacc, 0, slots * b->Gmax * 4 * sizeof(double), b->stream));
    RSC_CUDA(cudaMemsetAsync(b->d_ptick, 0, slots * sizeof(unsigned), b->stream));
    rsc::PersistArgs A;
    memset(&A, 0, sizeof(A));
    A.adv = b->d_adv;
    A.pulse = b->d_pulse;
    A.steps = b->d_steps;
    A.seg = b->d_pseg;
    A.seg_off = b->d_pseg_off;
    A.nblk = b->d_pnblk;
    A.acc = b->d_pacc;
    A.tick = b->d_ptick;
    A.out = b->d_out;
    A.out_stride = b->Gmax;
    A.Gmax = b->Gmax;
    A.steps_n = steps;
    A.ninst = (int)n;
    const unsigned g = b->persist_blocks;
    const size_t sm = b->persist_smem;
    const unsigned t = rsc::kPersistThreads;
    if (b->mode == RSC_PULSE_PLAIN && b->tri) {
        rsc::k_batch_persist<0, 1><<<g, t, sm, b->stream>>>(A);
    } else if (b->mode == RSC_PULSE_PLAIN) {
        rsc::k_batch_persist<0, -1><<<g, t, sm, b->stream>>>(A);
    } else if (b->tri) {
        rsc::k_batch_persist<1, 1><<<g, t, sm, b->stream>>>(A);
    } else {
        rsc::k_batch_persist<1, -1><<<g, t, sm, b->stream>>>(A);
    }
    RSC_CUDA(cudaGetLastError());
    b->launches += 1;
    return RSC_OK;
}

int batch_run(rsc_batch *b, int steps, const float *sim_descs, const int *les_ids, float *pulses_out, int use_graph,
              bool wait) {
    int s = check_batch(b);
    if (s) return s;
    if (steps < 1) return fail(RSC_ERR_ARG, "steps %d", steps);
    if (sim_descs == nullptr || les_ids == nullptr) return fail(RSC_ERR_ARG, "sim_descs / les_ids is NULL");
    s = batch_reserve(b, steps);
    if (s) return s;
    s = batch_fill_steps(b, steps, sim_descs, les_ids);
    if (s) return s;
    for (rsc_worker *x : b->w) {
        s = flush_pending(x);
        if (s == RSC_OK) s = settle_sig_aux(x, x->stream);
        if (s) return s;
    }
    s = batch_join_workers(b);
    if (s) return s;
    const size_t n = b->w.size();
    for (size_t i = 0; i < n; i++) {
        s = maybe_sort(b->w[i], &b->pops[i], b->h_steps[i].sim, b->stream);
        if (s) return s;
        /* the advances write both pairs: scatterers outside the population
         * ranges carry over into the other one */
        s = copy_unadvanced(b->w[i], &b->pops[i], b->stream);
        if (s) return s;
    }
    s = batch_prepare(b, b->h_steps);
    if (s) return s;
    batch_fill_pairs(b, steps);
    /* LES slots this run reads: wait for their pending refills */
    std::vector<char> used(2 * n, 0);
    for (size_t r = 0; r < (size_t)steps * n; r++) used[2 * (r % n) + (b->h_steps[r].les_id & 1)] = 1;
    for (size_t q = 0; q < 2 * n; q++) {
        if (used[q] && b->slot_pending[q]) {
            RSC_CUDA(cudaStreamWaitEvent(b->stream, b->slot_ready[q], 0));
            b->slot_pending[q] = 0;
        }
        rsc_worker *x = b->w[q / 2];
        if (used[q] && x->les_wait[q & 1]) {
            /* a frame from rsc_les_upload_async */
            RSC_CUDA(cudaStreamWaitEvent(b->stream, x->les_ready[q & 1], 0));
            x->les_wait[q & 1] = false;
        }
    }
    RSC_CUDA(cudaMemcpyAsync(b->d_steps, b->h_steps, (size_t)steps * n * sizeof(rsc::BatchStep),
                             cudaMemcpyHostToDevice, b->stream));
    RSC_CUDA(cudaEventRecord(b->ev_h2d, b->stream));
    if (b->persist && b->mode != RSC_PULSE_F64) {
        s = batch_persist_prepare(b, steps);
        if (s == RSC_OK) s = batch_persist_launch(b, steps);
        if (s) return s;
    } else if (use_graph) {
        if (b->graph == nullptr || b->graph_steps != steps) {
            s = batch_capture(b, steps);
            if (s) return s;
        }
        RSC_CUDA(cudaGraphLaunch(b->graph, b->stream));
        b->launches += (uint64_t)steps * (1u + (b->rain_blocks ? 1u : 0u) + (b->deb_blocks ? 1u : 0u));
    } else {
        RSC_CUDA(batch_enqueue(b, steps));
        b->launches += (uint64_t)steps * (1u + (b->rain_blocks ? 1u : 0u) + (b->deb_blocks ? 1u : 0u));
    }
    batch_swap_pairs(b, steps);
    for (size_t q = 0; q < 2 * n; q++) {
        if (used[q]) RSC_CUDA(cudaEventRecord(b->slot_used[q], b->stream));
    }
    if (pulses_out) {
        RSC_CUDA(cudaMemcpyAsync(pulses_out, b->d_out, (size_t)steps * n * b->Gmax * sizeof(float4),
                                 cudaMemcpyDeviceToHost, b->stream));
    }
    RSC_CUDA(cudaEventRecord(b->ev_done, b->stream));
    for (size_t i = 0; i < n; i++) {
        rsc_worker *x = b->w[i];
        x->since_sort += (uint64_t)steps;
        RSC_CUDA(cudaStreamWaitEvent(x->stream, b->ev_done, 0));
        s = release_main(x);   /* the batch changed the state in place */
        if (s) return s;
        memcpy(x->last_sim, sim_descs + ((size_t)(steps - 1) * n + i) * 16, sizeof(x->last_sim));
        x->have_pulse_desc = true;
        x->sig_aux_stale = true;
        /* the last step's pulse read the pair its advance did not write */
        const bool advanced = b->rain_blocks != 0 || b->deb_blocks != 0;
        x->sa_pos = advanced ? x->pos_next : x->pos;
        x->sa_rcs = advanced ? x->rcs_next : x->rcs;
    }
    if (pulses_out && wait) RSC_CUDA(cudaStreamSynchronize(b->stream));
    return RSC_OK;
}

}  // namespace

extern "C" {

int rsc_batch_run(rsc_batch *b, int steps, const float *sim_descs, const int *les_ids, float *pulses_out,
                  int use_graph) {
    return batch_run(b, steps, sim_descs, les_ids, pulses_out, use_graph, true);
}

int rsc_batch_run_async(rsc_batch *b, int steps, const float *sim_descs, const int *les_ids, float *pulses_out,
                        int use_graph) {
    return batch_run(b, steps, sim_descs, les_ids, pulses_out, use_graph, false);
}

int rsc_batch_synchronize(rsc_batch *b) {
    int s = check_batch(b);
    if (s) return s;
    RSC_CUDA(cudaStreamSynchronize(b->stream));
    RSC_CUDA(cudaStreamSynchronize(b->copy_stream));
    return RSC_OK;
}

int rsc_batch_set_les_async(rsc_batch *b, int index, int slot, const float *uvwt4, const float *cpxx4, uint32_t nx,
                            uint32_t ny, uint32_t nz) {
    int s = check_batch(b);
    if (s) return s;
    if (index < 0 || index >= (int)b->w.size()) return fail(RSC_ERR_ARG, "instance %d of %zu", index, b->w.size());
    if (slot < 0 || slot > 1) return fail(RSC_ERR_ARG, "LES slot %d", slot);
    if (uvwt4 == nullptr) return fail(RSC_ERR_ARG, "uvwt is NULL");
    rsc_worker *x = b->w[index];
    if (x->les_uvwt[slot] == nullptr || nx != x->les_nx || ny != x->les_ny || nz != x->les_nz) {
        return fail(RSC_ERR_STATE, "instance %d: LES of %ux%ux%u not set with rsc_set_les", index, nx, ny, nz);
    }
    const size_t q = 2 * (size_t)index + slot;
    const size_t nn = (size_t)nx * ny * nz, bytes = nn * sizeof(float4);
    /* uvwt to the batch's staging buffer (reused in copy-stream order) */
    s = ensure_buffer(&b->les_stage, &b->les_stage_n, nn, b->copy_stream);
    if (s) return s;
    RSC_CUDA(cudaMemcpyAsync(b->les_stage, uvwt4, bytes, cudaMemcpyHostToDevice, b->copy_stream));
    /* the slot changes after the last batch run and any worker-stream work that read it */
    s = flush_pending(x);   /* the worker's stream after its advance stream */
    if (s) return s;
    RSC_CUDA(cudaStreamWaitEvent(b->copy_stream, b->slot_used[q], 0));
    RSC_CUDA(cudaEventRecord(b->ev_join, x->stream));
    RSC_CUDA(cudaStreamWaitEvent(b->copy_stream, b->ev_join, 0));
    rsc::k_les_pairs<<<les_grid(nx, (size_t)ny * nz), rsc::kLesThreads, 0, b->copy_stream>>>(
        b->les_stage, (int)nx, (size_t)ny * nz, x->les_uvwt[slot]);
    RSC_CUDA(cudaGetLastError());
    b->launches++;
    if (cpxx4) RSC_CUDA(cudaMemcpyAsync(x->les_cpxx[slot], cpxx4, bytes, cudaMemcpyHostToDevice, b->copy_stream));
    RSC_CUDA(cudaEventRecord(b->slot_ready[q], b->copy_stream));
    b->slot_pending[q] = 1;
    return RSC_OK;
}

int rsc_batch_max_gates(rsc_batch *b, int *max_gates) {
    if (b == nullptr || max_gates == nullptr) return fail(RSC_ERR_ARG, "NULL argument");
    *max_gates = (int)b->Gmax;
    return RSC_OK;
}

int rsc_batch_launch_count(rsc_batch *b, uint64_t *count) {
    if (b == nullptr || count == nullptr) return fail(RSC_ERR_ARG, "NULL argument");
    *count = b->launches;
    return RSC_OK;
}

int rsc_batch_get_stream(rsc_batch *b, void **stream) {
    if (b == nullptr || stream == nullptr) return fail(RSC_ERR_ARG, "NULL argument");
    *stream = (void *)b->stream;
    return RSC_OK;
}

int rsc_batch_set_persistent(rsc_batch *b, int enable) {
    if (b == nullptr) return fail(RSC_ERR_ARG, "batch is NULL");
    b->persist = enable != 0;
    return RSC_OK;
}

int rsc_batch_get_shape(rsc_batch *b, int *warps, int *blocks_per_sm) {
    if (b == nullptr) return fail(RSC_ERR_ARG, "batch is NULL");
    if (warps) *warps = b->tune_warps;
    if (blocks_per_sm) *blocks_per_sm = b->tune_per_sm;
    return RSC_OK;
}

/* ---- pulse formation that allocates nothing ---------------------------------
 * The pulse kernel needs scratch memory beyond its inputs and outputs: an FP64
 * accumulator per gate and lane, a completion counter, and the gate origins
 * and weight tables in device memory.  rsc_make_pulse takes them from buffers
 * rsc_worker_malloc allocated.  rsc_make_pulse_noalloc takes them from the
 * fixed array below instead, so a caller that must not allocate device memory
 * can still form a pulse from its own device buffers. */
#define RSC_NA_ACC_OFF 0
#define RSC_NA_ACC_BYTES ((size_t)RSC_NOALLOC_MAX_GATES * 4 * sizeof(double))
#define RSC_NA_RK_OFF (RSC_NA_ACC_OFF + RSC_NA_ACC_BYTES)
#define RSC_NA_RW_OFF (RSC_NA_RK_OFF + (size_t)RSC_NOALLOC_MAX_GATES * 4)
#define RSC_NA_AW_OFF (RSC_NA_RW_OFF + (size_t)RSC_NOALLOC_MAX_RANGE_TABLE * 4)
#define RSC_NA_COUNTER_OFF (RSC_NA_AW_OFF + (size_t)RSC_NOALLOC_MAX_ANGULAR_TABLE * 4)
#define RSC_NA_BYTES (RSC_NA_COUNTER_OFF + 256)

/* One copy per device that loads this library, held until the process exits.
 * Host code only ever uses the address cudaGetSymbolAddress returns for it. */
static __device__ __align__(256) unsigned char g_pulse_scratch[RSC_NA_BYTES];

namespace {

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_na_mu;
void *g_na_addr[kNoAllocMaxDevices] = {nullptr};

/* Device address of g_pulse_scratch on the current device, looked up once per
 * device (the first call on each device does it, with that device current). */
int noalloc_scratch(void **out) {
    int dev = 0;
    RSC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(RSC_ERR_UNSUPPORTED, "device %d", dev);
    std::lock_guard<std::mutex> lock(g_na_mu);
    if (g_na_addr[dev] == nullptr) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_pulse_scratch);
        if (e != cudaSuccess || p == nullptr) {
            return cuda_fail(RSC_ERR_CUDA, "cudaGetSymbolAddress(pulse scratch) on device %d: %s", dev,
                        cudaGetErrorString(e));
        }
        g_na_addr[dev] = p;
    }
    *out = g_na_addr[dev];
    return RSC_OK;
}

/* What the pulse kernel's scratch must hold before it runs, passed by value
 * in the launch's parameters (about 4.4 KB), so the call reads no host
 * memory after it returns and queues no host-to-device copy. */
struct NoAllocSetup {
    float rw[RSC_NOALLOC_MAX_RANGE_TABLE];
    float aw[RSC_NOALLOC_MAX_ANGULAR_TABLE];
    uint32_t rw_n, aw_n, G;
    float range_start, range_delta;
    unsigned char *scratch;
};

/* Fill the scratch: the weight tables, the gate origins as the FP32 running
 * sum of make_pulse_pass_1 (rs.cl:1214), and a zero accumulator and counter
 * (the pulse kernel leaves both at zero, but a launch that failed part way
 * might not have).  One block. */
__global__ void __launch_bounds__(256) k_noalloc_setup(const NoAllocSetup a) {
    float *rk = reinterpret_cast<float *>(a.scratch + RSC_NA_RK_OFF);
    float *rw = reinterpret_cast<float *>(a.scratch + RSC_NA_RW_OFF);
    float *aw = reinterpret_cast<float *>(a.scratch + RSC_NA_AW_OFF);
    double *acc = reinterpret_cast<double *>(a.scratch + RSC_NA_ACC_OFF);
    for (uint32_t i = threadIdx.x; i < a.rw_n; i += blockDim.x) rw[i] = a.rw[i];
    for (uint32_t i = threadIdx.x; i < a.aw_n; i += blockDim.x) aw[i] = a.aw[i];
    for (uint32_t i = threadIdx.x; i < 4 * a.G; i += blockDim.x) acc[i] = 0.0;
    if (threadIdx.x == 0) {
        float r = a.range_start;
        for (uint32_t k = 0; k < a.G; k++) {
            rk[k] = r;
            r = r + a.range_delta;
        }
        *reinterpret_cast<unsigned *>(a.scratch + RSC_NA_COUNTER_OFF) = 0u;
    }
}

}  // namespace

int rsc_make_pulse_noalloc(const float *pos4, const float *rcs4, size_t num_scats, const float *range_weight,
                           uint32_t range_n, const float range_desc[4], const float *angular_weight,
                           uint32_t angular_n, const float angular_desc[4], float range_start, float range_delta,
                           uint32_t range_count, const float sim_desc[16], float *pulse4, void *stream) {
    if (pos4 == nullptr || rcs4 == nullptr || pulse4 == nullptr || range_weight == nullptr ||
        range_desc == nullptr || angular_weight == nullptr || angular_desc == nullptr || sim_desc == nullptr) {
        return fail(RSC_ERR_ARG, "rsc_make_pulse_noalloc: NULL argument");
    }
    if (num_scats == 0) return fail(RSC_ERR_ARG, "rsc_make_pulse_noalloc: num_scats is 0");
    if (range_count == 0 || range_count > RSC_NOALLOC_MAX_GATES) {
        return fail(RSC_ERR_ARG, "rsc_make_pulse_noalloc: range_count %u outside [1, %d]", range_count,
                    RSC_NOALLOC_MAX_GATES);
    }
    if (range_n == 0 || range_n > RSC_NOALLOC_MAX_RANGE_TABLE) {
        return fail(RSC_ERR_ARG, "rsc_make_pulse_noalloc: range weight table of %u entries, limit %d", range_n,
                    RSC_NOALLOC_MAX_RANGE_TABLE);
    }
    if (angular_n == 0 || angular_n > RSC_NOALLOC_MAX_ANGULAR_TABLE) {
        return fail(RSC_ERR_ARG, "rsc_make_pulse_noalloc: angular weight table of %u entries, limit %d", angular_n,
                    RSC_NOALLOC_MAX_ANGULAR_TABLE);
    }
    /* the descriptors' max index must lie inside the table: compared as
     * floats before any conversion (a NaN or a huge value fails here) */
    if (!(range_desc[2] >= 0.0f && range_desc[2] < (float)range_n) ||
        !(angular_desc[2] >= 0.0f && angular_desc[2] < (float)angular_n)) {
        return fail(RSC_ERR_ARG, "rsc_make_pulse_noalloc: table max index beyond its table");
    }
    if (!(fabsf(range_start) < INFINITY) || !(fabsf(range_delta) < INFINITY)) {
        return fail(RSC_ERR_ARG, "rsc_make_pulse_noalloc: range_start / range_delta not finite");
    }
    void *base = nullptr;
    int s = noalloc_scratch(&base);
    if (s) return s;
    unsigned char *b = static_cast<unsigned char *>(base);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint32_t G = range_count;
    NoAllocSetup setup;
    memset(&setup, 0, sizeof(setup));
    memcpy(setup.rw, range_weight, range_n * sizeof(float));
    memcpy(setup.aw, angular_weight, angular_n * sizeof(float));
    setup.rw_n = range_n;
    setup.aw_n = angular_n;
    setup.G = G;
    setup.range_start = range_start;
    setup.range_delta = range_delta;
    setup.scratch = b;
    PulseArgs P;
    memset(&P, 0, sizeof(P));
    P.pos = reinterpret_cast<const float4 *>(pos4);
    P.rcs = reinterpret_cast<const float4 *>(rcs4);
    P.n = num_scats;
    P.aw = reinterpret_cast<const float *>(b + RSC_NA_AW_OFF);
    memcpy(P.awd, angular_desc, sizeof(P.awd));
    P.rw = reinterpret_cast<const float *>(b + RSC_NA_RW_OFF);
    memcpy(P.rwd, range_desc, sizeof(P.rwd));
    P.rk = reinterpret_cast<const float *>(b + RSC_NA_RK_OFF);
    P.G = G;
    memcpy(P.sim, sim_desc, sizeof(P.sim));
    rsc::beam_norm_df(P.sim, P.bn_hi, P.bn_lo);
    P.rs = range_start;
    P.inv_delta = range_delta != 0.0f ? 1.0f / range_delta : 0.0f;
    P.rdelta = range_delta;
    P.rw_n = range_n;
    for (uint32_t k = 0; k < 4; k++) P.rwv[k] = k < range_n ? range_weight[k] : 0.0f;
    P.rw_tri = is_triangle(range_n, P.rwv, range_desc) ? 1 : 0;
    P.acc64 = reinterpret_cast<double *>(b + RSC_NA_ACC_OFF);
    P.counter = reinterpret_cast<unsigned *>(b + RSC_NA_COUNTER_OFF);
    P.pulse = reinterpret_cast<float4 *>(pulse4);
    /* sparse gate window when both edge weights are zero (see fill_pulse_args);
     * the drift of the FP32 running sum is measured on the host */
    P.dense = 1;
    const float xs = range_desc[0], x0 = range_desc[1], xm = range_desc[2];
    if (range_delta > 0.0f && xs > 0.0f && range_weight[0] == 0.0f && range_weight[(uint32_t)xm] == 0.0f) {
        double d_lo = -(double)x0 / (double)xs, d_hi = ((double)xm - (double)x0) / (double)xs;
        double drift = 0.0;
        float rf = range_start;
        for (uint32_t k = 0; k < G; k++) {
            drift = fmax(drift, fabs((double)rf - ((double)range_start + (double)k * (double)range_delta)));
            rf = rf + range_delta;
        }
        const double margin = window_margin(drift, range_start, range_delta, G, d_lo, d_hi);
        double lo = d_lo / (double)range_delta - margin, hi = d_hi / (double)range_delta + margin;
        if (hi - lo + 1.0 < (double)rsc::kMaxCandidates) {
            P.dense = 0;
            P.win_lo = (float)lo;
            P.win_hi = (float)hi;
        }
    }
    /* launch geometry of the plain pulse kernel */
    const PulseKernel kern = pulse_kernel(RSC_PULSE_PLAIN, pulse_path(P, RSC_PULSE_PLAIN));
    int dev = 0, sms = 0, per_sm = 1;
    RSC_CUDA(cudaGetDevice(&dev));
    RSC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int threads = 16 * 32;
    const size_t smem = 16 * rsc::pulse_warp_bytes(RSC_PULSE_PLAIN, G) + 2 * G * sizeof(float);
    RSC_CUDA(kernel_occupancy(kern, threads, smem, &per_sm));
    if (per_sm < 1) per_sm = 1;
    if (per_sm > 4) per_sm = 4;
    const int grid = sms * per_sm;
    k_noalloc_setup<<<1, 256, 0, st>>>(setup);
    RSC_CUDA(cudaGetLastError());
    kern<<<grid, threads, smem, st>>>(P);
    RSC_CUDA(cudaGetLastError());
    return RSC_OK;
}

int rsc_eval_math(int fn, const float *a, const float *b, float *out, size_t n) {
    if (a == nullptr || out == nullptr || n == 0) return fail(RSC_ERR_ARG, "eval_math arguments");
    float *da = nullptr, *db = nullptr, *dout = nullptr;
    RSC_CUDA(cudaMalloc((void **)&da, n * sizeof(float)));
    RSC_CUDA(cudaMalloc((void **)&db, n * sizeof(float)));
    RSC_CUDA(cudaMalloc((void **)&dout, n * sizeof(float)));
    RSC_CUDA(cudaMemcpy(da, a, n * sizeof(float), cudaMemcpyHostToDevice));
    RSC_CUDA(cudaMemcpy(db, b ? b : a, n * sizeof(float), cudaMemcpyHostToDevice));
    if (fn >= 9 && fn <= 12) {
        rsc::k_eval_phase<<<(unsigned)((n + 255) / 256), 256>>>(fn, da, db, dout, n);
    } else {
        rsc::k_eval_math<<<(unsigned)((n + 255) / 256), 256>>>(fn, da, db, dout, n);
    }
    RSC_CUDA(cudaGetLastError());
    RSC_CUDA(cudaMemcpy(out, dout, n * sizeof(float), cudaMemcpyDeviceToHost));
    cudaFree(da);
    cudaFree(db);
    cudaFree(dout);
    return RSC_OK;
}

}  // extern "C"
