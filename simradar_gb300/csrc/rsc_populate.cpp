/*
 * rsc_populate.cpp -- the initial scatterer state of RS_populate (rs.c:4568-
 * 4814) on the host.
 *
 * RS_populate draws every value from the C library's rand() in a fixed
 * order, so the same seed gives the same scatterers only through the same
 * generator.  RandState is the glibc generator (random_r, TYPE_3): the
 * published additive lagged-Fibonacci recurrence r[i] = r[i-3] + r[i-31]
 * (mod 2^32) returning r[i] >> 1, its 31 words seeded by the Park-Miller
 * step 16807 r mod (2^31 - 1) (Schrage's factorisation), its first 310
 * outputs discarded, seed 0 taken as 1.  It reproduces glibc's rand() on
 * x86-64 and aarch64 alike; it is sequential, as RS_populate is.
 *
 * Order of the draws (the branch of RS_populate without fixed positions):
 * for each type, each scatterer of the worker: x, y, z (z within 10 m of the
 * domain floor), age, then the four respawn seeds; then srand(2 seed) and,
 * for the background type, one draw per scatterer for its drop-size bin.
 * Every "(float)rand() / RAND_MAX * a + b" is formed with FP32 roundings
 * after each operation (no fused multiply-add).
 */
#include "rsc_populate.h"

#include <string.h>

namespace rscpop {

namespace {
constexpr int32_t kRandMax = 2147483647;

inline float unit(RandState *s) { return (float)rand_next(s) / (float)kRandMax; }

inline float span(RandState *s, float size, float origin) {
    volatile float t = unit(s) * size;   /* two roundings, as RS_populate compiles without contraction */
    return t + origin;
}
}  // namespace

void rand_seed(RandState *s, uint32_t seed) {
    int32_t word = (int32_t)(seed == 0 ? 1u : seed);
    s->r[0] = (uint32_t)word;
    for (int i = 1; i < 31; i++) {
        const int32_t hi = word / 127773;
        const int32_t lo = word % 127773;
        word = 16807 * lo - 2836 * hi;
        if (word < 0) word += kRandMax;
        s->r[i] = (uint32_t)word;
    }
    for (int i = 31; i < 34; i++) s->r[i] = s->r[i - 31];
    for (int i = 34; i < 344; i++) s->r[i % 34] = s->r[(i + 3) % 34] + s->r[(i + 31) % 34];
    s->pos = 344 % 34;
}

int32_t rand_next(RandState *s) {
    const int p = s->pos;
    const uint32_t v = s->r[(p + 3) % 34] + s->r[(p + 31) % 34];   /* r[i - 31] + r[i - 3] */
    s->r[p] = v;
    s->pos = p + 1 == 34 ? 0 : p + 1;
    return (int32_t)(v >> 1);
}

int Generator::init(const rsc_populate_args *args, const char **why) {
    a = *args;
    if (a.num_types < 1 || a.num_types > RSC_MAX_TYPES) {
        *why = "num_types outside [1, RSC_MAX_TYPES]";
        return RSC_ERR_ARG;
    }
    if (a.sim_concept & 0x20u) {
        *why = "fixed-position scatterers (anchor planes) are populated by rs.c";
        return RSC_ERR_UNSUPPORTED;
    }
    uint64_t acc = 0;
    for (uint32_t k = 0; k < a.num_types; k++) {
        if (a.origins[k] != acc) {
            *why = "type ranges must follow one another from slot 0";
            return RSC_ERR_ARG;
        }
        acc += a.counts[k];
    }
    if (a.dsd_count > 0 && (a.dsd_r == nullptr || a.dsd_cdf == nullptr)) {
        *why = "DSD tables are NULL";
        return RSC_ERR_ARG;
    }
    total = (size_t)acc;
    next_slot = 0;
    rand_seed(&main_rs, a.seed);
    rand_seed(&dsd_rs, a.seed + a.seed);
    return RSC_OK;
}

void Generator::fill(size_t n, float *pos4, float *aux4, uint32_t *rnd4, uint32_t *dsd_pop) {
    const size_t rain_end = (size_t)a.counts[0];
    for (size_t j = 0; j < n && next_slot < total; j++, next_slot++) {
        const float x = span(&main_rs, a.domain_size[0], a.domain_origin[0]);
        const float y = span(&main_rs, a.domain_size[1], a.domain_origin[1]);
        const float z = span(&main_rs, 10.0f, a.domain_origin[2]);
        const float age = unit(&main_rs);
        float radius = 0.0f, bin_index = 0.0f;
        for (int q = 0; q < 4; q++) rnd4[4 * j + q] = (uint32_t)rand_next(&main_rs);
        if (next_slot < rain_end && a.dsd_count > 0) {
            const float u = unit(&dsd_rs);
            int bin = 0;
            if (a.sim_concept & 0x10u) {   /* uniform DSD, scaled RCS */
                bin = (int)(u * (float)a.dsd_count);
            } else {
                for (int k = (int)a.dsd_count - 1; k >= 0; k--) {
                    if (u >= a.dsd_cdf[k]) {
                        bin = k;
                        break;
                    }
                }
            }
            if (dsd_pop) dsd_pop[bin]++;
            radius = a.dsd_r[bin];
            bin_index = ((float)bin + 0.5f) / (float)a.dsd_count;
        }
        pos4[4 * j + 0] = x;
        pos4[4 * j + 1] = y;
        pos4[4 * j + 2] = z;
        pos4[4 * j + 3] = radius;
        aux4[4 * j + 0] = 0.0f;
        aux4[4 * j + 1] = age;
        aux4[4 * j + 2] = bin_index;
        aux4[4 * j + 3] = 1.0f;
    }
}

}  // namespace rscpop

namespace {
thread_local char g_pop_err[256] = "";
int pop_fail(int code, const char *msg) {
    strncpy(g_pop_err, msg, sizeof(g_pop_err) - 1);
    return code;
}
}  // namespace

extern "C" {

const char *rsc_populate_last_error(void) { return g_pop_err; }

int rsc_rand_sequence(uint32_t seed, uint32_t count, int32_t *out) {
    if (out == nullptr && count) return pop_fail(RSC_ERR_ARG, "out is NULL");
    rscpop::RandState s;
    rscpop::rand_seed(&s, seed);
    for (uint32_t i = 0; i < count; i++) out[i] = rscpop::rand_next(&s);
    return RSC_OK;
}

int rsc_populate_host(const rsc_populate_args *args, size_t num_scats, float *pos4, float *vel4, float *ori4,
                      float *tum4, float *aux4, float *rcs4, uint32_t *rnd4, uint32_t *dsd_pop) {
    if (args == nullptr || pos4 == nullptr || aux4 == nullptr || rnd4 == nullptr) {
        return pop_fail(RSC_ERR_ARG, "NULL argument");
    }
    rscpop::Generator g;
    const char *why = "";
    int s = g.init(args, &why);
    if (s) return pop_fail(s, why);
    if (g.total > num_scats) return pop_fail(RSC_ERR_ARG, "the type ranges exceed num_scats");
    if (dsd_pop && args->dsd_count) memset(dsd_pop, 0, args->dsd_count * sizeof(uint32_t));
    memset(pos4, 0, num_scats * 16);
    memset(aux4, 0, num_scats * 16);
    memset(rnd4, 0, num_scats * 16);
    g.fill(g.total, pos4, aux4, rnd4, dsd_pop);
    const float ori[4] = {0.5f, -0.5f, -0.5f, 0.5f}, tum[4] = {0.0f, 0.0f, 0.0f, 1.0f};
    const float rcs[4] = {1.0f, 0.0f, 1.0f, 0.0f}, vel[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (size_t i = 0; i < num_scats; i++) {
        const bool used = i < g.total;
        for (int q = 0; q < 4; q++) {
            if (vel4) vel4[4 * i + q] = vel[q];
            if (ori4) ori4[4 * i + q] = used ? ori[q] : 0.0f;
            if (tum4) tum4[4 * i + q] = used ? tum[q] : 0.0f;
            if (rcs4) rcs4[4 * i + q] = used ? rcs[q] : 0.0f;
        }
    }
    return RSC_OK;
}

}  // extern "C"
