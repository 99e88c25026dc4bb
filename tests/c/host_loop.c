/*
 * host_loop.c -- a C99 host that drives the backend through include/rsc.h
 * exactly as rs.c would after the integration (each rs.c step below mapped
 * to the calls that replace its OpenCL block), replaying a session recorded
 * from the reference host.
 *
 * Input (argv[1]): a record file (RSREF001 format, written by
 * tests/test_gpu_ref_session.py from tests/golden/ref_session_*.npz): the
 * tables, descriptors, population layout, DSD and event list rs.c produced.
 * argv[2]: the LES folder (<tables>/les/suctvort).  argv[3]: the output
 * record file.
 *
 *   rsc_worker_create / rsc_worker_malloc              RS_worker_init / RS_worker_malloc
 *   rsc_set_range_weight / _angular_weight / _rcs_ellipsoid / _adm / _rcs
 *                                                      the table setters
 *   rsc_les_open, rsc_les_descriptor, rsc_les_read + rsc_set_les,
 *   rsc_les_upload_async                               RS_set_vel_data_to_config,
 *                                                      the frame swap of RS_advance_time
 *   rsc_populate_upload                                RS_populate + RS_upload
 *   rsc_advance_time / rsc_update_debris_rcs / rsc_make_pulse
 *   rsc_download_pulse (gain 1, and the gain of RS_merge_pulse_tmp)
 *   rsc_download                                       RS_download
 *
 * The population block follows rs.c's type ranges and the round-robin
 * ADM / RCS table indices of rs.c:5351-5373.  Output: the pulses read back, the merged and
 * scaled pulses, FNV-1a hashes of the uploaded state, of every LES frame
 * read and of the final state, and the final state every 8th scatterer.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rsc.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

enum { EV_LES = 1, EV_ADVANCE = 2, EV_DEBRIS_RCS = 3, EV_PULSE = 4, EV_UPLOAD = 5 };

/* ---- record files ---- */

typedef struct {
    char name[48];
    char dtype[8];
    uint32_t ndim;
    uint64_t shape[4];
    uint64_t nbytes;
    unsigned char *data;
} Rec;

static Rec *g_recs;
static int g_nrec;

static int read_records(const char *path) {
    FILE *f = fopen(path, "rb");
    if (f == NULL) return -1;
    char magic[8];
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "RSREF001", 8) != 0) {
        fclose(f);
        return -2;
    }
    int cap = 64;
    g_recs = (Rec *)calloc(cap, sizeof(Rec));
    for (;;) {
        Rec r;
        uint32_t nd[2];
        if (fread(r.name, 1, 48, f) != 48) break;
        if (fread(r.dtype, 1, 8, f) != 8 || fread(nd, 4, 2, f) != 2 || fread(r.shape, 8, 4, f) != 4 ||
            fread(&r.nbytes, 8, 1, f) != 1) {
            fclose(f);
            return -3;
        }
        r.ndim = nd[0];
        r.data = (unsigned char *)malloc(r.nbytes ? r.nbytes : 1);
        if (r.nbytes && fread(r.data, 1, r.nbytes, f) != r.nbytes) {
            fclose(f);
            return -4;
        }
        if (g_nrec == cap) {
            cap *= 2;
            g_recs = (Rec *)realloc(g_recs, cap * sizeof(Rec));
        }
        g_recs[g_nrec++] = r;
    }
    fclose(f);
    return 0;
}

static const Rec *find(const char *name) {
    for (int i = 0; i < g_nrec; i++) {
        if (strcmp(g_recs[i].name, name) == 0) return &g_recs[i];
    }
    return NULL;
}

static const void *need(const char *name) {
    const Rec *r = find(name);
    if (r == NULL) {
        fprintf(stderr, "host_loop: record %s missing\n", name);
        exit(2);
    }
    return r->data;
}

static uint64_t need_u(const char *name) { return *(const uint64_t *)need(name); }
static float need_f(const char *name) { return *(const float *)need(name); }

static FILE *g_out;

static void put(const char *name, const char *dtype, const void *data, uint64_t nbytes, uint32_t ndim, uint64_t d0,
                uint64_t d1, uint64_t d2) {
    char nm[48] = {0}, dt[8] = {0};
    strncpy(nm, name, sizeof(nm) - 1);
    strncpy(dt, dtype, sizeof(dt) - 1);
    uint32_t nd[2] = {ndim, 0};
    uint64_t shape[4] = {d0, d1, d2, 0};
    fwrite(nm, 1, 48, g_out);
    fwrite(dt, 1, 8, g_out);
    fwrite(nd, 4, 2, g_out);
    fwrite(shape, 8, 4, g_out);
    fwrite(&nbytes, 8, 1, g_out);
    if (nbytes) fwrite(data, 1, nbytes, g_out);
}

static uint64_t fnv1a(const void *p, size_t n) {
    const unsigned char *c = (const unsigned char *)p;
    uint64_t h = 14695981039346656037ull;
    for (size_t i = 0; i < n; i++) {
        h ^= c[i];
        h *= 1099511628211ull;
    }
    return h;
}

#define CHECK(call)                                                                                 \
    do {                                                                                            \
        int st_ = (call);                                                                           \
        if (st_ != RSC_OK) {                                                                        \
            fprintf(stderr, "host_loop: %s failed (%d): %s\n", #call, st_, rsc_last_error());        \
            exit(3);                                                                                \
        }                                                                                           \
    } while (0)

static void hash_state(rsc_worker *w, size_t n, uint64_t h[8], float **keep) {
    float *a[8];
    for (int k = 0; k < 8; k++) a[k] = (float *)malloc(n * 16);
    CHECK(rsc_download(w, 0, n, a[0], a[1], a[2], a[3], a[4], a[5], a[6], (uint32_t *)a[7]));
    for (int k = 0; k < 8; k++) {
        h[k] = fnv1a(a[k], n * 16);
        if (keep) {
            keep[k] = a[k];
        } else {
            free(a[k]);
        }
    }
}

int main(int argc, char **argv) {
    if (argc != 4) {
        fprintf(stderr, "usage: host_loop SESSION LES_DIR OUT\n");
        return 2;
    }
    if (read_records(argv[1]) != 0) {
        fprintf(stderr, "host_loop: cannot read %s\n", argv[1]);
        return 2;
    }
    const size_t N = (size_t)need_u("num_scats");
    const uint32_t G = (uint32_t)need_u("range_count");
    const uint32_t num_types = (uint32_t)need_u("num_types");
    const uint32_t adm_count = (uint32_t)need_u("adm_count"), rcs_count = (uint32_t)need_u("rcs_count");
    const uint64_t *origins = (const uint64_t *)need("origins");
    const uint64_t *counts = (const uint64_t *)need("counts");

    /* RS_worker_init, RS_worker_malloc */
    rsc_worker *w = NULL;
    CHECK(rsc_worker_create(0, &w));
    CHECK(rsc_worker_malloc(w, N, need_f("range_start"), need_f("range_delta"), G));

    /* the table setters */
    const Rec *rw = find("range_weight"), *aw = find("angular_weight"), *el = find("rcs_ellipsoid");
    CHECK(rsc_set_range_weight(w, (const float *)rw->data, (uint32_t)(rw->nbytes / 4),
                               (const float *)need("range_weight_desc")));
    CHECK(rsc_set_angular_weight(w, (const float *)aw->data, (uint32_t)(aw->nbytes / 4),
                                 (const float *)need("angular_weight_desc")));
    CHECK(rsc_set_rcs_ellipsoid(w, (const float *)el->data, (uint32_t)(el->nbytes / 16),
                                (const float *)need("rcs_ellipsoid_desc")));
    char nm[48];
    for (uint32_t a = 0; a < adm_count; a++) {
        snprintf(nm, sizeof(nm), "adm_cd_%u", a);
        const Rec *cd = find(nm);
        snprintf(nm, sizeof(nm), "adm_cm_%u", a);
        const Rec *cm = find(nm);
        snprintf(nm, sizeof(nm), "adm_desc_%u", a);
        CHECK(rsc_set_adm(w, (int)a, (const float *)cd->data, (const float *)cm->data, (uint32_t)cd->shape[1],
                          (uint32_t)cd->shape[0], (const float *)need(nm)));
    }
    for (uint32_t r = 0; r < rcs_count; r++) {
        snprintf(nm, sizeof(nm), "rcs_real_%u", r);
        const Rec *re = find(nm);
        snprintf(nm, sizeof(nm), "rcs_imag_%u", r);
        const Rec *im = find(nm);
        snprintf(nm, sizeof(nm), "rcs_desc_%u", r);
        CHECK(rsc_set_rcs(w, (int)r, (const float *)re->data, (const float *)im->data, (uint32_t)re->shape[1],
                          (uint32_t)re->shape[0], (const float *)need(nm)));
    }

    /* the LES folder: the backend's reader and descriptor */
    rsc_les_source *src = NULL;
    if (rsc_les_open(argv[2], "suctvort", &src) != RSC_OK) {
        fprintf(stderr, "host_loop: rsc_les_open failed: %s\n", rsc_les_last_error());
        return 3;
    }
    rsc_les_info info;
    CHECK(rsc_les_get_info(src, &info));
    float les_desc[16];
    CHECK(rsc_les_descriptor(&info, les_desc));
    const size_t nn = (size_t)info.nx * info.ny * info.nz;
    float *uvwt = (float *)malloc(nn * 16), *cpxx = (float *)malloc(nn * 16);

    /* the population: rs.c's type ranges and table indices (rs.c:5351-5373) */
    rsc_population pop;
    memset(&pop, 0, sizeof(pop));
    int a = 0, r = 0;
    for (int k = 0; k < RSC_MAX_TYPES; k++) {
        pop.origins[k] = origins[k];
        pop.counts[k] = (uint32_t)k < num_types ? counts[k] : 0;
        pop.adm_index[k] = a;
        pop.rcs_index[k] = r;
        if (k >= 1) {
            r = r == (int)rcs_count - 1 ? 0 : r + 1;
            a = a == (int)adm_count - 1 ? 0 : a + 1;
        }
    }
    /* RS_populate's draws (rsc_populate_args: what RS_populate reads) */
    rsc_populate_args pa;
    memset(&pa, 0, sizeof(pa));
    pa.seed = (uint32_t)need_u("random_seed");
    pa.sim_concept = (uint32_t)need_u("sim_concept");
    const float *dom = (const float *)need("domain");
    for (int k = 0; k < 3; k++) {
        pa.domain_origin[k] = dom[k];
        pa.domain_size[k] = dom[3 + k];
    }
    pa.num_types = num_types;
    for (int k = 0; k < RSC_MAX_TYPES; k++) {
        pa.origins[k] = origins[k];
        pa.counts[k] = counts[k];
    }
    const Rec *dr = find("dsd_r");
    uint32_t dsd_pop[64];
    if (dr) {
        pa.dsd_r = (const float *)dr->data;
        pa.dsd_cdf = (const float *)need("dsd_cdf");
        pa.dsd_count = (uint32_t)(dr->nbytes / 4);
    }
    /* the gain of RS_merge_pulse_tmp (rs.c:5086), the same expression (the
     * division by 4 pi in double, as rs.c's M_PI makes it) */
    const float g = powf(10.0f, 0.1f * need_f("antenna_gain_dbi")) * sqrtf(need_f("tx_power_watt")) / (4.0f * M_PI) *
                    1.0e6f;

    const Rec *ek = find("ev_kind");
    const uint32_t *kinds = (const uint32_t *)ek->data;
    const int32_t *ints = (const int32_t *)need("ev_int");
    const float *descs = (const float *)need("ev_desc");
    const size_t nev = ek->nbytes / 4;
    const Rec *pr = find("pulse_raw");
    const size_t P = pr->shape[0];
    float *raw = (float *)calloc(P * G * 4, sizeof(float));
    float *merged = (float *)calloc(P * G * 4, sizeof(float));
    uint64_t upload_hash[8] = {0}, les_hash[64][2];
    int nles = 0;
    /* the debris flux field tables rs.c derived from each LES frame (concept
     * bit 7): each advance names the one its debris launches read, which
     * goes into the advance's LES slot as rs.c's dff_icdf[les_id] */
    const Rec *dt = find("dff_tables");
    const float *dff_tab = dt ? (const float *)dt->data : NULL;
    const float *dff_desc = dt ? (const float *)need("dff_descs") : NULL;
    const uint32_t dff_n = dt ? (uint32_t)dt->shape[1] : 0u;
    int dff_set[2] = {-1, -1};
    for (size_t e = 0; e < nev; e++) {
        const int32_t *iv = ints + 4 * e;
        const float *sd = descs + 16 * e;
        switch (kinds[e]) {
            case EV_UPLOAD:
                CHECK(rsc_populate_upload(w, &pa, dsd_pop));
                hash_state(w, N, upload_hash, NULL);
                break;
            case EV_LES: {
                float t = 0.0f;
                CHECK(rsc_les_read(src, (uint32_t)iv[1], uvwt, cpxx, &t));
                if (nles < 64) {
                    les_hash[nles][0] = fnv1a(uvwt, nn * 16);
                    les_hash[nles][1] = fnv1a(cpxx, nn * 16);
                    nles++;
                }
                if (nles == 1) {
                    /* RS_set_vel_data_to_config: the first frame, synchronously */
                    CHECK(rsc_set_les(w, iv[0], uvwt, cpxx, info.nx, info.ny, info.nz, les_desc));
                } else {
                    /* the swap of RS_advance_time: raw planes on the copy stream */
                    CHECK(rsc_les_upload_async(w, src, iv[0], (uint32_t)iv[1], &t));
                }
                break;
            }
            case EV_ADVANCE:
                if (iv[3] >= 0 && dff_tab != NULL && dff_set[iv[0] & 1] != iv[3]) {
                    CHECK(rsc_set_dff(w, iv[0], dff_tab + (size_t)iv[3] * dff_n, dff_n, dff_desc + 16 * (size_t)iv[3]));
                    dff_set[iv[0] & 1] = iv[3];
                }
                CHECK(rsc_advance_time(w, &pop, iv[0], sd));
                break;
            case EV_DEBRIS_RCS:
                CHECK(rsc_update_debris_rcs(w, &pop, sd));
                break;
            case EV_PULSE:
                CHECK(rsc_make_pulse(w, sd));
                if (iv[0] >= 0 && (size_t)iv[0] < P) {
                    CHECK(rsc_download_pulse(w, raw + (size_t)iv[0] * G * 4, 1.0f));
                    CHECK(rsc_download_pulse(w, merged + (size_t)iv[0] * G * 4, g));
                }
                break;
            default:
                fprintf(stderr, "host_loop: unknown event %u\n", kinds[e]);
                return 4;
        }
    }
    uint64_t final_hash[8];
    float *fin[8];
    hash_state(w, N, final_hash, fin);
    uint64_t launches = 0;
    CHECK(rsc_launch_count(w, &launches));

    g_out = fopen(argv[3], "wb");
    if (g_out == NULL) return 5;
    fwrite("RSREF001", 1, 8, g_out);
    put("les_desc", "f4", les_desc, sizeof(les_desc), 1, 16, 0, 0);
    put("pulse_raw", "f4", raw, P * G * 16, 3, P, G, 4);
    put("pulse_merged", "f4", merged, P * G * 16, 3, P, G, 4);
    put("upload_hash", "u8", upload_hash, sizeof(upload_hash), 1, 8, 0, 0);
    put("les_hash", "u8", les_hash, (uint64_t)nles * 16, 2, (uint64_t)nles, 2, 0);
    put("final_hash", "u8", final_hash, sizeof(final_hash), 1, 8, 0, 0);
    static const char *names[8] = {"pos", "vel", "ori", "tum", "aux", "rcs", "sig", "rnd"};
    const size_t ns = (N + 7) / 8;
    float *sub = (float *)malloc(ns * 16);
    for (int k = 0; k < 8; k++) {
        for (size_t i = 0; i < ns; i++) memcpy(sub + 4 * i, fin[k] + 4 * (i * 8), 16);
        snprintf(nm, sizeof(nm), "final_%s_every8", names[k]);
        put(nm, k == 7 ? "u4" : "f4", sub, ns * 16, 2, ns, 4, 0);
    }
    put("launches", "u8", &launches, 8, 0, 0, 0, 0);
    fclose(g_out);
    CHECK(rsc_les_close(src));
    CHECK(rsc_worker_free(w));
    printf("host_loop: %zu events, %zu pulses, %d LES frames, %llu kernel launches\n", nev, P, nles,
           (unsigned long long)launches);
    return 0;
}
