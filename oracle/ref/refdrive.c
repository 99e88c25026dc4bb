/*
 * refdrive.c -- runs one session of the reference host (rs.c, unmodified) on
 * the CPU oracle device of clshim.c and records it.
 *
 * TEST INFRASTRUCTURE ONLY (built into oracle/_ref/ by oracle/ref/Makefile).
 *
 * The session is simradar's (simradar.c:796-1074) at a reduced density:
 * RS_init, concept, scan pattern, density, seed, Marshall-Palmer DSD, the LES
 * configuration, 30 m sampling, RS_suggest_scan_domain, debris, the debris
 * count rounding, RS_set_scan_box, RS_populate, warm-up advances at a PRT of
 * 1/60 s, then per pulse RS_make_pulse, RS_download_pulse_only,
 * RS_merge_pulse_tmp, RS_advance_time and RS_advance_beam.  The tables come
 * from the folder $HOME/Documents/tables, where the reference looks for them
 * (les.c:71-126, adm.c:56-110, rcs.c:93-145).
 *
 * Everything rs.c sends to the device is observed through the shim's hook
 * and written to OUT as named arrays:
 *   - the tables and descriptors rs.c derived (range / angular weight,
 *     ellipsoid RCS, ADM and RCS images, LES descriptor, population layout,
 *     radar parameters, DSD), read back from the device objects;
 *   - the event list: state uploads, LES frame writes (slot, frame), time
 *     advances (with the simulation descriptor and LES slot the kernels got,
 *     and with concept bit 7 the debris flux field table and descriptor
 *     db_atts read, as an index into dff_tables / dff_descs),
 *     debris RCS refreshes and pulses (descriptor, the pulse rs.c read back,
 *     the merged pulse with its gain, and the oracle's per-gate sums of |term|
 *     for the tolerance);
 *   - FNV-1a hashes of the uploaded state, of every LES frame written and of
 *     the final state, and a subsample of the final state.
 *
 * File format: "RSREF001", then records of name[48], dtype[8] ("f4", "u4",
 * "i4", "f8", "u8"), ndim (u32), pad (u32), shape[4] (u64), nbytes (u64) and
 * the data.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rs.h"
#include "rsoracle.h"
#include "clshim.h"

#define MAX_EVENTS 65536
#define MAX_PULSES 8192

enum { EV_UPLOAD = 5, EV_LES = 1, EV_ADVANCE = 2, EV_DEBRIS_RCS = 3, EV_PULSE = 4 };

typedef struct {
    uint32_t kind;
    int32_t i[4];
    float desc[16];
} Event;

static RSHandle *H;
static Event *g_ev;
static int g_nev;
static double *g_abs, *g_direct;  /* [pulse][gate][4] oracle sums of |term| and of term */
static int g_npulse_ev;       /* pulses formed (including RS_populate's) */
static int g_cur_pulse = -1;  /* event index of the latest pulse */
static uint64_t g_les_hash[256][2];
static int g_nles;
static uint64_t g_init_hash[8];
static int g_uploads;
static uint64_t g_deb_launch[8][4];
static int g_ndeb = -1;
/* debris flux field tables db_atts was given (concept bit 7), each kept once
 * in the order first seen, with the descriptor it came with */
#define MAX_DFF 64
static float *g_dff_tab[MAX_DFF];
static float g_dff_desc[MAX_DFF][16];
static size_t g_dff_n;
static int g_ndff;
static int g_adv_deb;         /* debris launches in the current advance */
static int g_fail;

static uint64_t fnv1a(const void *p, size_t n, uint64_t h) {
    const unsigned char *c = (const unsigned char *)p;
    for (size_t i = 0; i < n; i++) {
        h ^= c[i];
        h *= 1099511628211ull;
    }
    return h;
}
#define FNV0 14695981039346656037ull

static Event *new_event(uint32_t kind) {
    if (g_nev >= MAX_EVENTS) {
        fprintf(stderr, "refdrive: too many events\n");
        exit(2);
    }
    Event *e = &g_ev[g_nev++];
    memset(e, 0, sizeof(*e));
    e->kind = kind;
    e->i[0] = e->i[1] = e->i[2] = e->i[3] = -1;
    return e;
}

static int slot_of(cl_mem m, cl_mem *slots, int n) {
    for (int i = 0; i < n; i++) {
        if (slots[i] == m) return i;
    }
    return -1;
}

static void hook(const clshim_event *ev, void *user) {
    (void)user;
    RSWorker *C = &H->workers[0];
    if (ev->kind == CLSHIM_WRITE_BUFFER) {
        cl_mem arrays[8] = {C->scat_pos, C->scat_vel, C->scat_ori, C->scat_tum, C->scat_aux, C->scat_rcs,
                            C->scat_sig, C->scat_rnd};
        int a = slot_of(ev->mem, arrays, 8);
        if (a < 0) return;
        if (a == 0) {
            new_event(EV_UPLOAD);
            g_uploads++;
        }
        if (ev->offset != 0) {
            fprintf(stderr, "refdrive: state upload at offset %zu\n", ev->offset);
            g_fail = 1;
        }
        g_init_hash[a] = fnv1a(ev->ptr, ev->size, FNV0);
        return;
    }
    if (ev->kind == CLSHIM_WRITE_IMAGE) {
        int s = slot_of(ev->mem, C->les_uvwt, 2);
        int sc = slot_of(ev->mem, C->les_cpxx, 2);
        if (s >= 0) {
            Event *e = new_event(EV_LES);
            e->i[0] = s;
            e->i[1] = (int32_t)H->vel_idx;
            if (g_nles < 256) g_les_hash[g_nles][0] = fnv1a(ev->ptr, ev->size, FNV0);
        } else if (sc >= 0) {
            if (g_nles < 256) g_les_hash[g_nles][1] = fnv1a(ev->ptr, ev->size, FNV0);
            g_nles++;
        }
        return;
    }
    if (ev->kind != CLSHIM_LAUNCH) return;
    const char *n = ev->name;
    if (!strcmp(n, "el_atts") || !strcmp(n, "bg_atts") || !strcmp(n, "fp_atts")) {
        Event *e = new_event(EV_ADVANCE);
        cl_mem uvwt;
        clshim_kernel_arg(ev->kernel, 4, &uvwt, sizeof(uvwt));
        e->i[0] = slot_of(uvwt, C->les_uvwt, 2);
        e->i[1] = 0;
        e->i[2] = !strcmp(n, "bg_atts") ? 0 : (!strcmp(n, "el_atts") ? 1 : 2);
        clshim_kernel_arg(ev->kernel, 9, e->desc, sizeof(e->desc));
        if (ev->global_offset != C->origins[0] || ev->global_size != C->counts[0]) {
            fprintf(stderr, "refdrive: background launch [%zu, +%zu) is not the type-0 range\n", ev->global_offset,
                    ev->global_size);
            g_fail = 1;
        }
        g_adv_deb = 0;
    } else if (!strcmp(n, "db_atts")) {
        if (g_nev == 0 || g_ev[g_nev - 1].kind != EV_ADVANCE) {
            fprintf(stderr, "refdrive: debris launch outside an advance\n");
            g_fail = 1;
            return;
        }
        Event *e = &g_ev[g_nev - 1];
        cl_mem cd, rr;
        clshim_kernel_arg(ev->kernel, 9, &cd, sizeof(cd));
        clshim_kernel_arg(ev->kernel, 12, &rr, sizeof(rr));
        uint64_t rec[4] = {ev->global_offset, ev->global_size, (uint64_t)slot_of(cd, C->adm_cd, RS_MAX_ADM_TABLES),
                           (uint64_t)slot_of(rr, C->rcs_real, RS_MAX_RCS_TABLES)};
        /* the first advance fixes the debris launch list; later ones repeat it */
        if (g_ndeb < 0) g_ndeb = 0;
        if (g_adv_deb < 8) {
            if (g_adv_deb >= g_ndeb) {
                memcpy(g_deb_launch[g_adv_deb], rec, sizeof(rec));
                g_ndeb = g_adv_deb + 1;
            } else if (memcmp(g_deb_launch[g_adv_deb], rec, sizeof(rec)) != 0) {
                fprintf(stderr, "refdrive: debris launch %d changed between advances\n", g_adv_deb);
                g_fail = 1;
            }
        }
        if (H->sim_concept & RSSimulationConceptDebrisFluxFromVelocity) {
            /* the table (argument 15, dff_icdf[les_id]) and its descriptor
             * (16) this launch reads, recorded against the advance */
            cl_mem dm;
            float dd[16];
            size_t bytes = 0;
            clshim_kernel_arg(ev->kernel, 15, &dm, sizeof(dm));
            clshim_kernel_arg(ev->kernel, 16, dd, sizeof(dd));
            const float *tab = (const float *)clshim_mem_data(dm, &bytes, NULL);
            const size_t n = bytes / sizeof(float);
            int idx = -1;
            if (g_ndff > 0 && n == g_dff_n && !memcmp(g_dff_tab[g_ndff - 1], tab, bytes) &&
                !memcmp(g_dff_desc[g_ndff - 1], dd, sizeof(dd))) {
                idx = g_ndff - 1;
            } else if (g_ndff < MAX_DFF && (g_ndff == 0 || n == g_dff_n)) {
                g_dff_tab[g_ndff] = (float *)malloc(bytes);
                memcpy(g_dff_tab[g_ndff], tab, bytes);
                memcpy(g_dff_desc[g_ndff], dd, sizeof(dd));
                g_dff_n = n;
                idx = g_ndff++;
            } else {
                fprintf(stderr, "refdrive: debris flux field tables beyond %d or of changing size\n", MAX_DFF);
                g_fail = 1;
            }
            if (e->i[3] >= 0 && e->i[3] != idx) {
                fprintf(stderr, "refdrive: debris launches of one advance read different flux tables\n");
                g_fail = 1;
            }
            e->i[3] = idx;
        }
        float sd[16];
        clshim_kernel_arg(ev->kernel, 17, sd, sizeof(sd));
        if (memcmp(sd, e->desc, sizeof(sd)) != 0) {
            fprintf(stderr, "refdrive: debris and background got different descriptors\n");
            g_fail = 1;
        }
        g_adv_deb++;
        e->i[1] = g_adv_deb;
    } else if (!strcmp(n, "db_rcs")) {
        Event *e;
        if (g_nev > 0 && g_ev[g_nev - 1].kind == EV_DEBRIS_RCS) {
            e = &g_ev[g_nev - 1];
        } else {
            e = new_event(EV_DEBRIS_RCS);
            e->i[1] = 0;
            clshim_kernel_arg(ev->kernel, 6, e->desc, sizeof(e->desc));
        }
        e->i[1]++;
    } else if (!strcmp(n, "scat_sig_aux")) {
        Event *e = new_event(EV_PULSE);
        clshim_kernel_arg(ev->kernel, 6, e->desc, sizeof(e->desc));
        e->i[0] = -1;                 /* set when the pulse is read back */
        e->i[1] = g_npulse_ev;
        g_cur_pulse = g_nev - 1;
        /* the oracle's exact per-gate sums of the FP32 terms and of |term|,
         * from the state the kernel is about to read */
        if (g_npulse_ev < MAX_PULSES) {
            const uint32_t G = H->params.range_count;
            size_t bytes;
            const of4 *pos = (const of4 *)clshim_mem_data(C->scat_pos, &bytes, NULL);
            const of4 *rcs = (const of4 *)clshim_mem_data(C->scat_rcs, NULL, NULL);
            const float *aw = (const float *)clshim_mem_data(C->angular_weight, NULL, NULL);
            const float *rw = (const float *)clshim_mem_data(C->range_weight, NULL, NULL);
            float awd[4], rwd[4];
            clshim_kernel_arg(ev->kernel, 5, awd, sizeof(awd));
            clshim_kernel_arg(C->kern_make_pulse_pass_1, 5, rwd, sizeof(rwd));
            or_make_pulse_direct(g_direct + (size_t)g_npulse_ev * G * 4, g_abs + (size_t)g_npulse_ev * G * 4, pos, rcs,
                                 ev->global_size, aw, awd, rw, rwd, H->params.range_start, H->params.range_delta, G,
                                 e->desc);
        }
        g_npulse_ev++;
    }
}

/* ---- output ---- */

static FILE *g_out;

static void put(const char *name, const char *dtype, const void *data, size_t nbytes, int ndim, uint64_t d0,
                uint64_t d1, uint64_t d2, uint64_t d3) {
    char nm[48] = {0}, dt[8] = {0};
    snprintf(nm, sizeof(nm), "%s", name);
    snprintf(dt, sizeof(dt), "%s", dtype);
    uint32_t nd[2] = {(uint32_t)ndim, 0};
    uint64_t shape[4] = {d0, d1, d2, d3};
    uint64_t nb = nbytes;
    fwrite(nm, 1, 48, g_out);
    fwrite(dt, 1, 8, g_out);
    fwrite(nd, 4, 2, g_out);
    fwrite(shape, 8, 4, g_out);
    fwrite(&nb, 8, 1, g_out);
    if (nbytes) fwrite(data, 1, nbytes, g_out);
}

static void put_f1(const char *name, const float *v, size_t n) { put(name, "f4", v, n * 4, 1, n, 0, 0, 0); }
static void put_scalar_f(const char *name, float v) { put(name, "f4", &v, 4, 0, 0, 0, 0, 0); }
static void put_scalar_u(const char *name, uint64_t v) { put(name, "u8", &v, 8, 0, 0, 0, 0, 0); }

static void put_mem(const char *name, cl_mem m) {
    size_t bytes, dims[3];
    const void *p = clshim_mem_data(m, &bytes, dims);
    if (p == NULL) {
        fprintf(stderr, "refdrive: %s is not a device object\n", name);
        g_fail = 1;
        return;
    }
    if (dims[2] > 1) {
        put(name, "f4", p, bytes, 4, dims[2], dims[1], dims[0], 4);
    } else if (dims[1] > 1) {
        put(name, "f4", p, bytes, 3, dims[1], dims[0], 4, 0);
    } else {
        put(name, "f4", p, bytes, 1, bytes / 4, 0, 0, 0);
    }
}

static void usage(void) {
    fprintf(stderr,
            "usage: refdrive OUT [--density D] [--scan S] [--pulses K] [--warmup W] [--seed N] [--concept BITS]\n"
            "                    [--les CONFIG] [--debris TYPE:COUNT]... [--gate M] [--bundle DIR]\n"
            "                    [--kernels oracle|rscl]\n");
    exit(2);
}

int main(int argc, char **argv) {
    if (argc < 2) usage();
    const char *out_path = argv[1];
    float density = 0.3f, gate = 30.0f;
    const char *scan_str = "P:3.0,-12:12:0.24";
    int pulses = 40, warmup = 0, seed = 19760520;
    unsigned concept = RSSimulationConceptDraggedBackground | RSSimulationConceptBoundedParticleVelocity |
                       RSSimulationConceptUniformDSDScaledRCS;
    const char *les = LESConfigSuctionVortices;
    const char *bundle = ".";
    int deb_type[8], deb_count[8], ndeb = 0;
    for (int i = 2; i < argc; i++) {
        if (!strcmp(argv[i], "--density") && i + 1 < argc) density = (float)atof(argv[++i]);
        else if (!strcmp(argv[i], "--scan") && i + 1 < argc) scan_str = argv[++i];
        else if (!strcmp(argv[i], "--pulses") && i + 1 < argc) pulses = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--warmup") && i + 1 < argc) warmup = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--seed") && i + 1 < argc) seed = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--concept") && i + 1 < argc) concept = (unsigned)strtoul(argv[++i], NULL, 0);
        else if (!strcmp(argv[i], "--les") && i + 1 < argc) les = argv[++i];
        else if (!strcmp(argv[i], "--gate") && i + 1 < argc) gate = (float)atof(argv[++i]);
        else if (!strcmp(argv[i], "--bundle") && i + 1 < argc) bundle = argv[++i];
        else if (!strcmp(argv[i], "--kernels") && i + 1 < argc) {
            /* oracle: the oracle's restatement; rscl: the reference's rs.cl */
            const char *kk = argv[++i];
            if (!strcmp(kk, "rscl")) clshim_set_kernels(CLSHIM_KERNELS_RSCL);
            else if (!strcmp(kk, "oracle")) clshim_set_kernels(CLSHIM_KERNELS_ORACLE);
            else usage();
        } else if (!strcmp(argv[i], "--debris") && i + 1 < argc && ndeb < 8) {
            if (sscanf(argv[++i], "%d:%d", &deb_type[ndeb], &deb_count[ndeb]) != 2) usage();
            ndeb++;
        } else usage();
    }
    if (pulses > MAX_PULSES - 2) usage();

    g_ev = (Event *)calloc(MAX_EVENTS, sizeof(Event));
    clshim_set_hook(hook, NULL);

    /* simradar.c:796-955 */
    /* RS_init_verbose with the folder of rs_enum.h / rs.cl given (the shim
     * reads the kernel source; it runs the oracle's kernels, or with
     * --kernels rscl the reference's rs.cl compiled for the CPU) */
    H = RS_init_with_path(bundle, RS_METHOD_GPU, 0xFF, 0, 0);
    if (H == NULL) return 3;
    RS_set_concept(H, concept);
    POSPattern scan;
    memset(&scan, 0, sizeof(scan));
    POS_parse_from_string(&scan, scan_str);
    RS_set_scan_pattern(H, &scan);
    RS_set_density(H, density);
    RS_set_random_seed(H, seed);
    if (!(H->sim_concept & RSSimulationConceptFixedScattererPosition)) RS_set_dsd_to_mp(H);
    RS_set_vel_data_to_config(H, (LESConfig)les);
    RS_set_sampling_spacing(H, gate, 1.0f, 1.0f);
    RSBox box = RS_suggest_scan_domain(H);
    for (int k = 0; k < ndeb; k++) RS_add_debris(H, deb_type[k], deb_count[k]);
    RS_revise_debris_counts_to_gpu_preference(H);
    RS_set_scan_box(H, box);
    const float prt = H->params.prt;
    const uint32_t G = H->params.range_count;
    g_abs = (double *)calloc((size_t)(pulses + 2) * G * 4, sizeof(double));
    g_direct = (double *)calloc((size_t)(pulses + 2) * G * 4, sizeof(double));
    RS_populate(H);
    RSWorker *C = &H->workers[0];
    if (warmup > 0) {
        RS_set_prt(H, 1.0f / 60.0f);
        for (int k = 0; k < warmup; k++) RS_advance_time(H);
    }
    RS_set_prt(H, prt);
    float *raw = (float *)calloc((size_t)pulses * G * 4, sizeof(float));
    float *merged = (float *)calloc((size_t)pulses * G * 4, sizeof(float));
    float *abs4 = (float *)calloc((size_t)pulses * G * 4, sizeof(float));
    double *direct = (double *)calloc((size_t)pulses * G * 4, sizeof(double));
    for (int k = 0; k < pulses; k++) {
        RS_make_pulse(H);
        RS_download_pulse_only(H);
        RS_merge_pulse_tmp(H);
        if (g_cur_pulse < 0) return 4;
        Event *e = &g_ev[g_cur_pulse];
        e->i[0] = k;
        memcpy(raw + (size_t)k * G * 4, H->pulse_tmp[0], G * 16);
        memcpy(merged + (size_t)k * G * 4, H->pulse, G * 16);
        for (size_t j = 0; j < (size_t)G * 4; j++) {
            abs4[(size_t)k * G * 4 + j] = (float)g_abs[(size_t)e->i[1] * G * 4 + j];
            direct[(size_t)k * G * 4 + j] = g_direct[(size_t)e->i[1] * G * 4 + j];
        }
        RS_advance_time(H);
        RS_advance_beam(H);
    }
    RS_download(H);

    g_out = fopen(out_path, "wb");
    if (g_out == NULL) return 5;
    fwrite("RSREF001", 1, 8, g_out);
    /* scene and radar parameters */
    put_scalar_u("num_scats", C->num_scats);
    put_scalar_u("num_types", H->num_types);
    put_scalar_u("range_count", G);
    put_scalar_f("range_start", H->params.range_start);
    put_scalar_f("range_delta", H->params.range_delta);
    put_scalar_f("antenna_gain_dbi", H->params.antenna_gain_dbi);
    put_scalar_f("tx_power_watt", H->params.tx_power_watt);
    put_scalar_f("prt", prt);
    put_scalar_f("lambda", H->params.lambda);
    put_scalar_u("random_seed", H->random_seed);
    put_scalar_u("sim_concept", H->sim_concept);
    put_scalar_u("adm_count", C->adm_count);
    put_scalar_u("rcs_count", C->rcs_count);
    uint64_t oc[2][RS_MAX_DEBRIS_TYPES];
    for (int k = 0; k < RS_MAX_DEBRIS_TYPES; k++) {
        oc[0][k] = C->origins[k];
        oc[1][k] = C->counts[k];
    }
    put("origins", "u8", oc[0], sizeof(oc[0]), 1, RS_MAX_DEBRIS_TYPES, 0, 0, 0);
    put("counts", "u8", oc[1], sizeof(oc[1]), 1, RS_MAX_DEBRIS_TYPES, 0, 0, 0);
    RSVolume dom = RS_get_domain(H);
    float domain[6] = {dom.origin.x, dom.origin.y, dom.origin.z, dom.size.x, dom.size.y, dom.size.z};
    put_f1("domain", domain, 6);
    put_f1("sim_desc_final", H->sim_desc.s, 16);
    if (H->dsd_count > 0) {
        put_f1("dsd_r", H->dsd_r, H->dsd_count);
        put_f1("dsd_cdf", H->dsd_cdf, H->dsd_count);
        uint64_t pop[64];
        for (int i = 0; i < H->dsd_count && i < 64; i++) pop[i] = H->dsd_pop[i];
        put("dsd_pop", "u8", pop, 8 * (size_t)(H->dsd_count < 64 ? H->dsd_count : 64), 1,
            H->dsd_count < 64 ? H->dsd_count : 64, 0, 0, 0);
    }
    /* tables and descriptors as rs.c left them on the device */
    put_mem("range_weight", C->range_weight);
    put_f1("range_weight_desc", C->range_weight_desc.s, 4);
    put_mem("angular_weight", C->angular_weight);
    put_f1("angular_weight_desc", C->angular_weight_desc.s, 4);
    put_mem("rcs_ellipsoid", C->rcs_ellipsoid);
    put_f1("rcs_ellipsoid_desc", C->rcs_ellipsoid_desc.s, 4);
    put_f1("les_desc", C->les_desc.s, 16);
    size_t ldims[3];
    clshim_mem_data(C->les_uvwt[0], NULL, ldims);
    uint64_t ld[3] = {ldims[0], ldims[1], ldims[2]};
    put("les_dims", "u8", ld, sizeof(ld), 1, 3, 0, 0, 0);
    char nm[48];
    for (unsigned a = 0; a < C->adm_count; a++) {
        snprintf(nm, sizeof(nm), "adm_cd_%u", a);
        put_mem(nm, C->adm_cd[a]);
        snprintf(nm, sizeof(nm), "adm_cm_%u", a);
        put_mem(nm, C->adm_cm[a]);
        snprintf(nm, sizeof(nm), "adm_desc_%u", a);
        put_f1(nm, C->adm_desc[a].s, 16);
    }
    for (unsigned r = 0; r < C->rcs_count; r++) {
        snprintf(nm, sizeof(nm), "rcs_real_%u", r);
        put_mem(nm, C->rcs_real[r]);
        snprintf(nm, sizeof(nm), "rcs_imag_%u", r);
        put_mem(nm, C->rcs_imag[r]);
        snprintf(nm, sizeof(nm), "rcs_desc_%u", r);
        put_f1(nm, C->rcs_desc[r].s, 16);
    }
    put_f1("dff_desc", C->dff_desc.s, 16);
    if (g_ndff > 0) {
        float *all = (float *)malloc((size_t)g_ndff * g_dff_n * sizeof(float));
        for (int k = 0; k < g_ndff; k++) memcpy(all + (size_t)k * g_dff_n, g_dff_tab[k], g_dff_n * sizeof(float));
        put("dff_tables", "f4", all, (size_t)g_ndff * g_dff_n * 4, 2, g_ndff, g_dff_n, 0, 0);
        put("dff_descs", "f4", g_dff_desc, (size_t)g_ndff * 64, 2, g_ndff, 16, 0, 0);
        free(all);
    }
    /* events */
    uint32_t *kinds = (uint32_t *)malloc((size_t)g_nev * 4);
    int32_t *ints = (int32_t *)malloc((size_t)g_nev * 16);
    float *descs = (float *)malloc((size_t)g_nev * 64);
    for (int i = 0; i < g_nev; i++) {
        kinds[i] = g_ev[i].kind;
        memcpy(ints + 4 * i, g_ev[i].i, 16);
        memcpy(descs + 16 * i, g_ev[i].desc, 64);
    }
    put("ev_kind", "u4", kinds, (size_t)g_nev * 4, 1, g_nev, 0, 0, 0);
    put("ev_int", "i4", ints, (size_t)g_nev * 16, 2, g_nev, 4, 0, 0);
    put("ev_desc", "f4", descs, (size_t)g_nev * 64, 2, g_nev, 16, 0, 0);
    if (g_ndeb > 0) put("debris_launches", "u8", g_deb_launch, (size_t)g_ndeb * 32, 2, g_ndeb, 4, 0, 0);
    put("pulse_raw", "f4", raw, (size_t)pulses * G * 16, 3, pulses, G, 4, 0);
    put("pulse_merged", "f4", merged, (size_t)pulses * G * 16, 3, pulses, G, 4, 0);
    put("pulse_abs", "f4", abs4, (size_t)pulses * G * 16, 3, pulses, G, 4, 0);
    put("pulse_direct", "f8", direct, (size_t)pulses * G * 32, 3, pulses, G, 4, 0);
    /* hashes */
    put("init_hash", "u8", g_init_hash, sizeof(g_init_hash), 1, 8, 0, 0, 0);
    put("les_hash", "u8", g_les_hash, (size_t)g_nles * 16, 2, g_nles, 2, 0, 0);
    cl_mem arrays[8] = {C->scat_pos, C->scat_vel, C->scat_ori, C->scat_tum, C->scat_aux, C->scat_rcs, C->scat_sig,
                        C->scat_rnd};
    static const char *names[8] = {"pos", "vel", "ori", "tum", "aux", "rcs", "sig", "rnd"};
    uint64_t fh[8];
    const size_t N = C->num_scats;
    const size_t step = 8, ns = (N + step - 1) / step;
    float *sub = (float *)malloc(ns * 16);
    for (int a = 0; a < 8; a++) {
        const unsigned char *p = (const unsigned char *)clshim_mem_data(arrays[a], NULL, NULL);
        fh[a] = fnv1a(p, N * 16, FNV0);
        for (size_t i = 0; i < ns; i++) memcpy(sub + 4 * i, p + 16 * (i * step), 16);
        snprintf(nm, sizeof(nm), "final_%s_every8", names[a]);
        put(nm, a == 7 ? "u4" : "f4", sub, ns * 16, 2, ns, 4, 0, 0);
    }
    put("final_hash", "u8", fh, sizeof(fh), 1, 8, 0, 0, 0);
    /* launches the device ran */
    static const char *kn[] = {"el_atts", "bg_atts", "fp_atts", "db_atts", "db_rcs", "scat_sig_aux",
                               "make_pulse_pass_1", "make_pulse_pass_2_local", "make_pulse_pass_2_range",
                               "make_pulse_pass_2_group"};
    uint64_t lc[10];
    for (int i = 0; i < 10; i++) lc[i] = clshim_launches(kn[i]);
    put("launches", "u8", lc, sizeof(lc), 1, 10, 0, 0, 0);
    put_scalar_u("uploads", (uint64_t)g_uploads);
    put_scalar_u("failed", (uint64_t)g_fail);
    fclose(g_out);
    printf("refdrive: %zu scatterers, %u gates, %d events, %d pulses, %d LES writes%s\n", N, G, g_nev, pulses, g_nles,
           g_fail ? ", FAILED checks" : "");
    RS_free(H);
    return g_fail ? 6 : 0;
}
