/*
 * refapi.c -- flat entry points into the reference's own loaders (les.c,
 * pos.c, adm.c, rcs.c, obj.c, compiled unmodified into oracle/_ref/libref.so)
 * for the tests' ctypes binding (oracle/refbind.py).
 *
 * TEST INFRASTRUCTURE ONLY.  Each call opens the reference module on the
 * given folder, copies out what the module produced and closes it again.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "les.h"
#include "obj.h"
#include "pos.h"

/* LES_init_with_config_path looks for <path>/tables/les/<config> (les.c:82),
 * so `parent` is the folder holding "tables".  LES_get_frame(frame) into
 * uvwt / cpxx (nn float4 each, may be NULL to query), dims = nx, ny, nz,
 * consts = tr, tp, ax, ay, az, rx, ry, rz, is_stretched, frame count. */
int ref_les_frame(const char *parent, const char *config, int frame, float *uvwt, float *cpxx, uint32_t dims[3],
                  float consts[10]) {
    LESHandle h = LES_init_with_config_path((const LESConfig)config, parent);
    if (h == NULL) return -1;
    const size_t count = LES_get_table_count(h);
    LESTable *t = LES_get_frame(h, frame);
    if (t == NULL) {
        LES_free(h);
        return -2;
    }
    dims[0] = t->nx;
    dims[1] = t->ny;
    dims[2] = t->nz;
    const float c[10] = {t->tr, t->tp, t->ax, t->ay, t->az, t->rx, t->ry, t->rz, t->is_stretched ? 1.0f : 0.0f,
                         (float)count};
    memcpy(consts, c, sizeof(c));
    if (uvwt) memcpy(uvwt, t->uvwt, (size_t)t->nn * sizeof(LESFloat4));
    if (cpxx) memcpy(cpxx, t->cpxx, (size_t)t->nn * sizeof(LESFloat4));
    LES_free(h);
    return 0;
}

/* The first `count` beam positions of a scan string: POS_init_with_string
 * then POS_get_next_angles (pos.c:34-56) `count` times. */
int ref_pos_angles(const char *scan, int count, float *az, float *el) {
    POSPattern *p = POS_init_with_string(scan);
    if (p == NULL) return -1;
    for (int k = 0; k < count; k++) {
        POS_get_next_angles(p);
        az[k] = p->az;
        el[k] = p->el;
    }
    POS_free(p);
    return 0;
}

/* ADM_get_table (adm.c:152-225) of <path>/adm/<name>.adm: dims = nb, na;
 * data = cdx, cdy, cdz, cmx, cmy, cmz (nn floats each; NULL to query);
 * phys = x, y, z, rho, mass, Ta, inv_inln_x, inv_inln_y, inv_inln_z. */
int ref_adm_table(const char *path, const char *name, uint32_t dims[2], float *data, float phys[9]) {
    ADMHandle h = ADM_init_with_path(path);
    if (h == NULL) return -1;
    ADMTable *t = ADM_get_table(h, (const ADMConfig)name);
    if (t == NULL) {
        ADM_free(h);
        return -2;
    }
    dims[0] = t->nb;
    dims[1] = t->na;
    if (data) {
        const float *c[6] = {t->data.cdx, t->data.cdy, t->data.cdz, t->data.cmx, t->data.cmy, t->data.cmz};
        for (int i = 0; i < 6; i++) memcpy(data + (size_t)i * t->nn, c[i], (size_t)t->nn * sizeof(float));
    }
    const float p[9] = {t->phys.x, t->phys.y, t->phys.z, t->phys.rho, t->phys.mass, t->phys.Ta,
                        t->phys.inv_inln_x, t->phys.inv_inln_y, t->phys.inv_inln_z};
    memcpy(phys, p, sizeof(p));
    ADM_free(h);
    return 0;
}

/* RCS_get_table (rcs.c:181-246) of <path>/rcs/<name>.rcs: dims = na, nb;
 * data = hh, vv, hv real, then hh, vv, hv imaginary (nn floats each). */
int ref_rcs_table(const char *path, const char *name, uint32_t dims[2], float *data) {
    RCSHandle h = RCS_init_with_path(path);
    if (h == NULL) return -1;
    RCSTable *t = RCS_get_table(h, (const RCSConfig)name);
    if (t == NULL) {
        RCS_free(h);
        return -2;
    }
    dims[0] = t->na;
    dims[1] = t->nb;
    if (data) {
        const float *c[6] = {t->data.hh_real, t->data.vv_real, t->data.hv_real,
                             t->data.hh_imag, t->data.vv_imag, t->data.hv_imag};
        for (int i = 0; i < 6; i++) memcpy(data + (size_t)i * t->nn, c[i], (size_t)t->nn * sizeof(float));
    }
    RCS_free(h);
    return 0;
}

/* OBJ_get_table (obj.c:102-148) for a debris type, with the tables found the
 * way rs.c finds them (OBJ_init: the current folder, then ~/Documents/tables
 * and the other folders of adm.c / rcs.c): the ADM table's physical
 * constants after ADM_dimension_set (as ref_adm_table's phys) and the names
 * of the two tables. */
int ref_obj_table(int type, float phys[9], char *adm_name, char *rcs_name, size_t name_size) {
    OBJHandle h = OBJ_init();
    if (h == NULL) return -1;
    OBJTable *t = OBJ_get_table(h, type);
    if (t == NULL || t->adm_table == NULL || t->rcs_table == NULL) {
        OBJ_free(h);
        return -2;
    }
    const ADMBase *b = &t->adm_table->phys;
    const float p[9] = {b->x, b->y, b->z, b->rho, b->mass, b->Ta, b->inv_inln_x, b->inv_inln_y, b->inv_inln_z};
    memcpy(phys, p, sizeof(p));
    snprintf(adm_name, name_size, "%s", t->adm_table->name);
    snprintf(rcs_name, name_size, "%s", t->rcs_table->name);
    OBJ_free(h);
    return 0;
}

/* The LES descriptor rs.c derives for a configuration: RS_init_with_path on
 * the CPU oracle device (bundle = the folder of rs_enum.h and rs.cl), then
 * RS_set_vel_data_to_config, which finds the tables from $HOME as rs.c
 * always does and runs RS_set_vel_data_to_LES_table (rs.c:3029-3126) and
 * RS_set_vel_data (rs.c:2854-2978) on frame 0. */
#include "rs.h"
int ref_les_descriptor(const char *bundle, const char *config, float desc[16]) {
    RSHandle *H = RS_init_with_path(bundle, RS_METHOD_GPU, 0xFF, 0, 0);
    if (H == NULL) return -1;
    RS_set_vel_data_to_config(H, (LESConfig)config);
    if (H->L == NULL) {
        RS_free(H);
        return -2;
    }
    memcpy(desc, H->workers[0].les_desc.s, 16 * sizeof(float));
    RS_free(H);
    return 0;
}
