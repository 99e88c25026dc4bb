/*
 * rscl.h -- the reference's own rs.cl kernels, compiled for the CPU through
 * oracle/ref/clc/opencl_c.hpp into oracle/_ref/ (test infrastructure).
 *
 * Each entry point runs one launch of the kernel of the same name in rs.cl
 * over the global range [origin, origin + count) and takes the arguments of
 * the oracle's restatement (oracle/rsoracle.h) in the same order, so that a
 * caller can run either on the same arrays and compare.  Arguments rs.cl
 * declares but the kernel never reads (the cpxx image of el_atts / bg_atts,
 * the seed and drop table of fp_atts) are supplied here.  Work-group kernels
 * (make_pulse_pass_1 and the three pass-2 kernels) run their work items as
 * user-level contexts that meet at every barrier; their inputs are copied
 * into zero-padded scratch so that reads past the caller's arrays (pass 1
 * reads sig[i + local_size] for i < n) see zeros, as the oracle's do.
 */
#ifndef SIMRADAR_RSCL_H
#define SIMRADAR_RSCL_H

#include <stddef.h>
#include <stdint.h>

#include "rsoracle.h"

#ifdef __cplusplus
extern "C" {
#endif

void rscl_el_atts(of4 *p, of4 *v, of4 *x, ou4 *y, or_image uvwt, const float *wind_desc, const of4 *drop_rcs,
                  const float *drop_rcs_desc, const float *sim_desc, size_t origin, size_t count);
void rscl_bg_atts(of4 *p, of4 *v, of4 *x, ou4 *y, or_image uvwt, const float *wind_desc, const of4 *drop_rcs,
                  const float *drop_rcs_desc, const float *sim_desc, size_t origin, size_t count);
void rscl_fp_atts(of4 *p, of4 *v, of4 *x, or_image uvwt, or_image cpxx, const float *wind_desc,
                  const float *sim_desc, size_t origin, size_t count);
void rscl_db_atts(of4 *p, of4 *o, of4 *v, of4 *t, of4 *x, ou4 *y, or_image uvwt, const float *wind_desc,
                  or_image adm_cd, or_image adm_cm, const float *adm_desc, or_image rcs_real, or_image rcs_imag,
                  const float *rcs_desc, const float *dff_icdf, const float *dff_desc, const float *sim_desc,
                  size_t origin, size_t count);
void rscl_db_rcs(const of4 *p, const of4 *o, of4 *x, or_image rcs_real, or_image rcs_imag, const float *rcs_desc,
                 const float *sim_desc, size_t origin, size_t count);
void rscl_scat_sig_aux(of4 *s, of4 *a, const of4 *p, const of4 *x, const float *angular_weight,
                       const float *angular_weight_desc, const float *sim_desc, size_t count);
void rscl_pop(of4 *rcs, of4 *aux, of4 *pos, const float *sim_desc, size_t count);
void rscl_make_pulse_pass_1(of4 *work, const of4 *sig, const of4 *aux, size_t n_alloc, const float *range_weight,
                            const float *range_weight_desc, float range_start, float range_delta,
                            uint32_t range_count, uint32_t group_count, uint32_t n, uint32_t local_size);
/* pass 2 (rs.cl:1304-1441) with the launch geometry global / local (local 0:
 * one item per group); out holds global entries, in holds in_alloc */
void rscl_make_pulse_pass_2_local(of4 *out, const of4 *in, size_t in_alloc, uint32_t range_count, uint32_t n,
                                  size_t global, size_t local);
void rscl_make_pulse_pass_2_range(of4 *out, const of4 *in, size_t in_alloc, uint32_t range_count, uint32_t n,
                                  size_t global, size_t local);
void rscl_make_pulse_pass_2_group(of4 *out, const of4 *in, size_t in_alloc, uint32_t range_count, uint32_t n,
                                  size_t global, size_t local);
/* scat_sig_aux + pass 1 + pass 2 of rs.cl with the plan of
 * or_make_pulse_params, as or_make_pulse strings the oracle's together */
int rscl_make_pulse(of4 *pulse, of4 *sig, of4 *aux, const of4 *pos, const of4 *rcs, size_t num_scats,
                    size_t n_alloc, const float *angular_weight, const float *angular_weight_desc,
                    const float *range_weight, const float *range_weight_desc, float range_start,
                    float range_delta, uint32_t range_count, const float *sim_desc, uint32_t group_size_multiple,
                    uint32_t max_work_group_size, uint32_t local_mem_size, int name_swap);

#ifdef __cplusplus
}
#endif

#endif
