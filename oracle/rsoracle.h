/*
 * rsoracle.h -- CPU oracle for the SimRadar per-pulse emulation loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * OpenCL kernels in rs.cl and of the host arithmetic in rs.c that feeds them.
 * It is used by the tests, by __graft_entry__.smoke() and by the CPU-baseline
 * leg of bench.py as the checker and as the timed CPU baseline.  Nothing in the
 * simradar_gb300 package links, loads or calls it.
 *
 * Every function names the reference lines it follows.  Vector expressions of
 * OpenCL C are written out lane by lane in the same left-to-right order, and
 * the file is compiled with -ffp-contract=off, so each single-precision
 * operation is the one the kernel source spells.  The transcendental functions
 * come from simradar_gb300/csrc/rsmath.h (shared with the CUDA kernels, tested
 * on its own against float64 references).  OpenCL's read_imagef with
 * CLK_NORMALIZED_COORDS_FALSE | CLK_ADDRESS_CLAMP_TO_EDGE | CLK_FILTER_LINEAR
 * (rs.cl:8) is emulated with the OpenCL 1.2 formula in full single precision.
 */
#ifndef SIMRADAR_ORACLE_H
#define SIMRADAR_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float x, y, z, w; } of4;
typedef struct { uint32_t x, y, z, w; } ou4;

/* An image (OpenCL image2d_t / image3d_t of CL_RGBA CL_FLOAT), x fastest. */
typedef struct {
    const of4 *data;
    int nx, ny, nz;
} or_image;

/* concept bits (rs_enum.h:127-137) */
enum {
    OR_CONCEPT_CROSS_POL = 1,
    OR_CONCEPT_DRAGGED = 1 << 1,
    OR_CONCEPT_TRANSPARENT = 1 << 2,
    OR_CONCEPT_BOUNDED = 1 << 3,
    OR_CONCEPT_UNIFORM_DSD = 1 << 4,
    OR_CONCEPT_FIXED_POS = 1 << 5,
    OR_CONCEPT_VERTICAL = 1 << 6,
    OR_CONCEPT_DFF = 1 << 7
};

/* kernels: each processes indices [origin, origin + count), like
 * clEnqueueNDRangeKernel with a global work offset (rs.c:5342-5369) */
void or_el_atts(of4 *p, of4 *v, of4 *x, ou4 *y, or_image uvwt, const float *wind_desc,
                const of4 *drop_rcs, const float *drop_rcs_desc, const float *sim_desc,
                size_t origin, size_t count);
void or_bg_atts(of4 *p, of4 *v, of4 *x, ou4 *y, or_image uvwt, const float *wind_desc,
                const of4 *drop_rcs, const float *drop_rcs_desc, const float *sim_desc,
                size_t origin, size_t count);
void or_fp_atts(of4 *p, of4 *v, of4 *x, or_image uvwt, or_image cpxx, const float *wind_desc,
                const float *sim_desc, size_t origin, size_t count);
void or_db_atts(of4 *p, of4 *o, of4 *v, of4 *t, of4 *x, ou4 *y, or_image uvwt, const float *wind_desc,
                or_image adm_cd, or_image adm_cm, const float *adm_desc,
                or_image rcs_real, or_image rcs_imag, const float *rcs_desc,
                const float *dff_icdf, const float *dff_desc, const float *sim_desc,
                size_t origin, size_t count);
void or_db_rcs(const of4 *p, const of4 *o, of4 *x, or_image rcs_real, or_image rcs_imag,
               const float *rcs_desc, const float *sim_desc, size_t origin, size_t count);
void or_scat_sig_aux(of4 *s, of4 *a, const of4 *p, const of4 *x, const float *angular_weight,
                     const float *angular_weight_desc, const float *sim_desc, size_t count);
void or_pop(of4 *rcs, of4 *aux, of4 *pos, const float *sim_desc, size_t count);

/* RS_make_pulse_params (rs.c:1284-1386) */
typedef struct {
    uint32_t num_scats, user_max_groups, user_max_work_items, pass_2_method;
    uint32_t range_count;
    float range_start, range_delta;
    uint32_t entry_counts[2], group_counts[2];
    size_t global[2], local[2], local_mem_size[2];
} or_pulse_params;
enum { OR_PASS_2_UNIVERSAL = 0, OR_PASS_2_IN_RANGE = 1, OR_PASS_2_IN_LOCAL = 2 };
int or_make_pulse_params(or_pulse_params *out, uint32_t count, uint32_t group_size_multiple,
                         uint32_t user_max_groups, uint32_t max_local_mem_size,
                         float range_start, float range_delta, uint32_t range_count);

/* make_pulse_pass_1 (rs.cl:1125-1301); work = group_count x range_count float4.
 * sig/aux hold n_alloc entries; reads past n_alloc count as zero. */
void or_make_pulse_pass_1(of4 *work, const of4 *sig, const of4 *aux, size_t n_alloc,
                          const float *range_weight, const float *range_weight_desc,
                          float range_start, float range_delta, uint32_t range_count,
                          uint32_t group_count, uint32_t n, uint32_t local_size);
/* the three pass-2 bodies (rs.cl:1304-1441), run with the launch geometry of
 * the selected method; the kernel-name swap of rs.c:506-507 is applied by
 * or_make_pulse(). */
void or_make_pulse_pass_2_local_body(of4 *out, const of4 *in, size_t in_alloc, uint32_t range_count,
                                     uint32_t n, size_t global, size_t local);
void or_make_pulse_pass_2_range_body(of4 *out, const of4 *in, size_t in_alloc, uint32_t range_count,
                                     uint32_t n, size_t global);
void or_make_pulse_pass_2_group_body(of4 *out, const of4 *in, size_t in_alloc, uint32_t range_count,
                                     size_t local);
/* scat_sig_aux + pass 1 + pass 2 exactly as RS_make_pulse enqueues them
 * (rs.c:5563-5573), with the pass plan of or_make_pulse_params. */
int or_make_pulse(of4 *pulse, of4 *sig, of4 *aux, const of4 *pos, const of4 *rcs, size_t num_scats,
                  size_t n_alloc, const float *angular_weight, const float *angular_weight_desc,
                  const float *range_weight, const float *range_weight_desc,
                  float range_start, float range_delta, uint32_t range_count,
                  const float *sim_desc, uint32_t group_size_multiple, uint32_t max_work_group_size,
                  uint32_t local_mem_size, int name_swap);

/* The FP32 per-scatterer, per-gate contributions exactly as scat_sig_aux and
 * pass 1 form them (the values the reference adds), summed in double over
 * every gate: the pulse with the summation-order error removed. */
void or_make_pulse_direct(double *pulse4, double *abs_sum4, const of4 *pos, const of4 *rcs, size_t num_scats,
                          const float *angular_weight, const float *angular_weight_desc,
                          const float *range_weight, const float *range_weight_desc,
                          float range_start, float range_delta, uint32_t range_count, const float *sim_desc);

/* FP64 pulse of the same FP32 state: the reference of the error metric.
 * Ranges, angles, phases, weights and sums are all evaluated in double; the
 * gate origins are range_start + k * range_delta in double.  Also returns
 * (if abs_sum != NULL) the per-gate sum of |contribution| per lane. */
void or_make_pulse_f64(double *pulse4, double *abs_sum4, const of4 *pos, const of4 *rcs, size_t num_scats,
                       const float *angular_weight, const float *angular_weight_desc,
                       const float *range_weight, const float *range_weight_desc,
                       double range_start, double range_delta, uint32_t range_count,
                       const float *sim_desc);

/* diagnostics: evaluate the shared elementary functions on a vector */
void or_eval_math(int fn, const float *a, const float *b, float *out, size_t n);

int or_num_threads(void);

#ifdef __cplusplus
}
#endif

#endif
