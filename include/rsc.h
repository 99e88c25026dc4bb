/*
 * rsc.h -- GB300 (sm_103a) backend for SimRadar's per-pulse emulation loop.
 *
 * This is the C ABI that the RS framework host (rs.c) calls in place of its
 * OpenCL calls.  One rsc_worker owns the device state of one RSWorker
 * (rs.h:150-266): the scatterer attribute arrays, the lookup tables and the
 * pulse.  Every entry point names the rs.c code it replaces.  Plain pointers
 * and sizes only; every function returns RSC_OK (0) or a negative status and
 * never exits the process.  rsc_last_error() returns the message of the last
 * failure on the calling thread.
 *
 * Data layout (identical to the reference host arrays, rs.h:304-313):
 *   attribute arrays are float4 / uint4 per scatterer (16 B, x fastest):
 *     pos (x, y, z, radius)  vel (u, v, w, -)  ori, tum (quaternion x, y, z, w)
 *     aux (range, age, dsd bin, angular weight)  rcs, sig (Ih, Qh, Iv, Qv)
 *     rnd (4 x 32-bit seeds)
 *   images are float4 arrays, x fastest (CL_RGBA / CL_FLOAT, rs.c:2857).
 *   descriptors are the float[16] / float[4] vectors the kernels receive
 *   (sim_desc: rs_enum.h:93-110, table descriptors: rs_enum.h:10-91).
 */
#ifndef SIMRADAR_GB300_RSC_H
#define SIMRADAR_GB300_RSC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RSC_OK 0
#define RSC_ERR_ARG (-1)        /* invalid argument (NULL, size, index) */
#define RSC_ERR_CUDA (-2)       /* a CUDA runtime call failed */
#define RSC_ERR_NOMEM (-3)      /* device or pinned host allocation failed */
#define RSC_ERR_STATE (-4)      /* call out of order (e.g. before rsc_worker_malloc) */
#define RSC_ERR_UNSUPPORTED (-5) /* a table or mode the kernels do not handle */

#define RSC_MAX_TYPES 8         /* RS_MAX_DEBRIS_TYPES, rs_const.h:24 */
#define RSC_MAX_GATES 512       /* RS_MAX_GATES, rs_const.h:22 */

/* pulse-formation precision (additive; the reference has only RSC_PULSE_PLAIN) */
#define RSC_PULSE_PLAIN 0       /* FP32 exactly as rs.cl scat_sig_aux + pass 1 (gate weights bit-exact) */
#define RSC_PULSE_COMPENSATED 1 /* double-float terms (split range phase), FP64 gate origins, error-free sums */
#define RSC_PULSE_F64 2         /* FP64 reference of the same FP32 state (error metric oracle) */

typedef struct rsc_worker rsc_worker;

/* Population layout of one worker: type 0 is the background (rain), types
 * 1..RSC_MAX_TYPES-1 are debris; counts[k] scatterers start at origins[k]
 * (RSWorker.origins / .counts, rs.h:160-161, set by RS_update_origins_offsets
 * rs.c:2259-2359).  Debris type k uses ADM table adm_index[k] and RCS table
 * rcs_index[k] (the round-robin a / r indices of rs.c:5351-5373). */
typedef struct {
    uint64_t origins[RSC_MAX_TYPES];
    uint64_t counts[RSC_MAX_TYPES];
    int32_t adm_index[RSC_MAX_TYPES];
    int32_t rcs_index[RSC_MAX_TYPES];
} rsc_population;

/* Last error message of this thread (never NULL). */
const char *rsc_last_error(void);

/* Number of visible CUDA devices (replaces get_device_info, rs.c:95-223). */
int rsc_device_count(int *count);

/* Create a worker on a device: stream, events and the kernels' launch
 * configuration.  Replaces RS_worker_init's context / queue / program /
 * kernel creation (rs.c:383-545). */
int rsc_worker_create(int device, rsc_worker **out);

/* Release every device allocation of the worker.  Replaces RS_worker_free
 * (rs.c:547-621) and the device half of RS_free_scat_memory (rs.c:1182-1246). */
int rsc_worker_free(rsc_worker *w);

/* Allocate the attribute arrays for num_scats scatterers (padded to a multiple
 * of 64, the padding zeroed) and the pulse for range_count gates starting at
 * range_start every range_delta.  aux, rcs and sig start at zero.  Replaces
 * RS_worker_malloc (rs.c:623-944): its clCreateBuffer calls, the zero fill of
 * aux / rcs / sig and the pass-1 gate arguments (rs.c:872-884). */
int rsc_worker_malloc(rsc_worker *w, size_t num_scats, float range_start, float range_delta,
                      uint32_t range_count);

/* Range weight table W[n] with descriptor (scale, origin, max, user) --
 * RS_set_range_weight, rs.c:2548-2618. */
int rsc_set_range_weight(rsc_worker *w, const float *table, uint32_t n, const float desc[4]);

/* Angular weight table -- RS_set_angular_weight, rs.c:2626-2699. */
int rsc_set_angular_weight(rsc_worker *w, const float *table, uint32_t n, const float desc[4]);

/* Ellipsoid (drop) RCS table of n float4 -- RS_set_rcs_ellipsoid_table,
 * rs.c:2472-2546. */
int rsc_set_rcs_ellipsoid(rsc_worker *w, const float *table4, uint32_t n, const float desc[4]);

/* Upload one LES volume (uvwt and cpxx, nx*ny*nz float4 each) into buffer
 * slot 0 or 1 of the double buffer, and set the LES descriptor.  Replaces the
 * clCreateImage / clEnqueueWriteImage / descriptor code of RS_set_vel_data
 * (rs.c:2854-2978).  Synchronous, like the reference (clWaitForEvents,
 * rs.c:2940).  The dimensions must not change between slots. */
int rsc_set_les(rsc_worker *w, int slot, const float *uvwt4, const float *cpxx4, uint32_t nx,
                uint32_t ny, uint32_t nz, const float desc[16]);

/* Same upload, asynchronous: the copy is ordered before the next advance on
 * the worker's stream, so the caller may refill `slot` while the current one
 * is in use.  The host buffers must stay valid until rsc_synchronize(). */
int rsc_set_les_async(rsc_worker *w, int slot, const float *uvwt4, const float *cpxx4, uint32_t nx,
                      uint32_t ny, uint32_t nz, const float desc[16]);

/* ADM table `index` (drag cd and moment cm images, nx = beta, ny = alpha) --
 * RS_set_adm_data, rs.c:3642-3763.  index < RSC_MAX_TYPES. */
int rsc_set_adm(rsc_worker *w, int index, const float *cd4, const float *cm4, uint32_t nx, uint32_t ny,
                const float desc[16]);

/* RCS table `index` (real and imaginary images, nx = alpha, ny = beta) --
 * RS_set_rcs_data, rs.c:3852-3973. */
int rsc_set_rcs(rsc_worker *w, int index, const float *real4, const float *imag4, uint32_t nx, uint32_t ny,
                const float desc[16]);

/* Debris-flux-field inverse CDF of n floats into slot 0 or 1, and its
 * descriptor -- RS_set_debris_flux_field_by_icdf, rs.c:3328-3408. */
int rsc_set_dff(rsc_worker *w, int slot, const float *icdf, uint32_t n, const float desc[16]);

/* Host -> device copy of scatterers [offset, offset + count) of each array
 * given (NULL skips an array) -- RS_upload, rs.c:5124-5176. */
int rsc_upload(rsc_worker *w, size_t offset, size_t count, const float *pos4, const float *vel4,
               const float *ori4, const float *tum4, const float *aux4, const float *rcs4, const float *sig4,
               const uint32_t *rnd4);

/* Device -> host copy, same convention -- RS_download (rs.c:4961-5016),
 * RS_download_position_only (rs.c:5018-5040), RS_download_orientation_only
 * (rs.c:5042-5064).  aux and sig are those of the latest pulse, as rs.c's
 * last scat_sig_aux launch leaves them: when the pulse kernel did not write
 * them, they are formed from the state that pulse read (before a second
 * advance, a sort or an upload replaces it, or here). */
int rsc_download(rsc_worker *w, size_t offset, size_t count, float *pos4, float *vel4, float *ori4,
                 float *tum4, float *aux4, float *rcs4, float *sig4, uint32_t *rnd4);

/* One time step of every scatterer: the el_atts / bg_atts / fp_atts launch on
 * type 0 (chosen by the concept bits in sim_desc[5], rs.c:5339-5349) and the
 * db_atts launch for each debris type (rs.c:5350-5374), as two kernels: the
 * background range, and every debris range together beside it on a
 * high-priority stream, reading LES slot les_id.  Replaces the launches and the wait of
 * RS_advance_time (rs.c:5325-5388).  Asynchronous unless the caller
 * synchronises; rsc_download / rsc_download_pulse synchronise. */
int rsc_advance_time(rsc_worker *w, const rsc_population *pop, int les_id, const float sim_desc[16]);

/* Debris RCS refresh after a beam move: db_rcs for every debris type
 * (rs.c:5528-5562). */
int rsc_update_debris_rcs(rsc_worker *w, const rsc_population *pop, const float sim_desc[16]);

/* Form the pulse of the current state for the beam in sim_desc[0..2]:
 * scat_sig_aux + make_pulse_pass_1 + make_pulse_pass_2 (rs.c:5563-5573) as
 * one kernel.  The per-gate float4 (Ih, Qh, Iv, Qv) sums stay on the device. */
int rsc_make_pulse(rsc_worker *w, const float sim_desc[16]);

/* Copy the pulse to host memory (range_count float4) and multiply by `gain`
 * -- RS_download_pulse_only + RS_merge_pulse_tmp for one worker
 * (rs.c:5096-5122, rs.c:5066-5094).  Waits for the pulse. */
int rsc_download_pulse(rsc_worker *w, float *pulse4, float gain);

/* Wait for all work queued on the worker (clFinish). */
int rsc_synchronize(rsc_worker *w);

/* The latest pulse copied to pulse4 (range_count float4, no gain) without
 * waiting: the copy runs on a stream of its own once the pulse is formed, so
 * the next advance does not wait for it (the next pulse does), and it is
 * complete after rsc_synchronize.  With page-locked pulse4 the host can queue
 * the next pulses while earlier copies are in flight (additive; the
 * reference reads each pulse with a blocking clEnqueueReadBuffer, rs.c:5115). */
int rsc_download_pulse_async(rsc_worker *w, float *pulse4);

/* Pulse-formation precision, RSC_PULSE_* (additive, default PLAIN). */
int rsc_set_pulse_precision(rsc_worker *w, int mode);

/* Write aux and sig on every pulse (as the reference does) instead of forming
 * them on download.  Default 0. */
int rsc_set_materialize_sig_aux(rsc_worker *w, int enable);

/* The compensated form's gate sums on the triangle range weight (additive,
 * default 1): 1 sums each scatterer's term into its one range interval as
 * two moments (the triangle is linear within an interval) and forms the
 * gates from them; 0 weighs every term into every gate it reaches.  Both
 * are error-free double-float sums; the pulses agree to the double-float's
 * precision.  Read by rsc_make_pulse and by a batch's runs. */
int rsc_set_pulse_moments(rsc_worker *w, int enable);

/* Number of kernel launches this worker has issued (for accounting). */
int rsc_launch_count(rsc_worker *w, uint64_t *count);

/* The CUDA stream the worker issues pulses and every other call on (as a
 * void pointer, for callers that time with events on it).  Each call that
 * reads the state first makes it wait for the advance stream. */
int rsc_get_stream(rsc_worker *w, void **stream);
/* The stream rsc_advance_time issues on, beside the pulse of the same step
 * (the fused step form issues on the worker's stream instead).  Work queued
 * on the worker's stream after a wait for this one sees every advance. */
int rsc_get_advance_stream(rsc_worker *w, void **stream);

/* ---- spatial order (additive) ----
 * The worker keeps its background scatterers (type 0) in Morton order of
 * their cell in the scan box, restored by a counting sort after every
 * `steps` calls of rsc_advance_time (and after an upload of positions); 0
 * keeps the caller's order.  The order is invisible at the ABI: upload and
 * download map the caller's indices, and no result depends on it beyond the
 * rounding of the gate sums.  Default 128. */
int rsc_set_sort_interval(rsc_worker *w, int steps);
/* Number of sorts the worker has made. */
int rsc_sort_count(rsc_worker *w, uint64_t *count);

/* ---- fused step (additive) ----
 * With the fused step on, rsc_advance_time records the advance
 * and the next rsc_make_pulse runs both in one kernel, one pass over the
 * state (the pulse reads exactly what the advance writes).  Any other call
 * that reads or changes the state or the tables (download, upload, table
 * setters, debris RCS, synchronize, a second advance, the batch) first runs
 * the recorded advance on its own, so every result is the one of the
 * separate calls; launch errors of a recorded advance are reported by the
 * call that runs it.  The FP64 precision mode never fuses.  Off by default:
 * both halves are bound by instruction issue, not by the state's bytes, and
 * on a GB300 the separate kernels (each at its own occupancy) are about 3%
 * faster per step than the fused one (2 M scatterers, 40 gates). */
int rsc_set_fused_step(rsc_worker *w, int enable);

/* ---- launch-shape autotuning (additive) ----
 * Time the pulse kernel of this worker at each candidate shape (warps per
 * block 4 / 8 / 16 and 1-4 resident blocks per SM) on the current state and
 * keep the fastest for later rsc_make_pulse calls.  sim_desc is the beam to
 * time with; the state is not changed (the pulse is recomputed). */
int rsc_autotune(rsc_worker *w, const float sim_desc[16], int *warps_out, int *blocks_per_sm_out);
/* Set the pulse kernel's shape directly: warps per block (1-16) and resident
 * blocks per SM (1-4), each capped by what the kernel's shared memory and
 * registers allow; 0 for either returns to the largest that fits.  Fewer
 * pulse blocks per SM leave room for the advance of the same step, which
 * runs beside the pulse on the advance stream. */
int rsc_set_pulse_shape(rsc_worker *w, int warps, int blocks_per_sm);
/* Background scatterers per thread of the advance (1 or 2; el_atts and
 * bg_atts): with 2 a thread forms two scatterers' steps before storing
 * either, overlapping their dependent loads.  The state is the same. */
int rsc_set_advance_shape(rsc_worker *w, int scatterers_per_thread);

/* ---- batching form (additive; no counterpart in rs.c) ----
 * A batch runs many emulation instances -- each an rsc_worker with its own
 * state, tables, gates, concept and population, all on one device -- one
 * time step at a time, with three launches per step for all of them (the
 * pulse, and beside it on a second stream the background advance and, on a
 * high-priority stream, the debris advance: the order of simradar's loop,
 * simradar.c:1032-1070, with the advance writing each instance's second
 * pos / rcs pair while the pulse reads the first).  Each instance evolves
 * exactly as it would alone. */
typedef struct rsc_batch rsc_batch;

/* The workers must be allocated and have their tables set.  The batch keeps
 * the pointers; free it before the workers. */
int rsc_batch_create(rsc_worker *const *workers, int count, rsc_batch **out);
int rsc_batch_free(rsc_batch *b);

/* Population layout of every instance (count entries). */
int rsc_batch_set_populations(rsc_batch *b, const rsc_population *pops);

/* RSC_PULSE_PLAIN / COMPENSATED / F64 for every instance. */
int rsc_batch_set_precision(rsc_batch *b, int mode);

/* Choose the batched pulse kernel's shape (warps per block 4 / 8 / 16 and
 * 1-4 resident blocks per SM) by timing it on the current state with the
 * given per-instance sim_descs (count x 16 floats, LES slot 0), then the
 * background advance's shape (threads per block 64 / 128 / 256, with every
 * block that fits resident or half of them) by timing it beside that pulse
 * on scratch copies of the arrays it updates in place.  The state is not
 * changed. */
int rsc_batch_autotune(rsc_batch *b, const float *sim_descs);
/* Set the batched background advance's shape directly: threads per block
 * (64, 128 or 256) and resident blocks per SM (0: as many as fit). */
int rsc_batch_set_advance_shape(rsc_batch *b, int threads, int blocks_per_sm);
/* The batched background advance's shape (128, 0 until set or tuned). */
int rsc_batch_get_advance_shape(rsc_batch *b, int *threads, int *blocks_per_sm);

/* Run `steps` time steps of every instance: for step k and instance i the
 * pulse for sim_descs[(k * count + i) * 16 ...] is formed, then the instance
 * advances with LES slot les_ids[k * count + i].  The pulses (range_count
 * float4 per instance, no gain applied) are copied to pulses_out as
 * [k][i][max_gates] float4 if it is not NULL.  With use_graph the 2 * steps
 * launches are captured once in a CUDA graph (per step count) and replayed.
 * Returns after the pulses are on the host (or the work is queued when
 * pulses_out is NULL; rsc_batch_synchronize waits). */
int rsc_batch_run(rsc_batch *b, int steps, const float *sim_descs, const int *les_ids, float *pulses_out,
                  int use_graph);
/* As rsc_batch_run, but returns once the work and the copy of the pulses are
 * queued: pulses_out must stay valid until rsc_batch_synchronize (page-locked
 * memory keeps the copy asynchronous; the I/Q streaming of long runs issues
 * one such call per block of pulses into a ring of pinned buffers).  The
 * descriptors are taken before the call returns. */
int rsc_batch_run_async(rsc_batch *b, int steps, const float *sim_descs, const int *les_ids, float *pulses_out,
                        int use_graph);
int rsc_batch_synchronize(rsc_batch *b);

/* Refill LES slot `slot` of instance `index` (a slot already set with
 * rsc_set_les, same dimensions and descriptor) on the batch's copy stream:
 * the copy starts once the runs that read the slot are done and overlaps the
 * runs queued meanwhile on the other slot; the first later run that reads
 * the slot waits for it.  The host buffers (page-locked for the copy to be
 * asynchronous) must stay valid until rsc_batch_synchronize.  Replaces the
 * blocking frame swap of RS_set_vel_data inside RS_advance_time
 * (rs.c:2854-2978, rs.c:5188-5200) for batched runs. */
int rsc_batch_set_les_async(rsc_batch *b, int index, int slot, const float *uvwt4, const float *cpxx4, uint32_t nx,
                            uint32_t ny, uint32_t nz);
/* The persistent form (additive, off by default): rsc_batch_run and
 * rsc_batch_run_async then run all steps of every instance in one launch.
 * Each block owns fixed segments of the instances' scatterers (cut on the
 * host to equal cost) and, step after step, forms their share of the pulse
 * and advances them; no block waits for another (the pulses of different
 * steps use separate accumulators, the last block of an instance's pulse
 * converting it).  The state and the pulses are the ones of the three-launch
 * form.  The FP64 precision mode always runs the three-launch form; use_graph
 * is ignored while this is on. */
int rsc_batch_set_persistent(rsc_batch *b, int enable);
/* The largest gate count of the batch (the row length of pulses_out). */
int rsc_batch_max_gates(rsc_batch *b, int *max_gates);
/* Kernel launches the batch has issued (per step the pulse, plus the
 * background and the debris advance where the batch has such scatterers,
 * plus the autotuner's). */
int rsc_batch_launch_count(rsc_batch *b, uint64_t *count);
/* The CUDA stream the batch issues on.  A run's advances run on streams of
 * its own, forked from this one at the run's start and joined back into it
 * before the run's end, so work queued here after a run sees all of it. */
int rsc_batch_get_stream(rsc_batch *b, void **stream);
/* The pulse shape chosen by rsc_batch_autotune (0, 0 before it runs). */
int rsc_batch_get_shape(rsc_batch *b, int *warps, int *blocks_per_sm);

/* ---- initial state (additive) ----
 * The scatterers RS_populate (rs.c:4568-4814) makes from RS_set_random_seed:
 * the same draws of the C library's rand() in the same order (glibc's
 * generator, reproduced, so the result does not depend on the host's libc),
 * for one worker whose type ranges follow one another from slot 0, outside
 * the fixed-position concept (whose anchor planes rs.c keeps making).  The
 * "(float)rand() / RAND_MAX * size + origin" products are rounded before the
 * sum (no fused multiply-add).  The ellipsoid table, the debris RCS refresh
 * and the warm-up advance of RS_populate stay in rs.c. */
typedef struct {
    uint32_t seed;                       /* H->random_seed */
    uint32_t sim_concept;                /* H->sim_concept bits */
    float domain_origin[3], domain_size[3];   /* RS_get_domain */
    uint32_t num_types;                  /* H->num_types (1 + debris types) */
    uint64_t origins[RSC_MAX_TYPES], counts[RSC_MAX_TYPES];
    const float *dsd_r, *dsd_cdf;        /* H->dsd_r / H->dsd_cdf, NULL when no DSD is set */
    uint32_t dsd_count;                  /* H->dsd_count, 0 when no DSD is set */
} rsc_populate_args;

/* The first `count` values of rand() after srand(seed). */
int rsc_rand_sequence(uint32_t seed, uint32_t count, int32_t *out);
/* The whole initial state into host arrays of num_scats float4 / uint4
 * (NULL skips vel, ori, tum, rcs); dsd_pop (dsd_count entries, may be NULL)
 * counts the drops per bin as H->dsd_pop does. */
int rsc_populate_host(const rsc_populate_args *a, size_t num_scats, float *pos4, float *vel4, float *ori4,
                      float *tum4, float *aux4, float *rcs4, uint32_t *rnd4, uint32_t *dsd_pop);
/* The same state made straight into an allocated worker: generated on the
 * host in blocks that go to the device by page-locked asynchronous copies
 * while the next block is generated (RS_populate + RS_upload without the
 * full host arrays). */
int rsc_populate_upload(rsc_worker *w, const rsc_populate_args *a, uint32_t *dsd_pop);
const char *rsc_populate_last_error(void);

/* ---- I/Q output file (additive) ----
 * The .iq file of simradar (simradar.c:340-366, headers iq.h:20-41, reader
 * matlab/simradariq.m), byte for byte: a 1024-byte file header, then per
 * pulse a 32-byte header (time, elevation, azimuth) and range_count float4
 * (Ih, Qh, Iv, Qv).  Writes go to a background thread, so a pulse loop that
 * streams I/Q blocks (rsc_batch_run_async into pinned buffers) is not held
 * by the file system.  The reference keeps every pulse in host memory and
 * writes the file at the end of the run. */
typedef struct {
    /* RSParams, rs_types.h:56-93 */
    float c, prt, loss, lambda, tx_power_watt, antenna_gain_dbi, antenna_bw_deg, tau;
    float range_start, range_end, range_delta;
    float azimuth_start_deg, azimuth_end_deg, azimuth_delta_deg;
    float elevation_start_deg, elevation_end_deg, elevation_delta_deg;
    float domain_pad_factor, body_per_cell, prf, va, fn, antenna_bw_rad, dr;
    uint32_t range_count;
} rsc_iq_params;
typedef struct rsc_iq_writer rsc_iq_writer;

int rsc_iq_open(const char *path, const rsc_iq_params *params, const uint32_t counts[RSC_MAX_TYPES],
                const char *scan_mode, float scan_start, float scan_end, float scan_delta, uint32_t seed,
                rsc_iq_writer **out);
/* Append `count` pulses: pulses4 holds count rows of row_gates float4 (the
 * first range_count of each row are written, times `gain`); times, el_deg
 * and az_deg hold one value per pulse (NULL writes zeros).  The data are
 * copied before the call returns. */
int rsc_iq_write(rsc_iq_writer *w, uint32_t count, const float *times, const float *el_deg, const float *az_deg,
                 const float *pulses4, uint32_t row_gates, float gain);
/* Wait until every appended pulse is in the file. */
int rsc_iq_flush(rsc_iq_writer *w);
int rsc_iq_close(rsc_iq_writer *w);
const char *rsc_iq_last_error(void);

/* ---- LES frame source (additive) ----
 * The LES ingest of les.c: the grid file fort.10_2 (les.c:477-518) and the
 * frame files LES_mean_1_6_fnum<k>.dat (k = 1, 2, ...; 10 volumes each, every
 * volume a time stamp and the u, v, w, p, t planes as Fortran records,
 * les.c:318-422) in one LES folder (<tables>/les/<config>, the folder
 * LES_init_with_config_path finds), the per-config constants of
 * les.c:158-208 and the remap of les.c:388-406 (u, v, w scaled by v0 into
 * uvwt with t * t0; p * p0 into cpxx lane 1, or lane 0 for "flat").  A
 * background thread reads the frame after the last one asked for, as
 * LES_background_read does; rsc_les_upload_async sends a frame's raw planes
 * (20 B per cell instead of the 32 B of uvwt + cpxx) to the device on a copy
 * stream and remaps them there, so the frame swap of RS_advance_time
 * (rs.c:5188-5200) overlaps the pulse loop. */
typedef struct {
    uint32_t nx, ny, nz;          /* cells per axis (the data grid, les.c:520-547) */
    uint32_t files;               /* frame files found */
    uint32_t volumes_per_file;    /* from the first file's size (les.c:212-244) */
    uint32_t frames;              /* files x volumes_per_file (LES_get_table_count) */
    int32_t is_stretched;         /* stretched grid (suctvort, suctvort_large) */
    int32_t p_for_cn2;            /* p goes to cpxx lane 0 (config "flat") */
    float tr, tp;                 /* refresh time, period of a frame (LES_get_table_period) */
    float v0, p0, t0;             /* scale of u, v, w / p / t */
    float ax, ay, az, rx, ry, rz; /* stretched: a r^n series; uniform: rx..rz = spacing */
} rsc_les_info;
typedef struct rsc_les_source rsc_les_source;

/* Open the LES folder `dir` (holding fort.10_2 and the frame files) with the
 * constants of `config` ("suctvort", "suctvort_large", "twocell", "flat" or
 * any other name, les.c:159-208) and start the read-ahead thread. */
int rsc_les_open(const char *dir, const char *config, rsc_les_source **out);
int rsc_les_get_info(rsc_les_source *src, rsc_les_info *info);
/* The data grid's node coordinates, nx * ny * nz floats each (LESTable
 * data.x / .y / .z); NULL skips an axis. */
int rsc_les_grid(rsc_les_source *src, float *x, float *y, float *z);
/* The 16-float LES descriptor RS_set_vel_data_to_LES_table (rs.c:3029-3126)
 * and RS_set_vel_data (rs.c:2947-2976) derive from the table constants. */
int rsc_les_descriptor(const rsc_les_info *info, float desc[16]);
/* Frame `frame` (0 .. frames-1) remapped into host uvwt4 / cpxx4 arrays of
 * nx * ny * nz float4 (LES_get_frame, les.c:666-694); *time (may be NULL)
 * gets the frame's time stamp.  The frame after it is read ahead. */
int rsc_les_read(rsc_les_source *src, uint32_t frame, float *uvwt4, float *cpxx4, float *time);
/* Start reading `frame` on the background thread. */
int rsc_les_prefetch(rsc_les_source *src, uint32_t frame);
/* Frame `frame` into LES slot `slot` of the worker (allocating the slots as
 * rsc_set_les does) with the descriptor of rsc_les_descriptor: the raw
 * planes go to the device on the worker's copy stream while earlier work
 * runs, the remap kernel writes the slot after the work queued so far on
 * the worker, and the first later advance that reads the slot waits for it.
 * The next frame is read ahead. */
int rsc_les_upload_async(rsc_worker *w, rsc_les_source *src, int slot, uint32_t frame, float *time);
/* Stop the thread, wait for copies out of the source's buffers, free it. */
int rsc_les_close(rsc_les_source *src);
/* Message of the last failed rsc_les_* call of this thread other than
 * rsc_les_upload_async, which reports through rsc_last_error. */
const char *rsc_les_last_error(void);

/* Limits of rsc_make_pulse_noalloc (its scratch is a fixed device array of
 * about 9 KB per GPU that loads this library). */
#define RSC_NOALLOC_MAX_GATES 128
#define RSC_NOALLOC_MAX_RANGE_TABLE 64
#define RSC_NOALLOC_MAX_ANGULAR_TABLE 1024

/* Form a pulse without allocating any device memory.  This entry point has no
 * counterpart in the reference: it is for callers that cannot call cudaMalloc
 * -- a real-time pulse loop that must not allocate, or an application whose
 * device memory is owned by another allocator or already fully reserved --
 * and that already hold the scatterer arrays in their own device buffers.
 *
 * Inputs: pos4 and rcs4 are device arrays of num_scats float4; pulse4 is a
 * device array of range_count float4 that receives the per-gate (Ih, Qh, Iv,
 * Qv) sums (no gain applied).  The weight tables, their descriptors and
 * sim_desc are host arrays read during the call: they travel to the device
 * by value in the launch parameters of two kernels (a one-block set-up that
 * fills the scratch, then the pulse), so the call queues no host-to-device
 * copy, reads no host memory after it returns, and does not wait for earlier
 * work on `stream` (a cudaStream_t, NULL for the default stream).  The pulse
 * is the one rsc_make_pulse forms in RSC_PULSE_PLAIN mode.
 *
 * The scratch the kernels need (an FP64 accumulator per gate, a completion
 * counter, gate origins, the weight tables) lives in one fixed __device__
 * array in the library instead of in memory the call allocates: every GPU
 * that loads the library holds about 9 KB for it until the process exits.
 * The accumulator and the counter are cleared at each call.  The first call
 * on a device looks the array's address up (once per device, with that
 * device current); make that first call before any stream capture.  All
 * calls share the one array and it keeps the contents of the last call: two
 * calls whose work overlaps on the GPU race, so order them on one stream or
 * synchronise between them.  Sizes above the RSC_NOALLOC_* limits, and a
 * descriptor whose max index is not inside its table, return RSC_ERR_ARG with
 * a message naming the limit.  No cudaMalloc, cudaFree or other allocating
 * call is made. */
int rsc_make_pulse_noalloc(const float *pos4, const float *rcs4, size_t num_scats, const float *range_weight,
                           uint32_t range_n, const float range_desc[4], const float *angular_weight,
                           uint32_t angular_n, const float angular_desc[4], float range_start, float range_delta,
                           uint32_t range_count, const float sim_desc[16], float *pulse4, void *stream);

/* Diagnostics: evaluate the shared elementary functions (rsmath.h) on the
 * device; fn: 0 sin, 1 cos, 2 log, 3 log1p, 4 acos, 5 atan2(a, b), 6 exp,
 * 7 pow(a, b), 8 the pulse kernel's closed-form range weight of distance a
 * on the triangle table {0, 1, 0} with scale b, origin 1, max 2; 9 / 10
 * the error (against double) of the compensated pulse's double-float sine /
 * cosine of the two-way phase b a for a range a and a wave number b,
 * 11 / 12 the same for the plain FP32 form.  Host arrays of n floats. */
int rsc_eval_math(int fn, const float *a, const float *b, float *out, size_t n);

#ifdef __cplusplus
}
#endif

#endif
