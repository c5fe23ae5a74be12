/*
 * psvwave.h -- C ABI of psvwave_gb300, a GB300 (sm_103a) implementation of
 * psvWave's P-SV finite-difference solver (larsgeb/psvWave).
 *
 * Each entry point replaces one member of the reference's `fdModel` class
 * (src/fdModel.h, src/fdModel.cpp) or of its Python binding
 * (src/psvWave.cpp); the citation beside each declaration names it.
 *
 * Conventions
 *  - Every function returns PSV_OK (0) or a PSV_ERR_* code; the message of
 *    the last failure on the calling thread is psv_last_error(). No C++
 *    exception crosses this boundary.
 *  - Host arrays are double precision, C-contiguous, in the reference's
 *    layouts: grids [nx][nz] with z fastest (src/contiguous_arrays.cpp:43-50),
 *    receiver data [n_shots][nr][nt], snapshots [n_shots][snapshots][nx][nz].
 *  - The wave fields are advanced in the precision chosen at creation:
 *    PSV_FP32 (production) or PSV_FP64 (the reference's own precision,
 *    bit-identical to it). Seismograms, misfit and kernel sums are FP64 in
 *    both modes.
 *  - Calls on one model are not thread-safe (the reference shares its fields
 *    between calls the same way). Distinct models are independent.
 *  - Device work is ordered on the model's CUDA stream; calls that hand data
 *    back to the host synchronise that stream.
 */
#ifndef PSVWAVE_H
#define PSVWAVE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PSVWAVE_ABI_VERSION 1

enum psv_status {
  PSV_OK = 0,
  PSV_ERR_INVALID_ARGUMENT = 1, /* std::invalid_argument in the reference */
  PSV_ERR_LENGTH = 2,           /* std::length_error in the reference */
  PSV_ERR_IO = 3,               /* file missing / wrong amount of data */
  PSV_ERR_CUDA = 4,             /* CUDA runtime failure */
  PSV_ERR_NUMERIC = 5,          /* non-finite wave field detected */
  PSV_ERR_INTERNAL = 6
};

enum psv_precision { PSV_FP32 = 0, PSV_FP64 = 1 };

typedef struct psv_model psv_model;

/* Scalar description of a model: the read-only attributes of the Python
 * class (src/psvWave.cpp:499-588) plus the configuration it was built from. */
typedef struct psv_info {
  int nt, nx, nz, nx_inner, nz_inner, nx_inner_boundary, nz_inner_boundary;
  int np_boundary, n_shots, n_sources, nr, snapshot_interval, snapshots;
  int nx_free_parameters, nz_free_parameters, free_parameters;
  int basis_gridpoints_x, basis_gridpoints_z;
  int precision, device;
  double dt, dx, dz, np_factor, peak_frequency, alpha, delay_cycles_per_shot;
  double source_timeshift, scalar_rho, scalar_vp, scalar_vs, misfit;
} psv_info;

/* Explicit-parameter description of a model; the arguments of the
 * reference's second constructor (src/fdModel.h:50-64). Source and receiver
 * indices are inner-grid indices (the absorbing boundary is added, as
 * src/fdModel.cpp:197-212 does). Shots are given in CSR form:
 * shot_sources[shot_offsets[s] .. shot_offsets[s+1]) fire in shot s. */
typedef struct psv_params {
  int nt, nx_inner, nz_inner, nx_inner_boundary, nz_inner_boundary;
  double dx, dz, dt;
  int np_boundary;
  double np_factor, scalar_rho, scalar_vp, scalar_vs;
  int npx, npz;
  double peak_frequency, source_timeshift, delay_cycles_per_shot;
  int n_sources, n_shots;
  const int *ix_sources, *iz_sources;
  const double *moment_angles;
  const int *shot_offsets, *shot_sources;
  int nr;
  const int *ix_receivers, *iz_receivers;
  int snapshot_interval;
  const char *observed_data_folder, *stf_folder;
} psv_params;

/* ---- library ---------------------------------------------------------- */
int psv_abi_version(void);
const char *psv_last_error(void);
/* Number of CUDA devices visible; 0 when none. */
int psv_device_count(int *count);

/* Page-locked host memory (cudaMallocHost / cudaFreeHost). Getters that copy
 * into it run at the host link's full rate instead of going through the
 * driver's staging of pageable memory. No counterpart in the reference (its
 * getters return fresh arrays, src/psvWave.cpp:33-63): psvwave_gb300.fdModel
 * backs the large arrays its getters return with blocks from a pool of these,
 * reused once an array is freed. */
int psv_host_alloc(size_t bytes, void **ptr);
int psv_host_free(void *ptr);

/* Parses and validates a configuration file (the reference's INI reading,
 * src/fdModel.cpp:470-523, and checks, src/fdModel.cpp:390-468) without
 * touching a GPU; fills `out` with precision = device = -1 and misfit = 0. */
int psv_config_info(const char *path, psv_info *out);

/* ---- construction ----------------------------------------------------- */
/* fdModel(const char *configuration_file) -- src/fdModel.cpp:16-27,470-523;
 * Python: fdModel(configuration_file_path) -- src/psvWave.cpp:465-471. */
int psv_create_from_ini(const char *path, int precision, int device, psv_model **out);
/* fdModel(nt, nx_inner, ...) -- src/fdModel.cpp:29-62. */
int psv_create(const psv_params *params, int precision, int device, psv_model **out);
/* fdModel(const fdModel&) -- src/fdModel.cpp:64-97; Python copy() --
 * src/psvWave.cpp:421-425. Deep copy incl. fields, data, kernels, snapshots. */
int psv_clone(const psv_model *m, psv_model **out);
/* ~fdModel() -- src/fdModel.cpp:99-137. Accepts NULL. */
int psv_destroy(psv_model *m);
int psv_get_info(const psv_model *m, psv_info *out);
/* which_source_to_fire_in_which_shot (src/psvWave.cpp:586-588) in CSR form:
 * offsets[n_shots+1], sources[n_sources]. */
int psv_get_shot_sources(const psv_model *m, int *offsets, int *sources);
/* Folders named by [output] (src/fdModel.cpp:517-518); buffers of `cap` bytes. */
int psv_get_folders(const psv_model *m, char *observed, char *stf, size_t cap);

/* ---- simulation ------------------------------------------------------- */
/* forward_simulate -- src/fdModel.cpp:526-787; Python binding
 * src/psvWave.cpp:112-158,476-498. `output_wavefields` writes
 * snapshots/vx%05d.txt and vz%05d.txt every 10 steps (src/fdModel.cpp:753-776). */
int psv_forward_simulate(psv_model *m, int i_shot, int store_fields, int verbose,
                         int output_wavefields);
/* adjoint_simulate -- src/fdModel.cpp:789-969; src/psvWave.cpp:160-205,634-650. */
int psv_adjoint_simulate(psv_model *m, int i_shot, int verbose);
/* calculate_l2_misfit -- src/fdModel.cpp:1128-1145. `misfit` may be NULL. */
int psv_calculate_l2_misfit(psv_model *m, double *misfit);
/* calculate_l2_adjoint_sources -- src/fdModel.cpp:1147-1162. */
int psv_calculate_l2_adjoint_sources(psv_model *m);
/* reset_kernels -- src/fdModel.cpp:1310-1324. */
int psv_reset_kernels(psv_model *m);
/* map_kernels_to_velocity -- src/fdModel.cpp:1164-1183. */
int psv_map_kernels_to_velocity(psv_model *m);
/* run_model(verbose, simulate_adjoint) -- src/fdModel.cpp:1291-1308: every
 * shot forward with storage, misfit, and (if simulate_adjoint) adjoint
 * sources, kernel reset, every shot adjoint and the velocity mapping. This is
 * one FWI gradient ("compute_gradients"). */
int psv_run_model(psv_model *m, int verbose, int simulate_adjoint);
/* update_from_velocity -- src/fdModel.cpp:1034-1051. */
int psv_update_from_velocity(psv_model *m);

/* ---- model, data and kernel transfer (host FP64 arrays) --------------- */
/* get_parameter_fields / set_parameter_fields -- src/psvWave.cpp:248-297
 * (set recomputes the Lame fields). */
int psv_get_parameter_fields(psv_model *m, double *vp, double *vs, double *rho);
int psv_set_parameter_fields(psv_model *m, const double *vp, const double *vs,
                             const double *rho);
/* load_model(de, vp, vs, verbose) -- src/fdModel.cpp:1185-1289: nx*nz
 * whitespace-separated values per file, ix-major. */
int psv_load_model(psv_model *m, const char *de_path, const char *vp_path,
                   const char *vs_path, int verbose);
/* get_kernels -- src/psvWave.cpp:299-306: (vp, vs, rho) velocity kernels. */
int psv_get_kernels(psv_model *m, double *vp_k, double *vs_k, double *rho_k);
/* The Lame-basis kernels (lambda, mu, density) the adjoint accumulates
 * (src/fdModel.h:224-226). */
int psv_get_lame_kernels(psv_model *m, double *lambda_k, double *mu_k, double *rho_k);
/* get/set_synthetic_data, get/set_observed_data -- src/psvWave.cpp:308-322,
 * 389-457. */
int psv_get_synthetic_data(psv_model *m, double *ux, double *uz);
int psv_set_synthetic_data(psv_model *m, const double *ux, const double *uz);
int psv_get_observed_data(psv_model *m, double *ux, double *uz);
int psv_set_observed_data(psv_model *m, const double *ux, const double *uz);
/* The adjoint sources a_stf_ux/uz (src/fdModel.h:246-247). */
int psv_get_adjoint_sources(psv_model *m, double *ux, double *uz);
/* get_snapshots -- src/psvWave.cpp:90-97: the five stored forward fields
 * vx, vz, txx, tzz, txz of all shots. Any pointer may be NULL to skip it. */
int psv_get_snapshots(psv_model *m, double *vx, double *vz, double *txx, double *tzz,
                      double *txz);
/* The current wave fields vx, vz, txx, tzz, txz (src/fdModel.h:209-213). */
int psv_get_wavefields(psv_model *m, double *vx, double *vz, double *txx, double *tzz,
                       double *txz);
/* The source time functions [n_sources][nt] (src/fdModel.h:240), the moment
 * tensors [n_sources][2][2] (src/fdModel.h:241) and the taper [nx][nz]
 * (src/fdModel.h:236). */
int psv_get_stf(psv_model *m, double *stf);
int psv_get_moment(psv_model *m, double *moment);
int psv_get_taper(psv_model *m, double *taper);

/* set_stf / set_moment -- no reference counterpart: the reference fixes
 * Ricker wavelets and dip-angle tensors (src/fdModel.cpp:214-246) and its
 * README lists the focal mechanism as not yet generalisable. They replace
 * the source time functions [n_sources][nt], or the moment tensors
 * [n_sources][2][2] (row-major M00 M01 M10 M11; M01 drives the (x,z)
 * couple and M10 the (z,x) couple of src/fdModel.cpp:681-751), for every
 * later simulation of this model, through the same injection terms. Values
 * must be finite. A Batch keeps the sources its members had when it was
 * built. */
int psv_set_stf(psv_model *m, const double *stf);
int psv_set_moment(psv_model *m, const double *moment);

/* get_model_vector / set_model_vector / get_gradient_vector --
 * src/fdModel.cpp:1358-1515; vectors of length free_parameters. */
int psv_get_model_vector(psv_model *m, double *out);
int psv_set_model_vector(psv_model *m, const double *in);
int psv_get_gradient_vector(psv_model *m, double *out);
/* load_vector(path, verbose) -- src/fdModel.cpp:1517-1572: reads
 * 3*nx_free*nz_free values (the unblocked size, as the reference does). */
int psv_load_vector(psv_model *m, const char *path, int verbose, double *out);

/* get_sources / get_receivers -- src/psvWave.cpp:324-387. */
int psv_get_sources(psv_model *m, int in_units, int include_boundary, double *x, double *z);
int psv_get_receivers(psv_model *m, int in_units, int include_boundary, double *x,
                      double *z);
/* get_coordinates -- src/psvWave.cpp:207-246. */
int psv_get_coordinates(psv_model *m, int in_units, double *ix, double *iz);
/* get_extent -- src/psvWave.cpp:99-110: out[4] = xmin, xmax, zmin, zmax. */
int psv_get_extent(psv_model *m, int include_boundary, double *out4);

/* ---- text I/O --------------------------------------------------------- */
/* write_receivers(prefix) -- src/fdModel.cpp:971-1006. */
int psv_write_receivers(psv_model *m, const char *prefix);
/* load_receivers(verbose) -- src/fdModel.cpp:1053-1126. */
int psv_load_receivers(psv_model *m, int verbose);
/* write_sources -- src/fdModel.cpp:1008-1032. */
int psv_write_sources(psv_model *m);
/* write_kernels -- src/fdModel.cpp:1326-1356. */
int psv_write_kernels(psv_model *m);

/* ---- device-side interface (PyTorch layer) ----------------------------- */
/* Order the model's device work on `stream` (a cudaStream_t; NULL = the
 * model's own stream). */
int psv_set_stream(psv_model *m, void *stream);
/* Make forward/adjoint return without waiting for the GPU (1) or wait, as
 * the reference's calls do (0, the default). */
int psv_set_async(psv_model *m, int async_calls);
/* Replay repeated forward/adjoint time loops as CUDA graphs (1, the
 * default: a loop is captured on its second identical call) or always launch
 * kernel by kernel (0). No counterpart in the reference. */
int psv_set_graph_capture(psv_model *m, int enable);
int psv_synchronize(psv_model *m);
/* Parameter fields from device FP64 buffers [nx][nz]. */
int psv_set_parameter_fields_device(psv_model *m, const double *vp, const double *vs,
                                    const double *rho);
/* Observed data from device FP64 buffers [n_shots][nr][nt]. */
int psv_set_observed_data_device(psv_model *m, const double *ux, const double *uz);
/* Copy the synthetic data / velocity kernels into device FP64 buffers. */
int psv_get_synthetic_data_device(psv_model *m, double *ux, double *uz);
int psv_get_kernels_device(psv_model *m, double *vp_k, double *vs_k, double *rho_k);
/* Bytes of device memory the model holds. */
int psv_device_bytes(const psv_model *m, size_t *bytes);

/* ---- measurement -------------------------------------------------------- */
/* Runs the first n_steps forward time steps of `i_shot` (no storage) with a
 * CUDA event around every kernel launch on the model's stream, and reports
 * the average device time per time step (*per_step_ms) and per launch of
 * each of the step's kernels (kernel_ms[k], in launch order; names from
 * psv_step_kernel_name). *n_kernels receives the launches per step. Has no
 * counterpart in the reference (which times with omp_get_wtime only,
 * src/fdModel.cpp:545-549). */
int psv_profile_forward(psv_model *m, int i_shot, int n_steps, double *per_step_ms,
                        double *kernel_ms, int max_kernels, int *n_kernels);
const char *psv_step_kernel_name(const psv_model *m, int k);

/* Time-step kernel variant: PSV_VARIANT_FUSED (one launch per step over
 * ping-pong buffers; FP32 only), PSV_VARIANT_TWO_KERNEL (separate stress and
 * velocity launches, as the reference's two loop nests; the only FP64
 * variant), PSV_VARIANT_FUSED_TMA (the fused step with TMA tile loads, one
 * launch per step; FP32, the default) or PSV_VARIANT_FUSED_TMA_PERSISTENT
 * (the same step, every time step of a simulation in one persistent launch
 * whose tiles start a step as soon as their neighbours have finished the
 * previous one). Results of the FP32 variants agree to FP32 rounding. No
 * counterpart in the reference. */
enum psv_variant {
  PSV_VARIANT_FUSED = 0,
  PSV_VARIANT_TWO_KERNEL = 1,
  PSV_VARIANT_FUSED_TMA = 2,
  PSV_VARIANT_FUSED_TMA_PERSISTENT = 3
};
int psv_set_kernel_variant(psv_model *m, int variant);
int psv_get_kernel_variant(const psv_model *m, int *variant);

/* Tile shape of the FP32 TMA step (x rows by z columns): PSV_TILE_32X60
 * (256 threads; large grids), PSV_TILE_16X28 or PSV_TILE_20X28 (128
 * threads). By default, grids with less than one wave of 32 x 60 tiles take
 * 16 x 28. psv_autotune times every tile shape with both TMA
 * launch schemes (PSV_VARIANT_FUSED_TMA and _PERSISTENT) on n_steps forward
 * steps of shot 0, replayed as CUDA graphs, keeps the fastest pair and
 * returns its shape in *chosen. No counterpart in the reference. */
enum psv_tile_shape { PSV_TILE_32X60 = 0, PSV_TILE_16X28 = 1, PSV_TILE_20X28 = 2 };
int psv_set_tile_shape(psv_model *m, int shape);
int psv_get_tile_shape(const psv_model *m, int *shape);
int psv_autotune(psv_model *m, int n_steps, int *chosen);

/* ---- exact discrete adjoint --------------------------------------------- */
/* Gradient of the L2 misfit (src/fdModel.cpp:1128-1145) over all shots with
 * respect to vp, vs and rho by the exact discrete adjoint: the transpose of
 * the time-stepping operator, run backwards. Unlike the reference's adjoint
 * (src/fdModel.cpp:789-969, a reverse-time re-run of the forward scheme),
 * it agrees with finite differences of the discrete misfit. Forward states
 * are rebuilt from checkpoints taken every `checkpoint_every` steps
 * (checkpoint_every >= nt keeps every state of the run). *misfit receives the
 * misfit; the gradient ([nx][nz] each) is read with psv_get_exact_gradient
 * (host) or psv_get_exact_gradient_device. psv_exact_bytes estimates the
 * device memory of a given checkpoint interval. */
int psv_exact_gradient(psv_model *m, int checkpoint_every, double *misfit);
/* The same over the listed shots only (each at most once): their misfit and
 * gradient, the per-rank part of a gradient sharded by shot across GPUs
 * (shots are independent, src/fdModel.cpp:1293-1305). */
int psv_exact_gradient_shots(psv_model *m, int checkpoint_every, const int *shots, int n,
                             double *misfit);
int psv_get_exact_gradient(psv_model *m, double *g_vp, double *g_vs, double *g_rho);
int psv_get_exact_gradient_device(psv_model *m, double *g_vp, double *g_vs, double *g_rho);
int psv_exact_bytes(const psv_model *m, int checkpoint_every, size_t *bytes);

/* ---- batched simulation --------------------------------------------------- */
/* A batch advances shots of many FP32 models -- of uneven grid sizes -- in
 * one TMA-step launch per time step, the whole time loop replayed as one CUDA
 * graph. Members must share nt and live on the batch's device; models must
 * outlive the batch. Seismograms (and, with store_fields, snapshots) land in
 * each member model's own arrays for that shot, as forward_simulate would
 * leave them. No counterpart in the reference, which runs one shot of one
 * model at a time (src/fdModel.cpp:1293-1296). */
typedef struct psv_batch psv_batch;
int psv_batch_create(int device, psv_batch **out);
int psv_batch_destroy(psv_batch *b);
int psv_batch_add(psv_batch *b, psv_model *m, int i_shot);
/* Forward simulation of every member over its first n_steps steps (all if
 * n_steps <= 0). */
int psv_batch_forward(psv_batch *b, int store_fields, int n_steps);
int psv_batch_set_tile_shape(psv_batch *b, int shape);
/* psv_batch_autotune times every tile shape with both launch schemes (one
 * launch per step, persistent) on n_steps steps of the active members, keeps
 * the fastest pair and returns its shape in *chosen (the scheme is read
 * with psv_batch_get_persistent). */
int psv_batch_autotune(psv_batch *b, int n_steps, int *chosen);
int psv_batch_info(const psv_batch *b, int *members, int *tiles, double *cells);
/* Which members (in the order added) the next psv_batch_forward advances:
 * flags[k] != 0; NULL = all (the default). Inactive members' CTAs exit at
 * once, so the captured time loop serves every subset. */
int psv_batch_set_active(psv_batch *b, const int *flags, int n);
/* L2 misfit of each member's model after psv_batch_forward, as
 * psv_calculate_l2_misfit computes it (src/fdModel.cpp:1128-1145), bit for
 * bit: out[k] for the n == members members in the order added (NaN for
 * inactive ones), one reduction per member on the batch's stream and one
 * copy back. Each active model's misfit is updated as
 * psv_calculate_l2_misfit would. */
int psv_batch_misfits(psv_batch *b, double *out, int n);
/* psv_set_parameter_fields_device (src/psvWave.cpp:256-297, from device
 * arrays) for every member k with flags[k] != 0 (all when flags is NULL):
 * its vp, vs and rho ([nx][nz] each, consecutive) start at
 * fields + k * member_stride (doubles, device memory). A model that is a
 * member more than once is set once; each model queues its copies and
 * medium update on its own stream, as its own call does, and the next
 * psv_batch_forward waits for them. */
int psv_batch_set_parameter_fields_device(psv_batch *b, const double *fields,
                                          long long member_stride, const int *flags);
/* Launch scheme of psv_batch_forward: 0 (the default) launches once per
 * time step, the loop captured as one CUDA graph; persistent != 0 runs every
 * time step of every member in one persistent launch over the batch's tile
 * table, tiles starting a step as soon as their neighbours have finished the
 * previous one. Results are identical. */
int psv_batch_set_persistent(psv_batch *b, int persistent);
int psv_batch_get_persistent(const psv_batch *b, int *persistent);
/* Cluster-resident scheme: cluster != 0 runs every member in its own
 * thread-block cluster that keeps the member's whole grid in shared memory
 * for every time step, all members in one launch (the batched form of the
 * model variant fused_cluster, whose results it equals bit for bit).
 * PSV_ERR_INVALID_ARGUMENT when a member does not fit a cluster; *fits
 * (psv_batch_cluster_fits) tells beforehand. psv_batch_set_persistent
 * switches it off; psv_batch_autotune also times it when the members fit. */
int psv_batch_set_cluster(psv_batch *b, int cluster);
int psv_batch_get_cluster(const psv_batch *b, int *cluster);
int psv_batch_cluster_fits(psv_batch *b, int *fits);

/* ---- no-allocation entry point ------------------------------------------ */
/* L2 misfit 0.5 dt sum((obs - syn)^2) over both components, written to the
 * device double *misfit, from caller-owned device arrays of n samples each
 * (e.g. n_shots * nr * nt), on `stream` (a cudaStream_t; NULL = the legacy
 * default stream). No counterpart in the reference: it is the same
 * reduction as psv_calculate_l2_misfit, for callers that cannot allocate
 * device memory (a TensorRT plugin's enqueue, an XLA custom call, a
 * pre-planned memory arena, a region being captured into a CUDA graph).
 * It allocates nothing: its partial sums live in a fixed 64 KiB __device__
 * array that every GPU loading this library holds until exit, so n is
 * limited to 16,777,216 samples; larger n returns PSV_ERR_INVALID_ARGUMENT.
 * The first call on a device (made current by the caller) looks up that
 * array's address; make that first call before any stream capture. The
 * address is kept per device ordinal for the life of the process: it
 * belongs to the device's primary context (the one the CUDA runtime uses),
 * so call this under that context, and not after cudaDeviceReset on the
 * device, which unloads the array and leaves the kept address stale. All calls
 * share the array: calls that overlap on the GPU race and must be ordered
 * (one stream, or events) by the caller. Asynchronous: the result is ready
 * when `stream` reaches it. */
int psv_l2_misfit_noalloc(const double *obs_ux, const double *syn_ux, const double *obs_uz,
                          const double *syn_uz, size_t n, double dt, double *misfit,
                          void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PSVWAVE_H */
