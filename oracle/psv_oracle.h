/*
 * psv_oracle -- CPU restatement of psvWave's P-SV solver (larsgeb/psvWave,
 * src/fdModel.cpp), in plain C with OpenMP.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker that the GPU library is
 * compared against (tests/, __graft_entry__.smoke()) and the CPU baseline that
 * bench.py times; the product never links, loads or calls it.
 *
 * Parity of this restatement is pinned against the reference's own solver
 * (oracle/_ref, built from src/fdModel.cpp by oracle/build_ref.sh): bit-exact
 * seismograms, snapshots and kernels on the reference's test configuration,
 * and the known answers of the reference's Notebook 2 (misfit 1920401.82,
 * gradient max-norm 77.1590).
 *
 * Layout follows the reference: every grid is [nx][nz] with z fastest
 * (src/contiguous_arrays.cpp:43-50); receiver data is [shots][nr][nt];
 * snapshots are [shots][snapshots][nx][nz].
 */
#ifndef PSV_ORACLE_H
#define PSV_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct po_params {
  int nt, nx_inner, nz_inner, nx_inner_boundary, nz_inner_boundary;
  double dx, dz, dt;
  int np_boundary;
  double np_factor;
  double scalar_rho, scalar_vp, scalar_vs;
  int npx, npz;
  double peak_frequency, source_timeshift, delay_cycles_per_shot;
  int n_sources, n_shots;
  const int *ix_sources, *iz_sources; /* n_sources, inner-grid indices */
  const double *moment_angles;        /* n_sources, degrees */
  const int *shot_offsets;            /* n_shots + 1, CSR into shot_sources */
  const int *shot_sources;            /* source ids fired per shot */
  int nr;
  const int *ix_receivers, *iz_receivers; /* nr, inner-grid indices */
  int snapshot_interval;
} po_params;

typedef struct po_model po_model;

/* Constructors: explicit parameters (src/fdModel.cpp:29-62) or an INI file
 * (src/fdModel.cpp:16-27,470-523). NULL on error; the message is copied into
 * err (errlen bytes). */
po_model *po_create(const po_params *p, char *err, int errlen);
po_model *po_create_from_ini(const char *path, char *err, int errlen);
po_model *po_copy(const po_model *m); /* src/fdModel.cpp:64-97 */
void po_destroy(po_model *m);

/* Integer attributes: nt nx nz nx_inner nz_inner nx_inner_boundary
 * nz_inner_boundary np_boundary n_shots n_sources nr snapshot_interval
 * snapshots nx_free_parameters nz_free_parameters free_parameters npx npz */
void po_info(const po_model *m, int *out18);
/* dt dx dz np_factor peak_frequency alpha delay_cycles_per_shot misfit */
void po_scalars(const po_model *m, double *out8);

/* Pointer to one of the model's arrays by the reference's member name
 * (vx vz txx tzz txz lm la mu b_vx b_vz rho vp vs taper stf moment rtf_ux
 * rtf_uz rtf_ux_true rtf_uz_true a_stf_ux a_stf_uz lambda_kernel mu_kernel
 * density_l_kernel vp_kernel vs_kernel density_v_kernel accu_vx accu_vz
 * accu_txx accu_tzz accu_txz), or NULL. */
double *po_array(po_model *m, const char *name);
/* ix_sources iz_sources ix_receivers iz_receivers (absolute grid indices). */
int *po_int_array(po_model *m, const char *name);

void po_update_from_velocity(po_model *m);          /* src/fdModel.cpp:1034 */
void po_forward(po_model *m, int shot, int store);  /* src/fdModel.cpp:526 */
void po_adjoint(po_model *m, int shot);             /* src/fdModel.cpp:789 */
double po_misfit(po_model *m);                      /* src/fdModel.cpp:1128 */
void po_adjoint_sources(po_model *m);               /* src/fdModel.cpp:1147 */
void po_reset_kernels(po_model *m);                 /* src/fdModel.cpp:1310 */
void po_map_kernels(po_model *m);                   /* src/fdModel.cpp:1164 */
void po_run_model(po_model *m, int adjoint);        /* src/fdModel.cpp:1291 */
void po_get_model_vector(const po_model *m, double *out);   /* :1358 */
void po_set_model_vector(po_model *m, const double *in);    /* :1414 */
void po_get_gradient_vector(const po_model *m, double *out);/* :1459 */

/* Forward simulation of `shot` over time steps [0, n_steps) only -- used to
 * time a bounded sample of a long run. Same arithmetic as po_forward. */
void po_forward_steps(po_model *m, int shot, int store, int n_steps);

#ifdef __cplusplus
}
#endif
#endif
