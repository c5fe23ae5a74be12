// C entry points over the psvWave reference's own fdModel class, so that the
// unmodified reference solver (src/fdModel.cpp, src/contiguous_arrays.cpp)
// can be driven from Python through ctypes. This replaces the reference's
// pybind11 module (src/psvWave.cpp), which needs Eigen's pybind11 bridge that
// is absent here; every call below forwards to the reference method named in
// its comment and copies arrays the way src/psvWave.cpp:33-63,256-297 does.
//
// Test infrastructure only: compiled into oracle/_ref by oracle/build_ref.sh
// and used to pin the oracle port and to make golden fixtures.
#include <cstring>
#include <exception>
#include <string>

#include "fdModel.h"

namespace {
std::string g_err;
template <class F>
int guarded(F f) {
  try {
    f();
    return 0;
  } catch (std::exception &e) {
    g_err = e.what();
    return 1;
  }
}
}  // namespace

extern "C" {

const char *ref_last_error() { return g_err.c_str(); }

// fdModel(const char*) -- src/fdModel.cpp:16-27
void *ref_create(const char *ini) {
  fdModel *m = nullptr;
  if (guarded([&] { m = new fdModel(ini); })) return nullptr;
  return m;
}

// fdModel(const fdModel&) -- src/fdModel.cpp:64-97
void *ref_copy(void *h) { return new fdModel(*static_cast<fdModel *>(h)); }

void ref_destroy(void *h) { delete static_cast<fdModel *>(h); }

// Integer attributes in a fixed order (the read-only attributes of
// src/psvWave.cpp:499-588).
void ref_info(void *h, int *o) {
  fdModel *m = static_cast<fdModel *>(h);
  int v[] = {m->nt, m->nx, m->nz, m->nx_inner, m->nz_inner, m->nx_inner_boundary,
             m->nz_inner_boundary, m->np_boundary, m->n_shots, m->n_sources, m->nr,
             m->snapshot_interval, m->snapshots, m->nx_free_parameters,
             m->nz_free_parameters, m->free_parameters, m->basis_gridpoints_x,
             m->basis_gridpoints_z};
  std::memcpy(o, v, sizeof(v));
}

void ref_scalars(void *h, double *o) {
  fdModel *m = static_cast<fdModel *>(h);
  double v[] = {m->dt, m->dx, m->dz, m->np_factor, m->peak_frequency, m->alpha,
                m->delay_cycles_per_shot, m->misfit};
  std::memcpy(o, v, sizeof(v));
}

// Raw pointers to the reference's own arrays, by name.
double *ref_array(void *h, const char *name) {
  fdModel *m = static_cast<fdModel *>(h);
  std::string n(name);
  if (n == "vx") return m->vx;
  if (n == "vz") return m->vz;
  if (n == "txx") return m->txx;
  if (n == "tzz") return m->tzz;
  if (n == "txz") return m->txz;
  if (n == "lm") return m->lm;
  if (n == "la") return m->la;
  if (n == "mu") return m->mu;
  if (n == "b_vx") return m->b_vx;
  if (n == "b_vz") return m->b_vz;
  if (n == "rho") return m->rho;
  if (n == "vp") return m->vp;
  if (n == "vs") return m->vs;
  if (n == "taper") return m->taper;
  if (n == "stf") return m->stf;
  if (n == "moment") return m->moment;
  if (n == "rtf_ux") return m->rtf_ux;
  if (n == "rtf_uz") return m->rtf_uz;
  if (n == "rtf_ux_true") return m->rtf_ux_true;
  if (n == "rtf_uz_true") return m->rtf_uz_true;
  if (n == "a_stf_ux") return m->a_stf_ux;
  if (n == "a_stf_uz") return m->a_stf_uz;
  if (n == "lambda_kernel") return m->lambda_kernel;
  if (n == "mu_kernel") return m->mu_kernel;
  if (n == "density_l_kernel") return m->density_l_kernel;
  if (n == "vp_kernel") return m->vp_kernel;
  if (n == "vs_kernel") return m->vs_kernel;
  if (n == "density_v_kernel") return m->density_v_kernel;
  if (n == "accu_vx") return m->accu_vx;
  if (n == "accu_vz") return m->accu_vz;
  if (n == "accu_txx") return m->accu_txx;
  if (n == "accu_tzz") return m->accu_tzz;
  if (n == "accu_txz") return m->accu_txz;
  return nullptr;
}

int *ref_int_array(void *h, const char *name) {
  fdModel *m = static_cast<fdModel *>(h);
  std::string n(name);
  if (n == "ix_sources") return m->ix_sources;
  if (n == "iz_sources") return m->iz_sources;
  if (n == "ix_receivers") return m->ix_receivers;
  if (n == "iz_receivers") return m->iz_receivers;
  return nullptr;
}

// set_parameter_fields -- src/psvWave.cpp:256-297
void ref_set_parameter_fields(void *h, const double *vp, const double *vs, const double *rho) {
  fdModel *m = static_cast<fdModel *>(h);
  std::size_t n = static_cast<std::size_t>(m->nx) * m->nz;
  std::memcpy(m->vp, vp, n * sizeof(double));
  std::memcpy(m->vs, vs, n * sizeof(double));
  std::memcpy(m->rho, rho, n * sizeof(double));
  m->update_from_velocity();
}

// set_observed_data / set_synthetic_data -- src/psvWave.cpp:389-457
void ref_set_data(void *h, int observed, const double *ux, const double *uz) {
  fdModel *m = static_cast<fdModel *>(h);
  std::size_t n = static_cast<std::size_t>(m->n_shots) * m->nr * m->nt;
  std::memcpy(observed ? m->rtf_ux_true : m->rtf_ux, ux, n * sizeof(double));
  std::memcpy(observed ? m->rtf_uz_true : m->rtf_uz, uz, n * sizeof(double));
}

void ref_forward(void *h, int shot, int store) {  // src/fdModel.cpp:526
  static_cast<fdModel *>(h)->forward_simulate(shot, store != 0, false, false);
}
// The same with the reference's wave-field dumps (snapshots/vx%05d.txt and
// vz%05d.txt every 10 steps, relative to the working directory,
// src/fdModel.cpp:753-776).
void ref_forward_output(void *h, int shot, int store) {
  static_cast<fdModel *>(h)->forward_simulate(shot, store != 0, false, true);
}
void ref_adjoint(void *h, int shot) {  // src/fdModel.cpp:789
  static_cast<fdModel *>(h)->adjoint_simulate(shot, false);
}
double ref_misfit(void *h) {  // src/fdModel.cpp:1128
  fdModel *m = static_cast<fdModel *>(h);
  m->calculate_l2_misfit();
  return m->misfit;
}
void ref_adjoint_sources(void *h) {  // src/fdModel.cpp:1147
  static_cast<fdModel *>(h)->calculate_l2_adjoint_sources();
}
void ref_reset_kernels(void *h) { static_cast<fdModel *>(h)->reset_kernels(); }
void ref_map_kernels(void *h) { static_cast<fdModel *>(h)->map_kernels_to_velocity(); }
void ref_run_model(void *h, int adjoint) {  // src/fdModel.cpp:1291
  static_cast<fdModel *>(h)->run_model(false, adjoint != 0);
}

// Model/gradient vectors -- src/fdModel.cpp:1358-1515
void ref_get_model_vector(void *h, double *out) {
  dynamic_vector v = static_cast<fdModel *>(h)->get_model_vector();
  std::memcpy(out, v.data(), v.size() * sizeof(double));
}
void ref_set_model_vector(void *h, const double *in) {
  fdModel *m = static_cast<fdModel *>(h);
  dynamic_vector v(m->free_parameters, 1);
  std::memcpy(v.data(), in, v.size() * sizeof(double));
  m->set_model_vector(v);
}
void ref_get_gradient_vector(void *h, double *out) {
  dynamic_vector v = static_cast<fdModel *>(h)->get_gradient_vector();
  std::memcpy(out, v.data(), v.size() * sizeof(double));
}
int ref_load_vector(void *h, const char *path, double *out) {
  fdModel *m = static_cast<fdModel *>(h);
  return guarded([&] {
    dynamic_vector v = m->load_vector(path, false);
    std::memcpy(out, v.data(), v.size() * sizeof(double));
  });
}
int ref_load_model(void *h, const char *de, const char *vp, const char *vs) {
  fdModel *m = static_cast<fdModel *>(h);
  return guarded([&] { m->load_model(de, vp, vs, false); });
}
void ref_write_receivers(void *h) { static_cast<fdModel *>(h)->write_receivers(); }
int ref_load_receivers(void *h) {
  fdModel *m = static_cast<fdModel *>(h);
  return guarded([&] { m->load_receivers(false); });
}
void ref_write_sources(void *h) { static_cast<fdModel *>(h)->write_sources(); }
void ref_write_kernels(void *h) { static_cast<fdModel *>(h)->write_kernels(); }

}  // extern "C"
