// extern "C" boundary of psvwave_gb300 (declared in include/psvwave.h).
// Every call catches C++ exceptions and turns them into a status code plus a
// per-thread message, so nothing is thrown across the ABI.
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>

#include "../../include/psvwave.h"
#include "psv_batch.hpp"
#include "psv_model.hpp"

struct psv_model {
  psv::Model impl;
  template <typename... A>
  explicit psv_model(A &&...a) : impl(std::forward<A>(a)...) {}
};

struct psv_batch {
  psv::Batch impl;
  explicit psv_batch(int device) : impl(device) {}
};

namespace {

thread_local std::string g_last_error;

template <class F>
int guarded(F &&f) {
  try {
    f();
    return PSV_OK;
  } catch (const psv::Error &e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    g_last_error = "host memory allocation failed";
    return PSV_ERR_INTERNAL;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return PSV_ERR_INTERNAL;
  }
}

void need(const void *p, const char *what) {
  if (!p) throw psv::Error(PSV_ERR_INVALID_ARGUMENT, std::string(what) + " must not be NULL");
}

psv::Model &M(psv_model *m) {
  need(m, "model");
  return m->impl;
}

const psv::Model &M(const psv_model *m) {
  need(m, "model");
  return m->impl;
}

}  // namespace

extern "C" {

int psv_abi_version(void) { return PSVWAVE_ABI_VERSION; }

const char *psv_last_error(void) { return g_last_error.c_str(); }

int psv_device_count(int *count) {
  return guarded([&] {
    need(count, "count");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
      cudaGetLastError();
      n = 0;
    }
    *count = n;
  });
}

int psv_host_alloc(size_t bytes, void **ptr) {
  return guarded([&] {
    need(ptr, "ptr");
    *ptr = nullptr;
    if (!bytes) return;
    const cudaError_t e = cudaMallocHost(ptr, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      *ptr = nullptr;
      throw psv::Error(PSV_ERR_CUDA, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
    }
  });
}

int psv_host_free(void *ptr) {
  return guarded([&] {
    if (!ptr) return;
    const cudaError_t e = cudaFreeHost(ptr);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw psv::Error(PSV_ERR_CUDA, std::string("cudaFreeHost: ") + cudaGetErrorString(e));
    }
  });
}

int psv_create_from_ini(const char *path, int precision, int device, psv_model **out) {
  return guarded([&] {
    need(path, "path");
    need(out, "out");
    *out = nullptr;
    psv::Config cfg = psv::read_ini(path);
    *out = new psv_model(cfg, precision, device);
  });
}

int psv_create(const psv_params *p, int precision, int device, psv_model **out) {
  return guarded([&] {
    need(p, "params");
    need(out, "out");
    *out = nullptr;
    psv::Config c;
    c.nt = p->nt;
    c.nx_inner = p->nx_inner;
    c.nz_inner = p->nz_inner;
    c.nx_inner_boundary = p->nx_inner_boundary;
    c.nz_inner_boundary = p->nz_inner_boundary;
    c.dx = p->dx;
    c.dz = p->dz;
    c.dt = p->dt;
    c.np_boundary = p->np_boundary;
    c.np_factor = p->np_factor;
    c.scalar_rho = p->scalar_rho;
    c.scalar_vp = p->scalar_vp;
    c.scalar_vs = p->scalar_vs;
    c.npx = p->npx;
    c.npz = p->npz;
    c.peak_frequency = p->peak_frequency;
    c.source_timeshift = p->source_timeshift;
    c.delay_cycles_per_shot = p->delay_cycles_per_shot;
    c.n_sources = p->n_sources;
    c.n_shots = p->n_shots;
    if (p->n_sources > 0) {
      need(p->ix_sources, "ix_sources");
      need(p->iz_sources, "iz_sources");
      need(p->moment_angles, "moment_angles");
      c.ix_sources.assign(p->ix_sources, p->ix_sources + p->n_sources);
      c.iz_sources.assign(p->iz_sources, p->iz_sources + p->n_sources);
      c.moment_angles.assign(p->moment_angles, p->moment_angles + p->n_sources);
    }
    if (p->n_shots > 0) {
      need(p->shot_offsets, "shot_offsets");
      for (int s = 0; s < p->n_shots; ++s) {
        const int a = p->shot_offsets[s], b = p->shot_offsets[s + 1];
        if (a < 0 || b < a) throw psv::Error(PSV_ERR_INVALID_ARGUMENT, "bad shot_offsets");
        if (b > a) need(p->shot_sources, "shot_sources");
        c.shots.emplace_back(p->shot_sources + a, p->shot_sources + b);
      }
    }
    c.nr = p->nr;
    if (p->nr > 0) {
      need(p->ix_receivers, "ix_receivers");
      need(p->iz_receivers, "iz_receivers");
      c.ix_receivers.assign(p->ix_receivers, p->ix_receivers + p->nr);
      c.iz_receivers.assign(p->iz_receivers, p->iz_receivers + p->nr);
    }
    c.snapshot_interval = p->snapshot_interval;
    if (p->observed_data_folder) c.observed_data_folder = p->observed_data_folder;
    if (p->stf_folder) c.stf_folder = p->stf_folder;
    *out = new psv_model(c, precision, device);
  });
}

int psv_clone(const psv_model *m, psv_model **out) {
  return guarded([&] {
    need(out, "out");
    *out = nullptr;
    *out = new psv_model(M(m));
  });
}

int psv_destroy(psv_model *m) {
  return guarded([&] { delete m; });
}

namespace {
void fill_info(const psv::Config &c, const psv::Geometry &g, psv_info *o) {
    std::memset(o, 0, sizeof(*o));
    o->nt = c.nt;
    o->nx = g.nx;
    o->nz = g.nz;
    o->nx_inner = c.nx_inner;
    o->nz_inner = c.nz_inner;
    o->nx_inner_boundary = c.nx_inner_boundary;
    o->nz_inner_boundary = c.nz_inner_boundary;
    o->np_boundary = c.np_boundary;
    o->n_shots = c.n_shots;
    o->n_sources = c.n_sources;
    o->nr = c.nr;
    o->snapshot_interval = c.snapshot_interval;
    o->snapshots = g.snapshots;
    o->nx_free_parameters = g.nx_free;
    o->nz_free_parameters = g.nz_free;
    o->free_parameters = g.free_parameters;
    o->basis_gridpoints_x = c.npx;
    o->basis_gridpoints_z = c.npz;
    o->precision = -1;
    o->device = -1;
    o->dt = c.dt;
    o->dx = c.dx;
    o->dz = c.dz;
    o->np_factor = c.np_factor;
    o->peak_frequency = c.peak_frequency;
    o->alpha = g.alpha;
    o->delay_cycles_per_shot = c.delay_cycles_per_shot;
    o->source_timeshift = c.source_timeshift;
    o->scalar_rho = c.scalar_rho;
    o->scalar_vp = c.scalar_vp;
    o->scalar_vs = c.scalar_vs;
}
}  // namespace

int psv_config_info(const char *path, psv_info *o) {
  return guarded([&] {
    need(path, "path");
    need(o, "out");
    psv::Config c = psv::read_ini(path);
    psv::Geometry g = psv::validate(c);
    fill_info(c, g, o);
  });
}

int psv_get_info(const psv_model *m, psv_info *o) {
  return guarded([&] {
    need(o, "out");
    const psv::Model &x = M(m);
    fill_info(x.config(), x.geometry(), o);
    o->precision = x.precision();
    o->device = x.device();
    o->misfit = x.misfit();
  });
}

int psv_get_shot_sources(const psv_model *m, int *offsets, int *sources) {
  return guarded([&] {
    need(offsets, "offsets");
    const psv::Config &c = M(m).config();
    int k = 0;
    offsets[0] = 0;
    for (int s = 0; s < c.n_shots; ++s) {
      for (int id : c.shots[s]) {
        if (sources) sources[k] = id;
        ++k;
      }
      offsets[s + 1] = k;
    }
  });
}

int psv_get_folders(const psv_model *m, char *observed, char *stf, size_t cap) {
  return guarded([&] {
    const psv::Config &c = M(m).config();
    if (cap == 0) return;
    if (observed) {
      std::strncpy(observed, c.observed_data_folder.c_str(), cap - 1);
      observed[cap - 1] = 0;
    }
    if (stf) {
      std::strncpy(stf, c.stf_folder.c_str(), cap - 1);
      stf[cap - 1] = 0;
    }
  });
}

int psv_forward_simulate(psv_model *m, int i_shot, int store_fields, int verbose,
                         int output_wavefields) {
  return guarded([&] {
    M(m).forward_simulate(i_shot, store_fields != 0, verbose != 0, output_wavefields != 0);
  });
}

int psv_adjoint_simulate(psv_model *m, int i_shot, int verbose) {
  return guarded([&] { M(m).adjoint_simulate(i_shot, verbose != 0); });
}

int psv_calculate_l2_misfit(psv_model *m, double *misfit) {
  return guarded([&] {
    double v = M(m).calculate_l2_misfit();
    if (misfit) *misfit = v;
  });
}

int psv_calculate_l2_adjoint_sources(psv_model *m) {
  return guarded([&] { M(m).calculate_l2_adjoint_sources(); });
}

int psv_reset_kernels(psv_model *m) {
  return guarded([&] { M(m).reset_kernels(); });
}

int psv_map_kernels_to_velocity(psv_model *m) {
  return guarded([&] { M(m).map_kernels_to_velocity(); });
}

int psv_run_model(psv_model *m, int verbose, int simulate_adjoint) {
  return guarded([&] { M(m).run_model(verbose != 0, simulate_adjoint != 0); });
}

int psv_update_from_velocity(psv_model *m) {
  return guarded([&] { M(m).update_from_velocity(); });
}

int psv_get_parameter_fields(psv_model *m, double *vp, double *vs, double *rho) {
  return guarded([&] { M(m).get_parameter_fields(vp, vs, rho); });
}

int psv_set_parameter_fields(psv_model *m, const double *vp, const double *vs,
                             const double *rho) {
  return guarded([&] {
    need(vp, "vp");
    need(vs, "vs");
    need(rho, "rho");
    M(m).set_parameter_fields(vp, vs, rho, false);
    M(m).synchronize();
  });
}

int psv_load_model(psv_model *m, const char *de_path, const char *vp_path,
                   const char *vs_path, int verbose) {
  return guarded([&] {
    need(de_path, "de_path");
    need(vp_path, "vp_path");
    need(vs_path, "vs_path");
    M(m).load_model(de_path, vp_path, vs_path, verbose != 0);
  });
}

int psv_get_kernels(psv_model *m, double *vp_k, double *vs_k, double *rho_k) {
  return guarded([&] { M(m).get_kernels(vp_k, vs_k, rho_k, false); });
}

int psv_get_lame_kernels(psv_model *m, double *lambda_k, double *mu_k, double *rho_k) {
  return guarded([&] { M(m).get_lame_kernels(lambda_k, mu_k, rho_k); });
}

int psv_get_synthetic_data(psv_model *m, double *ux, double *uz) {
  return guarded([&] { M(m).get_data(psv::Model::kSynthetic, ux, uz, false); });
}

int psv_set_synthetic_data(psv_model *m, const double *ux, const double *uz) {
  return guarded([&] {
    need(ux, "ux");
    need(uz, "uz");
    M(m).set_data(psv::Model::kSynthetic, ux, uz, false);
    M(m).synchronize();
  });
}

int psv_get_observed_data(psv_model *m, double *ux, double *uz) {
  return guarded([&] { M(m).get_data(psv::Model::kObserved, ux, uz, false); });
}

int psv_set_observed_data(psv_model *m, const double *ux, const double *uz) {
  return guarded([&] {
    need(ux, "ux");
    need(uz, "uz");
    M(m).set_data(psv::Model::kObserved, ux, uz, false);
    M(m).synchronize();
  });
}

int psv_get_adjoint_sources(psv_model *m, double *ux, double *uz) {
  return guarded([&] { M(m).get_data(psv::Model::kAdjoint, ux, uz, false); });
}

int psv_get_snapshots(psv_model *m, double *vx, double *vz, double *txx, double *tzz,
                      double *txz) {
  return guarded([&] {
    double *out[5] = {vx, vz, txx, tzz, txz};
    M(m).get_snapshots(out);
  });
}

int psv_get_wavefields(psv_model *m, double *vx, double *vz, double *txx, double *tzz,
                       double *txz) {
  return guarded([&] {
    double *out[5] = {vx, vz, txx, tzz, txz};
    M(m).get_wavefields(out);
  });
}

int psv_get_stf(psv_model *m, double *stf) {
  return guarded([&] {
    need(stf, "stf");
    M(m).get_stf(stf);
  });
}

int psv_get_moment(psv_model *m, double *moment) {
  return guarded([&] {
    need(moment, "moment");
    M(m).get_moment(moment);
  });
}

int psv_set_stf(psv_model *m, const double *stf) {
  return guarded([&] {
    need(stf, "stf");
    M(m).set_stf(stf);
  });
}

int psv_set_moment(psv_model *m, const double *moment) {
  return guarded([&] {
    need(moment, "moment");
    M(m).set_moment(moment);
  });
}

int psv_get_taper(psv_model *m, double *taper) {
  return guarded([&] {
    need(taper, "taper");
    M(m).get_taper(taper);
  });
}

int psv_get_model_vector(psv_model *m, double *out) {
  return guarded([&] {
    need(out, "out");
    M(m).get_model_vector(out);
  });
}

int psv_set_model_vector(psv_model *m, const double *in) {
  return guarded([&] {
    need(in, "in");
    M(m).set_model_vector(in);
  });
}

int psv_get_gradient_vector(psv_model *m, double *out) {
  return guarded([&] {
    need(out, "out");
    M(m).get_gradient_vector(out);
  });
}

int psv_load_vector(psv_model *m, const char *path, int verbose, double *out) {
  return guarded([&] {
    need(path, "path");
    need(out, "out");
    M(m).load_vector(path, verbose != 0, out);
  });
}

int psv_get_sources(psv_model *m, int in_units, int include_boundary, double *x, double *z) {
  return guarded([&] {
    need(x, "x");
    need(z, "z");
    M(m).get_sources(in_units != 0, include_boundary != 0, x, z);
  });
}

int psv_get_receivers(psv_model *m, int in_units, int include_boundary, double *x,
                      double *z) {
  return guarded([&] {
    need(x, "x");
    need(z, "z");
    M(m).get_receivers(in_units != 0, include_boundary != 0, x, z);
  });
}

int psv_get_coordinates(psv_model *m, int in_units, double *ix, double *iz) {
  return guarded([&] {
    need(ix, "ix");
    need(iz, "iz");
    M(m).get_coordinates(in_units != 0, ix, iz);
  });
}

int psv_get_extent(psv_model *m, int include_boundary, double *out4) {
  return guarded([&] {
    need(out4, "out");
    M(m).get_extent(include_boundary != 0, out4);
  });
}

int psv_write_receivers(psv_model *m, const char *prefix) {
  return guarded([&] { M(m).write_receivers(prefix ? prefix : ""); });
}

int psv_load_receivers(psv_model *m, int verbose) {
  return guarded([&] { M(m).load_receivers(verbose != 0); });
}

int psv_write_sources(psv_model *m) {
  return guarded([&] { M(m).write_sources(); });
}

int psv_write_kernels(psv_model *m) {
  return guarded([&] { M(m).write_kernels(); });
}

int psv_set_stream(psv_model *m, void *stream) {
  return guarded([&] { M(m).set_stream(static_cast<cudaStream_t>(stream)); });
}

int psv_set_async(psv_model *m, int async_calls) {
  return guarded([&] { M(m).set_async(async_calls != 0); });
}

int psv_set_graph_capture(psv_model *m, int enable) {
  return guarded([&] { M(m).set_graphs(enable != 0); });
}

int psv_synchronize(psv_model *m) {
  return guarded([&] { M(m).synchronize(); });
}

int psv_set_parameter_fields_device(psv_model *m, const double *vp, const double *vs,
                                    const double *rho) {
  return guarded([&] {
    need(vp, "vp");
    need(vs, "vs");
    need(rho, "rho");
    M(m).set_parameter_fields(vp, vs, rho, true);
  });
}

int psv_set_observed_data_device(psv_model *m, const double *ux, const double *uz) {
  return guarded([&] {
    need(ux, "ux");
    need(uz, "uz");
    M(m).set_data(psv::Model::kObserved, ux, uz, true);
  });
}

int psv_get_synthetic_data_device(psv_model *m, double *ux, double *uz) {
  return guarded([&] { M(m).get_data(psv::Model::kSynthetic, ux, uz, true); });
}

int psv_get_kernels_device(psv_model *m, double *vp_k, double *vs_k, double *rho_k) {
  return guarded([&] { M(m).get_kernels(vp_k, vs_k, rho_k, true); });
}

int psv_profile_forward(psv_model *m, int i_shot, int n_steps, double *per_step_ms,
                        double *kernel_ms, int max_kernels, int *n_kernels) {
  return guarded([&] {
    int n = M(m).profile_forward(i_shot, n_steps, per_step_ms, kernel_ms, max_kernels);
    if (n_kernels) *n_kernels = n;
  });
}

const char *psv_step_kernel_name(const psv_model *m, int k) {
  if (!m) return "";
  return m->impl.step_kernel_name(k);
}

int psv_set_tile_shape(psv_model *m, int shape) {
  return guarded([&] { M(m).set_tile_cfg(shape); });
}

int psv_get_tile_shape(const psv_model *m, int *shape) {
  return guarded([&] {
    need(shape, "shape");
    *shape = M(m).tile_cfg();
  });
}

int psv_autotune(psv_model *m, int n_steps, int *chosen) {
  return guarded([&] {
    const int c = M(m).autotune(n_steps > 0 ? n_steps : 50);
    if (chosen) *chosen = c;
  });
}

int psv_set_kernel_variant(psv_model *m, int variant) {
  return guarded([&] { M(m).set_variant(variant); });
}

int psv_get_kernel_variant(const psv_model *m, int *variant) {
  return guarded([&] {
    need(variant, "variant");
    *variant = M(m).variant();
  });
}

int psv_exact_gradient(psv_model *m, int checkpoint_every, double *misfit) {
  return guarded([&] {
    const double v = M(m).exact_gradient(checkpoint_every);
    if (misfit) *misfit = v;
  });
}

int psv_exact_gradient_shots(psv_model *m, int checkpoint_every, const int *shots, int n,
                             double *misfit) {
  return guarded([&] {
    if (n < 0) throw psv::Error(PSV_ERR_INVALID_ARGUMENT, "n must not be negative");
    if (n) need(shots, "shots");
    const double v = M(m).exact_gradient(checkpoint_every, std::vector<int>(shots, shots + n));
    if (misfit) *misfit = v;
  });
}

int psv_get_exact_gradient(psv_model *m, double *g_vp, double *g_vs, double *g_rho) {
  return guarded([&] { M(m).get_exact_gradient(g_vp, g_vs, g_rho, false); });
}

int psv_get_exact_gradient_device(psv_model *m, double *g_vp, double *g_vs, double *g_rho) {
  return guarded([&] { M(m).get_exact_gradient(g_vp, g_vs, g_rho, true); });
}

int psv_exact_bytes(const psv_model *m, int checkpoint_every, size_t *bytes) {
  return guarded([&] {
    need(bytes, "bytes");
    *bytes = M(m).exact_bytes(checkpoint_every);
  });
}

int psv_batch_create(int device, psv_batch **out) {
  return guarded([&] {
    need(out, "out");
    *out = nullptr;
    *out = new psv_batch(device);
  });
}

int psv_batch_destroy(psv_batch *b) {
  return guarded([&] { delete b; });
}

int psv_batch_add(psv_batch *b, psv_model *m, int i_shot) {
  return guarded([&] {
    need(b, "batch");
    b->impl.add(&M(m), i_shot);
  });
}

int psv_batch_forward(psv_batch *b, int store_fields, int n_steps) {
  return guarded([&] {
    need(b, "batch");
    b->impl.forward(store_fields != 0, n_steps);
  });
}

int psv_batch_set_tile_shape(psv_batch *b, int shape) {
  return guarded([&] {
    need(b, "batch");
    b->impl.set_tile_cfg(shape);
  });
}

int psv_batch_autotune(psv_batch *b, int n_steps, int *chosen) {
  return guarded([&] {
    need(b, "batch");
    const int c = b->impl.autotune(n_steps > 0 ? n_steps : 50);
    if (chosen) *chosen = c;
  });
}

int psv_batch_set_persistent(psv_batch *b, int persistent) {
  return guarded([&] {
    need(b, "batch");
    b->impl.set_persistent(persistent != 0);
  });
}

int psv_batch_get_persistent(const psv_batch *b, int *persistent) {
  return guarded([&] {
    need(b, "batch");
    need(persistent, "persistent");
    *persistent = b->impl.persistent() ? 1 : 0;
  });
}

int psv_batch_set_parameter_fields_device(psv_batch *b, const double *fields,
                                          long long member_stride, const int *flags) {
  return guarded([&] {
    need(b, "batch");
    need(fields, "fields");
    if (member_stride < 0) throw psv::Error(PSV_ERR_INVALID_ARGUMENT, "negative member stride");
    b->impl.set_parameter_fields_device(fields, static_cast<size_t>(member_stride), flags);
  });
}

int psv_batch_set_cluster(psv_batch *b, int cluster) {
  return guarded([&] {
    need(b, "batch");
    b->impl.set_cluster(cluster != 0);
  });
}

int psv_batch_get_cluster(const psv_batch *b, int *cluster) {
  return guarded([&] {
    need(b, "batch");
    need(cluster, "cluster");
    *cluster = b->impl.cluster() ? 1 : 0;
  });
}

int psv_batch_cluster_fits(psv_batch *b, int *fits) {
  return guarded([&] {
    need(b, "batch");
    need(fits, "fits");
    *fits = b->impl.cluster_fits() ? 1 : 0;
  });
}

int psv_batch_set_active(psv_batch *b, const int *flags, int n) {
  return guarded([&] {
    need(b, "batch");
    b->impl.set_active(flags, n);
  });
}

int psv_batch_misfits(psv_batch *b, double *out, int n) {
  return guarded([&] {
    need(b, "batch");
    need(out, "out");
    b->impl.misfits(out, n);
  });
}

int psv_batch_info(const psv_batch *b, int *members, int *tiles, double *cells) {
  return guarded([&] {
    need(b, "batch");
    if (members) *members = b->impl.size();
    if (tiles) *tiles = b->impl.tiles();
    if (cells) *cells = b->impl.cells();
  });
}

int psv_device_bytes(const psv_model *m, size_t *bytes) {
  return guarded([&] {
    need(bytes, "bytes");
    *bytes = M(m).device_bytes();
  });
}

}  // extern "C"

namespace psv {
// Lets other translation units report through psv_last_error().
void set_last_error(const std::string &msg) { g_last_error = msg; }
}  // namespace psv
