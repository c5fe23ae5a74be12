// Configuration of one P-SV model: what the reference's constructors read
// (src/fdModel.cpp:29-62 explicit arguments, src/fdModel.cpp:470-523 INI
// file) and the geometry derived from it (src/fdModel.cpp:390-468).
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

namespace psv {

// Error carrying one of the psv_status codes of include/psvwave.h.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &msg) : std::runtime_error(msg), code(c) {}
};

struct Config {
  int nt = 0, nx_inner = 0, nz_inner = 0, nx_inner_boundary = 0, nz_inner_boundary = 0;
  double dx = 0, dz = 0, dt = 0;
  int np_boundary = 0;
  double np_factor = 0;
  double scalar_rho = 0, scalar_vp = 0, scalar_vs = 0;
  int npx = 1, npz = 1;
  double peak_frequency = 0, source_timeshift = 0, delay_cycles_per_shot = 0;
  int n_sources = 0, n_shots = 0;
  std::vector<int> ix_sources, iz_sources;  // inner-grid indices
  std::vector<double> moment_angles;        // degrees
  std::vector<std::vector<int>> shots;      // which_source_to_fire_in_which_shot
  int nr = 0;
  std::vector<int> ix_receivers, iz_receivers;  // inner-grid indices
  int snapshot_interval = 1;
  std::string observed_data_folder = ".", stf_folder = ".";
};

// Grid geometry derived from a Config (src/fdModel.cpp:398-407,460-467).
struct Geometry {
  int nx = 0, nz = 0;
  int nx_free = 0, nz_free = 0, free_parameters = 0;
  int snapshots = 0;
  double alpha = 0;  // 1 / peak_frequency, kept as the reference keeps it
  // Free (invertible) region in absolute grid indices, [x0, x1) x [z0, z1)
  // (src/fdModel.cpp:821-825).
  int fx0 = 0, fx1 = 0, fz0 = 0, fz1 = 0;
};

// Reads an INI configuration the way the reference does (inih rules, list
// syntax "{a, b}" and "{{a, b}, {c}}"). Throws Error.
Config read_ini(const std::string &path);

// Checks a configuration against the reference's rules (src/fdModel.cpp:
// 404-467) plus the bounds every source stencil and receiver must respect on
// the GPU, and derives the geometry. Throws Error.
Geometry validate(const Config &c);

}  // namespace psv
