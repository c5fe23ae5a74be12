// One P-SV model resident on a GPU: the GB300 counterpart of the reference's
// fdModel class (src/fdModel.h:35-318). The configuration and setup tables
// live on the host; every array the time loop touches lives in device memory.
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <map>
#include <memory>
#include <tuple>
#include <string>
#include <vector>

#include "psv_config.hpp"
#include "psv_solver.hpp"
#include "psv_exact_tma.hpp"
#include "psv_tma.hpp"

namespace psv {

// Throws Error(PSV_ERR_CUDA) with the CUDA message when e is not cudaSuccess.
void cuda_check(cudaError_t e, const char *what);

// Makes `device` current for the scope and restores the previous device.
class DeviceGuard {
 public:
  explicit DeviceGuard(int device) {
    cudaGetDevice(&prev_);
    if (prev_ != device) cuda_check(cudaSetDevice(device), "cudaSetDevice");
    restore_ = prev_ != device;
  }
  ~DeviceGuard() {
    if (restore_) cudaSetDevice(prev_);
  }
  DeviceGuard(const DeviceGuard &) = delete;
  DeviceGuard &operator=(const DeviceGuard &) = delete;

 private:
  int prev_ = 0;
  bool restore_ = false;
};

// Owning device allocation.
class DeviceBuffer {
 public:
  DeviceBuffer() = default;
  ~DeviceBuffer();
  DeviceBuffer(const DeviceBuffer &) = delete;
  DeviceBuffer &operator=(const DeviceBuffer &) = delete;
  DeviceBuffer(DeviceBuffer &&o) noexcept : ptr_(o.ptr_), bytes_(o.bytes_) {
    o.ptr_ = nullptr;
    o.bytes_ = 0;
  }
  DeviceBuffer &operator=(DeviceBuffer &&o) noexcept {
    if (this != &o) {
      release();
      ptr_ = o.ptr_;
      bytes_ = o.bytes_;
      o.ptr_ = nullptr;
      o.bytes_ = 0;
    }
    return *this;
  }
  void allocate(size_t bytes);  // zero-filled
  void release();
  void *get() const { return ptr_; }
  size_t bytes() const { return bytes_; }
  template <typename U>
  U *as() const {
    return static_cast<U *>(ptr_);
  }

 private:
  void *ptr_ = nullptr;
  size_t bytes_ = 0;
};

class Batch;

class Model {
  friend class Batch;

 public:
  Model(const Config &cfg, int precision, int device);
  Model(const Model &other);  // deep copy (src/fdModel.cpp:64-97)
  ~Model();

  const Config &config() const { return cfg_; }
  const Geometry &geometry() const { return geo_; }
  int precision() const { return prec_; }
  int device() const { return device_; }
  double misfit() const { return misfit_; }
  size_t device_bytes() const;

  // Simulation (src/fdModel.cpp:526-969, 1128-1183, 1291-1324).
  void forward_simulate(int shot, bool store, bool verbose, bool output_wavefields,
                        int n_steps = -1);
  void adjoint_simulate(int shot, bool verbose);
  double calculate_l2_misfit();
  void calculate_l2_adjoint_sources();
  void reset_kernels();
  void map_kernels_to_velocity();
  void run_model(bool verbose, bool simulate_adjoint);
  void update_from_velocity();
  // Forward time steps of `shot` with CUDA events around every launch;
  // fills the average device time per step and per launch kind (ms).
  int profile_forward(int shot, int n_steps, double *per_step_ms, double *kernel_ms,
                      int max_kernels);

  // Transfers of host FP64 arrays.
  void get_parameter_fields(double *vp, double *vs, double *rho);
  void set_parameter_fields(const double *vp, const double *vs, const double *rho,
                            bool device_pointers);
  void load_model(const std::string &de, const std::string &vp, const std::string &vs,
                  bool verbose);
  void get_kernels(double *vp_k, double *vs_k, double *rho_k, bool device_pointers);
  void get_lame_kernels(double *lam, double *mu, double *rho);
  void get_data(int which, double *ux, double *uz, bool device_pointers);
  void set_data(int which, const double *ux, const double *uz, bool device_pointers);
  void get_snapshots(double *out[5]);
  void get_wavefields(double *out[5]);
  void get_stf(double *out) const;
  void get_moment(double *out) const;
  // Source generalisation: custom wavelets [n_sources][nt] and full 2 x 2
  // moment tensors [n_sources][2][2] for every later simulation.
  void set_stf(const double *stf);
  void set_moment(const double *moment);
  void get_taper(double *out) const;

  void get_model_vector(double *out);
  void set_model_vector(const double *in);
  void get_gradient_vector(double *out);
  void load_vector(const std::string &path, bool verbose, double *out) const;

  void get_sources(bool in_units, bool include_boundary, double *x, double *z) const;
  void get_receivers(bool in_units, bool include_boundary, double *x, double *z) const;
  void get_coordinates(bool in_units, double *ix, double *iz) const;
  void get_extent(bool include_boundary, double *out4) const;

  void write_receivers(const std::string &prefix);
  void load_receivers(bool verbose);
  void write_sources() const;
  void write_kernels();

  // Time-step kernel variant (Variant in psv_solver.hpp); FP64 models only
  // run kTwoKernel.
  void set_variant(int v);
  // Tile shape of the TMA step (tma::TileCfg); autotune() times each shape
  // on a few forward steps of shot 0 and keeps the fastest.
  void set_tile_cfg(int cfg);
  int tile_cfg() const { return tile_cfg_; }
  int autotune(int n_steps);

  // Gradient of the L2 misfit over all shots with respect to (vp, vs, rho)
  // by the exact discrete adjoint (psv_exact.cuh), with the forward states
  // rebuilt from checkpoints taken every `checkpoint_every` steps (>= nt:
  // one segment, every state kept). Returns the misfit; the gradient stays on
  // the device (get_exact_gradient).
  double exact_gradient(int checkpoint_every);
  // The same over the listed shots only (misfit and gradient of those
  // shots): the per-rank part of a shot-sharded gradient.
  double exact_gradient(int checkpoint_every, const std::vector<int> &shots);
  void get_exact_gradient(double *g_vp, double *g_vs, double *g_rho, bool device_pointers);
  size_t exact_bytes(int checkpoint_every) const;
  int variant() const { return variant_; }
  int kernels_per_step() const { return variant_ == kTwoKernel ? 2 : 1; }
  // The FP32 variants built on the TMA step's descriptors (the cluster
  // variant shares them, and the exact adjoint's recompute runs the TMA step).
  bool is_tma() const {
    return variant_ == kFusedTma || variant_ == kFusedTmaPersistent || variant_ == kFusedCluster;
  }
  const char *step_kernel_name(int k) const;

  void set_stream(cudaStream_t s) { user_stream_ = s; }
  cudaStream_t stream() const { return user_stream_ ? user_stream_ : stream_; }
  void set_async(bool a) { async_ = a; }
  void set_graphs(bool on) {
    use_graphs_ = on;
    if (!on) clear_graphs();
  }
  void synchronize();

  enum DataKind { kSynthetic = 0, kObserved = 1, kAdjoint = 2 };

 private:
  void allocate();
  void build_tables();
  void build_plans();
  void ensure_snapshots();
  SolverArgs solver_args();
  void finish(const char *what);
  size_t grid_size() const { return static_cast<size_t>(geo_.nx) * geo_.nz; }
  // Wave-field and medium arrays are stored with rows padded to pitch_ points
  // (a multiple of 4, so every row starts on a 16-byte boundary).
  size_t padded_size() const { return static_cast<size_t>(geo_.nx) * pitch_; }
  size_t data_size() const { return static_cast<size_t>(cfg_.n_shots) * cfg_.nr * cfg_.nt; }
  size_t elem() const { return prec_ == 1 ? sizeof(double) : sizeof(float); }
  void widen(size_t n, const void *src, double *dst_device);
  void dump_wavefields_text(int it);

  Config cfg_;
  Geometry geo_;
  int prec_;
  int device_;
  cudaStream_t stream_ = nullptr;
  cudaStream_t user_stream_ = nullptr;
  bool async_ = false;
  double misfit_ = 0;

  // Host setup tables (src/fdModel.cpp:193-299).
  std::vector<int> ix_src_, iz_src_, ix_rec_, iz_rec_;  // absolute indices
  std::vector<double> stf_;                             // [n_sources][nt]
  std::vector<double> moment_;                          // [n_sources][2][2]
  std::vector<double> taper_tab_;                       // [np + 1]

  int pitch_ = 0;
  int variant_ = kTwoKernel;
  int cluster_nc_ = 0;  // CTAs of the cluster that holds the grid, 0 if none does
  static constexpr double kClusterCells = 1.0e5;  // default cluster-resident up to this size
  int cur_ = 0;  // fused variants: 0 = fields_ hold the current state, 1 = fields2_
  // TMA step: one simulation descriptor per (direction, shot) --
  // [0, n_shots) forward, [n_shots, 2 n_shots) adjoint -- on the host (their
  // tensor maps go out as kernel parameters) and in device memory.
  bool tma_ok_ = false;
  int tile_cfg_ = tma::kTile32x60;
  std::vector<tma::SimDesc> descs_h_;
  void build_descs();
  cudaError_t tma_forward(int shot, bool store, int it0, int it1, bool zero, bool finish,
                          cudaEvent_t *events,
                          bool allow_cluster = true);
  cudaError_t tma_adjoint(int shot);
  void check_device_error();

  // Whole time loops captured as CUDA graphs, keyed by (direction, shot,
  // store, steps). A loop runs eagerly the first time and is captured the
  // second time, then replayed; the graph fixes every launch's arguments, so
  // the cache is dropped whenever a kernel variant changes.
  struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    int uses = 0;
    int cur_after = 0;
  };
  std::map<std::tuple<int, int, int, int>, GraphEntry> graphs_;
  bool use_graphs_ = true;
  void run_loop(int direction, int shot, bool store, int n_steps,
                const std::function<void()> &enqueue);
  void clear_graphs();

  // Device arrays.
  DeviceBuffer fields_[5];                    // vx vz txx tzz txz   (T)
  DeviceBuffer fields2_[5];                   // second set (fused variant)
  DeviceBuffer lm_, la_, mu_, b_;             // medium              (T)
  DeviceBuffer vp_, vs_, rho_;                // medium              (FP64)
  DeviceBuffer taper_tab_d_;                  // (T)
  DeviceBuffer accu_[5];                      // snapshots           (T)
  DeviceBuffer rtf_[2], rtf_true_[2], a_stf_[2];  // data          (FP64)
  DeviceBuffer rec_raw_;                      // [2][nr][nt]         (T)
  DeviceBuffer rec_cell_;                     // [nr] int
  DeviceBuffer rec_start_, rec_order_;        // receivers grouped by cell (exact adjoint)
  DeviceBuffer rec_tile_start_, rec_tile_list_;  // receivers by tile (persistent step)
  DeviceBuffer sched_;                        // persistent step: item counter, tile progress
  int n_rec_groups_ = 0;
  DeviceBuffer stf_d_;                        // [n_sources][nt]     (FP64)
  DeviceBuffer klame_[3];                     // lambda mu rho       (FP64)
  DeviceBuffer kvel_[3];                      // vp vs rho           (FP64)
  DeviceBuffer partials_, scalar_;            // reduction scratch   (FP64)
  DeviceBuffer err_flag_;                     // int, raised by bounded device waits
  // exact adjoint: FP64 gradients wrt (lm, la, mu, b) and (vp, vs, rho),
  // receiver terms, adjoint state (lv x2, lt x3, ot x3), checkpoints, slots
  // Exact adjoint: FP64 gradient sums, outputs, receiver terms, adjoint
  // state planes (lv in/out: 0-1 / 8-9, lt in/out: 2-4 / 5-7), checkpoints
  // and state slots.
  static constexpr int kLamPlanes = 10;
  DeviceBuffer gex_[4], kexact_[3], adj_[2], lam_, ckpt_, slots_;
  DeviceBuffer exrec_start_, exrec_list_;  // receivers by tile of the exact TMA step
  DeviceBuffer gff_[4];  // FP32 exact step: float-float gradient sums (lm, la, mu, b)
  // FP32 exact adjoint with the TMA steps: the shots of a gradient run
  // concurrently in lanes, each lane a stream (lane 0: the model's) with its
  // own checkpoints, state slots, adjoint planes and raw receiver series;
  // shot k of a gradient runs in lane k % lanes. The gradient sums are kept
  // per shot ([n_shots][4][grid] float-float pairs) and added up in shot
  // order at the end, so the result does not depend on the lane count.
  struct ExactLane {
    cudaStream_t stream = nullptr;  // own stream (lanes >= 1)
    cudaEvent_t done = nullptr;
    // part: FP32 partial gradient sums, (lm, mu) pairs then b, padded grid
    DeviceBuffer ckpt, slots, lam, raw, part;
    std::vector<tma::Maps> slot_maps;  // input maps of each state slot
    exact_tma::Maps emaps;             // the exact step's maps over lam, slots, medium
    const void *maps_slots = nullptr;  // slots / lam / C / tile shape the maps were made for
    const void *maps_lam = nullptr;
    int maps_C = -1, maps_cfg = -1;
    tma::Maps rm_maps[2];               // run_model lanes: input maps of slots 0 and 1
    const void *rm_slots = nullptr;
    int rm_cfg = -1;
  };
  // run_model in lanes (FP32, TMA per-step launches): every shot's forward
  // with snapshots, then every shot's adjoint with kernel correlation into
  // per-shot sums (kshots_), added in shot order.
  DeviceBuffer kshots_;
  bool run_model_lanes_ok() const;
  void run_model_lanes(bool simulate_adjoint);
  int ensure_lanes(int K);  // makes exactly K lanes; returns 1 when lanes were (re)made
  std::vector<std::unique_ptr<ExactLane>> lanes_;
  DeviceBuffer gff_shots_;
  cudaEvent_t lanes_start_ = nullptr;
  static constexpr int kMaxLanes = 8;       // run_model lanes
  static constexpr int kMaxExactLanes = 4;  // exact-gradient lanes (measured at c3: 4 lanes
                                            // 1.02 s, 8 lanes 1.04 s, 2 lanes 1.15 s)
  static constexpr int kFlushSteps = 20;  // exact step: partial sums into the pairs
  int exact_lane_count(int C, int n_list) const;
  size_t exact_lane_bytes(int C) const;
  double exact_gradient_lanes(int C, const std::vector<int> &shot_list);
  void destroy_lanes();
  // Injection plans: one per shot (sources) and one for the adjoint receivers.
  std::vector<DeviceBuffer> plan_terms_, plan_maps_;
  std::vector<InjPlan> plans_;  // [n_shots] forward, [n_shots] = adjoint
  static constexpr int kPartials = 1024;
};

}  // namespace psv
