// Many simulations -- shots of many models, of uneven grid sizes -- advanced
// together: one TMA-step launch per time step covers the tiles of every
// simulation, and the whole time loop is replayed as one CUDA graph. No
// counterpart in the reference, which runs one shot of one model at a time
// (src/fdModel.cpp:1293-1296).
#pragma once

#include <cuda_runtime.h>

#include <utility>
#include <vector>

#include "psv_model.hpp"
#include "psv_tma.hpp"

namespace psv {

class Batch {
 public:
  explicit Batch(int device);
  ~Batch();
  Batch(const Batch &) = delete;
  Batch &operator=(const Batch &) = delete;

  // Adds shot `shot` of `model` (FP32, TMA step). All models of a batch share
  // nt. The models must outlive the batch.
  void add(Model *model, int shot);
  // Forward simulation of every member over its first n_steps time steps (all
  // steps if n_steps <= 0). Seismograms land in each model's synthetic data of
  // that shot; with store_fields, snapshots land in each model's snapshots.
  void forward(bool store_fields, int n_steps);
  // Times every tile shape on n_steps steps and keeps the fastest.
  int autotune(int n_steps);
  void set_tile_cfg(int cfg);
  // Which members the next forward() advances (non-zero = advance); all of
  // them by default. The others keep their previous seismograms.
  void set_active(const int *flags, int n);
  // L2 misfit of every active member's model (what calculate_l2_misfit
  // returns, bit for bit; n == size()), one reduction per member on the
  // batch's stream and one copy back; inactive members get NaN. Each active
  // model's misfit is updated as calculate_l2_misfit would.
  void misfits(double *out, int n);
  // set_parameter_fields from device arrays for every member flagged
  // non-zero in `flags` (all when null): member k's vp, vs and rho
  // ([nx][nz] each, consecutive) start at fields + k * member_stride. A
  // model that is a member more than once is set once. Each model queues
  // its copies and medium update on its own stream as its own call does.
  void set_parameter_fields_device(const double *fields, size_t member_stride, const int *flags);
  // Launch scheme: one launch per time step (false, the default) or every
  // step in one persistent launch over the tile table (true). A batch step
  // holds tens of thousands of tiles, many waves with no tail to recover,
  // so the per-item scheduling of the persistent scheme is measured slower.
  void set_persistent(bool on);
  bool persistent() const { return persistent_; }
  // Cluster-resident scheme: every member in its own thread-block cluster
  // that holds its whole grid in shared memory for every step, all members
  // in one launch (members must fit: cluster_fits()). Takes precedence over
  // the tile schemes while on; set_persistent() switches it off. Results
  // equal each model's own cluster-resident run (variant fused_cluster) bit
  // for bit.
  bool cluster_fits();
  void set_cluster(bool on);
  bool cluster() const { return cluster_; }
  int tile_cfg() const { return tile_cfg_; }
  int size() const { return static_cast<int>(members_.size()); }
  double cells() const;  // grid points summed over members
  int tiles() const { return n_tiles_[tile_cfg_]; }
  void synchronize();

 private:
  void build();
  void clear_graphs();

  int device_;
  cudaStream_t stream_ = nullptr;
  std::vector<std::pair<Model *, int>> members_;
  bool built_ = false;
  int nt_ = 0;
  int tile_cfg_ = tma::kTile16x28;
  DeviceBuffer arena_;   // wave-field buffer sets of every member
  DeviceBuffer raw_;     // receiver raw velocities of every member
  DeviceBuffer descs_d_;
  DeviceBuffer tiles_d_[tma::kNumTileCfgs];
  int n_tiles_[tma::kNumTileCfgs] = {};
  DeviceBuffer err_flag_;
  DeviceBuffer active_;              // per member flag, read by the step kernel
  DeviceBuffer misfit_d_;            // per member misfit (misfits())
  std::vector<int> active_h_;
  bool persistent_ = false;
  bool cluster_ = false;
  int cluster_nc_ = -1;      // -1: not planned yet; 0: the members do not fit
  size_t cluster_smem_ = 0;
  DeviceBuffer sched_;               // persistent scheme: item counter, tile progress
  DeviceBuffer rec_start_, rec_list_;  // receivers by member tile (persistent scheme)
  std::vector<size_t> raw_off_;  // per member, floats into raw_
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    int uses = 0;
    bool store = false;
    int steps = 0;
  } graph_;
};

}  // namespace psv
