// Batched forward simulation of many (model, shot) members; see psv_batch.hpp.
#include "psv_batch.hpp"

#include <algorithm>
#include <limits>

#include "../../include/psvwave.h"
#include "psv_cluster.hpp"

namespace psv {

Batch::Batch(int device) : device_(device) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    throw Error(PSV_ERR_CUDA, "no CUDA device is available");
  }
  if (device < 0 || device >= count) throw Error(PSV_ERR_INVALID_ARGUMENT, "CUDA device index out of range");
  int prev = 0;
  cudaGetDevice(&prev);
  cuda_check(cudaSetDevice(device_), "cudaSetDevice");
  cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  err_flag_.allocate(sizeof(int));
  cudaSetDevice(prev);
}

Batch::~Batch() {
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(device_);
  clear_graphs();
  if (stream_) {
    cudaStreamSynchronize(stream_);
    cudaStreamDestroy(stream_);
  }
  cudaSetDevice(prev);
}

void Batch::clear_graphs() {
  if (graph_.exec) cudaGraphExecDestroy(graph_.exec);
  graph_ = Graph();
}

void Batch::add(Model *m, int shot) {
  if (!m) throw Error(PSV_ERR_INVALID_ARGUMENT, "model must not be NULL");
  if (m->precision() != PSV_FP32 || !m->tma_ok_)
    throw Error(PSV_ERR_INVALID_ARGUMENT, "batched simulation needs FP32 models with the TMA step");
  if (m->device() != device_) throw Error(PSV_ERR_INVALID_ARGUMENT, "model lives on another device");
  if (shot < 0 || shot >= m->config().n_shots)
    throw Error(PSV_ERR_INVALID_ARGUMENT, "i_shot out of range");
  if (!members_.empty() && m->config().nt != nt_)
    throw Error(PSV_ERR_INVALID_ARGUMENT, "all members of a batch must share nt");
  nt_ = m->config().nt;
  members_.emplace_back(m, shot);
  active_h_.push_back(1);
  built_ = false;
  cluster_nc_ = -1;
  cluster_ = false;
  clear_graphs();
}

bool Batch::cluster_fits() {
  if (cluster_nc_ < 0) {
    std::vector<int> nx, nz, np;
    for (const auto &mb : members_) {
      nx.push_back(mb.first->geometry().nx);
      nz.push_back(mb.first->geometry().nz);
      np.push_back(mb.first->config().np_boundary);
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cuda_check(cudaSetDevice(device_), "cudaSetDevice");
    cluster_nc_ = cluster::plan_batch(nx.data(), nz.data(), np.data(), static_cast<int>(nx.size()),
                                      &cluster_smem_);
    cudaSetDevice(prev);
  }
  return cluster_nc_ > 0;
}

void Batch::set_cluster(bool on) {
  if (on && !cluster_fits())
    throw Error(PSV_ERR_INVALID_ARGUMENT, "a batch member does not fit a thread-block cluster");
  if (on == cluster_) return;
  cluster_ = on;
  clear_graphs();
}

double Batch::cells() const {
  double c = 0;
  for (const auto &mb : members_)
    c += static_cast<double>(mb.first->geometry().nx) * mb.first->geometry().nz;
  return c;
}

void Batch::build() {
  size_t arena = 0, raw = 0;
  raw_off_.clear();
  for (const auto &mb : members_) {
    arena += 10 * mb.first->padded_size();
    raw_off_.push_back(raw);
    raw += 2 * static_cast<size_t>(mb.first->config().nr) * nt_;
  }
  arena_.allocate(arena * sizeof(float));
  raw_.allocate(std::max<size_t>(raw, 1) * sizeof(float));
  std::vector<tma::SimDesc> descs(members_.size());
  std::vector<int4> tiles[tma::kNumTileCfgs];
  std::vector<int> rec_start, rec_list;  // per member: tiles + 1 offsets; receivers
  std::vector<size_t> rec_start_off(members_.size());
  float *next = arena_.as<float>();
  for (size_t k = 0; k < members_.size(); ++k) {
    Model &m = *members_[k].first;
    const int shot = members_[k].second;
    const Config &c = m.config();
    const Geometry &g = m.geometry();
    const size_t gp = m.padded_size();
    tma::SimDesc &d = descs[k];
    for (int s = 0; s < 2; ++s) {
      float *f[5];
      for (int i = 0; i < 5; ++i, next += gp) f[i] = next;
      d.set[s] = fast::Fields{f[0], f[1], f[2], f[3], f[4]};
    }
    d.nx = g.nx;
    d.nz = g.nz;
    d.pitch = m.pitch_;
    d.np = c.np_boundary;
    d.nt = c.nt;
    d.nr = c.nr;
    d.si = c.snapshot_interval;
    d.dt = static_cast<float>(c.dt);
    d.idx = static_cast<float>(1.0 / c.dx);
    d.idz = static_cast<float>(1.0 / c.dz);
    d.dt_d = c.dt;
    d.lm = m.lm_.as<float>();
    d.mu = m.mu_.as<float>();
    d.b = m.b_.as<float>();
    d.taper_tab = m.taper_tab_d_.as<float>();
    for (int f = 0; f < 5; ++f)
      d.accu[f] = m.accu_[f].get() ? m.accu_[f].as<float>() +
                                         static_cast<size_t>(shot) * g.snapshots * m.grid_size()
                                   : nullptr;
    d.rec_cell = m.rec_cell_.as<int>();
    d.rec_vx = c.nr ? raw_.as<float>() + raw_off_[k] : nullptr;
    d.rec_vz = c.nr ? raw_.as<float>() + raw_off_[k] + static_cast<size_t>(c.nr) * nt_ : nullptr;
    d.plan = m.plans_[shot];
    d.stf = m.stf_d_.as<double>();
    if (!tma::make_maps(d, m.mu_.as<float>(), tile_cfg_))
      throw Error(PSV_ERR_CUDA, "tensor-map encoding failed for a batch member");
    int tx, tz;
    tma::tile_dims(tile_cfg_, &tx, &tz);
    d.tile_base = static_cast<int>(tiles[tile_cfg_].size());
    d.tiles_x = (g.nx + tx - 1) / tx;
    d.tiles_z = (g.nz + tz - 1) / tz;
    for (int cfg = 0; cfg < tma::kNumTileCfgs; ++cfg)
      tma::append_tiles(cfg, static_cast<int>(k), g.nx, g.nz, tiles[cfg]);
    // This member's receivers by tile, for the persistent scheme.
    const int nt_m = d.tiles_x * d.tiles_z;
    const size_t s0 = rec_start.size(), l0 = rec_list.size();
    rec_start_off[k] = s0;
    rec_start.resize(s0 + nt_m + 1, 0);
    for (int r = 0; r < c.nr; ++r)
      ++rec_start[s0 + 1 + tma::tile_of(tile_cfg_, g.nz, m.ix_rec_[r], m.iz_rec_[r])];
    for (int t = 0; t < nt_m; ++t) rec_start[s0 + t + 1] += rec_start[s0 + t];
    for (int t = 0; t <= nt_m; ++t) rec_start[s0 + t] += static_cast<int>(l0);
    rec_list.resize(l0 + c.nr);
    std::vector<int> fill(rec_start.begin() + s0, rec_start.begin() + s0 + nt_m);
    for (int r = 0; r < c.nr; ++r)
      rec_list[fill[tma::tile_of(tile_cfg_, g.nz, m.ix_rec_[r], m.iz_rec_[r])]++] = r;
  }
  rec_start_.allocate(std::max<size_t>(rec_start.size(), 1) * sizeof(int));
  rec_list_.allocate(std::max<size_t>(rec_list.size(), 1) * sizeof(int));
  if (!rec_start.empty())
    cuda_check(cudaMemcpy(rec_start_.get(), rec_start.data(), rec_start.size() * sizeof(int),
                          cudaMemcpyHostToDevice),
               "upload batch receiver tiles");
  if (!rec_list.empty())
    cuda_check(cudaMemcpy(rec_list_.get(), rec_list.data(), rec_list.size() * sizeof(int),
                          cudaMemcpyHostToDevice),
               "upload batch receiver tiles");
  for (size_t k = 0; k < members_.size(); ++k) {
    descs[k].rec_start = rec_start_.as<int>() + rec_start_off[k];
    descs[k].rec_list = rec_list_.as<int>();
  }
  sched_.allocate(tma::sched_words_batch(static_cast<int>(tiles[tile_cfg_].size())) *
                  sizeof(unsigned));
  active_.allocate(members_.size() * sizeof(int));
  descs_d_.allocate(descs.size() * sizeof(tma::SimDesc));
  cuda_check(cudaMemcpy(descs_d_.get(), descs.data(), descs.size() * sizeof(tma::SimDesc),
                        cudaMemcpyHostToDevice),
             "upload batch descriptors");
  for (int cfg = 0; cfg < tma::kNumTileCfgs; ++cfg) {
    n_tiles_[cfg] = static_cast<int>(tiles[cfg].size());
    tiles_d_[cfg].allocate(tiles[cfg].size() * sizeof(int4));
    cuda_check(cudaMemcpy(tiles_d_[cfg].get(), tiles[cfg].data(), tiles[cfg].size() * sizeof(int4),
                          cudaMemcpyHostToDevice),
               "upload batch tiles");
  }
  built_ = true;
}

void Batch::set_tile_cfg(int cfg) {
  if (cfg < 0 || cfg >= tma::kNumTileCfgs) throw Error(PSV_ERR_INVALID_ARGUMENT, "unknown tile shape");
  if (cfg == tile_cfg_) return;
  clear_graphs();
  tile_cfg_ = cfg;
  built_ = false;  // the descriptors' tensor maps depend on the tile shape
}

void Batch::set_persistent(bool on) {
  if (on == persistent_ && !cluster_) return;
  persistent_ = on;
  cluster_ = false;
  clear_graphs();
}

void Batch::set_active(const int *flags, int n) {
  if (n != size()) throw Error(PSV_ERR_INVALID_ARGUMENT, "one flag per batch member is needed");
  for (int k = 0; k < n; ++k) active_h_[k] = flags ? (flags[k] != 0) : 1;
}

void Batch::synchronize() { cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize"); }

void Batch::forward(bool store, int n_steps) {
  if (members_.empty()) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cuda_check(cudaSetDevice(device_), "cudaSetDevice");
  struct Restore {
    int dev;
    ~Restore() { cudaSetDevice(dev); }
  } restore{prev};
  if (store) {
    bool missing = false;
    for (auto &mb : members_)
      if (!mb.first->accu_[0].get()) {
        mb.first->ensure_snapshots();
        missing = true;
      }
    if (missing) {
      built_ = false;
      clear_graphs();
    }
  }
  // Members' own streams may still be updating their media.
  for (auto &mb : members_) mb.first->synchronize();
  if (!built_) build();
  // The flags live in device memory that the (captured) step launches read.
  cuda_check(cudaMemcpyAsync(active_.get(), active_h_.data(), active_h_.size() * sizeof(int),
                             cudaMemcpyHostToDevice, stream_),
             "batch active flags");
  const int steps = (n_steps <= 0 || n_steps > nt_) ? nt_ : n_steps;
  const int cfg = tile_cfg_;
  auto enqueue = [&]() {
    cuda_check(cudaMemsetAsync(arena_.get(), 0, arena_.bytes(), stream_), "batch zero");
    if (cluster_) {
      cuda_check(cluster::steps_batch(descs_d_.as<tma::SimDesc>(), active_.as<int>(), size(),
                                      cluster_nc_, cluster_smem_, steps, store, stream_),
                 "batch cluster steps");
    } else if (persistent_) {
      cuda_check(cudaMemsetAsync(sched_.get(), 0, sched_.bytes(), stream_), "batch schedule");
      cuda_check(tma::steps_persistent_batch(descs_d_.as<tma::SimDesc>(),
                                             tiles_d_[cfg].as<int4>(), n_tiles_[cfg],
                                             active_.as<int>(), cfg, steps, store,
                                             err_flag_.as<int>(), sched_.as<unsigned>(), stream_),
                 "batch steps");
    } else {
      int parity = 0;
      for (int it = 0; it < steps; ++it) {
        cuda_check(tma::step(descs_d_.as<tma::SimDesc>(), tiles_d_[cfg].as<int4>(),
                             n_tiles_[cfg], active_.as<int>(), cfg, false, it, parity, store,
                             err_flag_.as<int>(), stream_),
                   "batch step");
        parity ^= 1;
      }
    }
    for (size_t k = 0; k < members_.size(); ++k) {
      Model &m = *members_[k].first;
      const Config &c = m.config();
      if (!c.nr) continue;
      const size_t off = static_cast<size_t>(members_[k].second) * c.nr * c.nt;
      const float *raw = raw_.as<float>() + raw_off_[k];
      cuda_check(receiver_cumsum_f32(c.nr, c.nt, steps, c.dt, c.dx * c.dz, raw,
                                     raw + static_cast<size_t>(c.nr) * nt_,
                                     m.rtf_[0].as<double>() + off, m.rtf_[1].as<double>() + off,
                                     stream_, active_.as<int>(), static_cast<int>(k)),
                 "batch seismograms");
    }
  };
  if (graph_.exec && graph_.store == store && graph_.steps == steps) {
    cuda_check(cudaGraphLaunch(graph_.exec, stream_), "cudaGraphLaunch");
  } else if (graph_.uses == 0 || graph_.store != store || graph_.steps != steps) {
    clear_graphs();
    graph_.uses = 1;
    graph_.store = store;
    graph_.steps = steps;
    enqueue();
  } else {
    cuda_check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal),
               "cudaStreamBeginCapture");
    try {
      enqueue();
    } catch (...) {
      cudaGraph_t broken = nullptr;
      cudaStreamEndCapture(stream_, &broken);
      if (broken) cudaGraphDestroy(broken);
      throw;
    }
    cudaGraph_t graph = nullptr;
    cuda_check(cudaStreamEndCapture(stream_, &graph), "cudaStreamEndCapture");
    cudaError_t e = cudaGraphInstantiate(&graph_.exec, graph, 0);
    cudaGraphDestroy(graph);
    cuda_check(e, "cudaGraphInstantiate");
    cuda_check(cudaGraphLaunch(graph_.exec, stream_), "cudaGraphLaunch");
  }
  synchronize();
  int flag = 0;
  cuda_check(cudaMemcpy(&flag, err_flag_.get(), sizeof(int), cudaMemcpyDeviceToHost), "error flag");
  if (flag) {
    cudaMemset(err_flag_.get(), 0, sizeof(int));
    throw Error(PSV_ERR_CUDA, "a CTA timed out waiting for its TMA tile copies");
  }
}

void Batch::misfits(double *out, int n) {
  if (n != size()) throw Error(PSV_ERR_INVALID_ARGUMENT, "expected one value per member");
  if (members_.empty()) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cuda_check(cudaSetDevice(device_), "cudaSetDevice");
  struct Restore {
    int dev;
    ~Restore() { cudaSetDevice(dev); }
  } restore{prev};
  if (misfit_d_.bytes() < static_cast<size_t>(n) * sizeof(double))
    misfit_d_.allocate(static_cast<size_t>(n) * sizeof(double));
  auto active = [&](int k) {
    return k >= static_cast<int>(active_h_.size()) || active_h_[k] != 0;
  };
  for (int k = 0; k < n; ++k) {
    if (!active(k)) continue;
    Model &m = *members_[k].first;
    // The same reduction as Model::calculate_l2_misfit, into slot k.
    const size_t nd = m.data_size();
    int parts = static_cast<int>(std::min<size_t>(Model::kPartials, (nd + 255) / 256));
    if (parts < 1) parts = 1;
    cuda_check(misfit_l2(nd, m.cfg_.dt, m.rtf_true_[0].as<double>(), m.rtf_[0].as<double>(),
                         m.rtf_true_[1].as<double>(), m.rtf_[1].as<double>(),
                         m.partials_.as<double>(), parts, misfit_d_.as<double>() + k, stream_),
               "batch misfits");
  }
  std::vector<double> v(n);
  cuda_check(cudaMemcpyAsync(v.data(), misfit_d_.get(), static_cast<size_t>(n) * sizeof(double),
                             cudaMemcpyDeviceToHost, stream_),
             "batch misfits copy");
  synchronize();
  for (int k = 0; k < n; ++k) {
    if (active(k)) {
      out[k] = v[k];
      members_[k].first->misfit_ = v[k];
    } else {
      out[k] = std::numeric_limits<double>::quiet_NaN();
    }
  }
}

void Batch::set_parameter_fields_device(const double *fields, size_t member_stride,
                                        const int *flags) {
  if (!fields) throw Error(PSV_ERR_INVALID_ARGUMENT, "fields must not be NULL");
  std::vector<const Model *> done;
  for (size_t k = 0; k < members_.size(); ++k) {
    if (flags && !flags[k]) continue;
    Model *m = members_[k].first;
    if (std::find(done.begin(), done.end(), m) != done.end()) continue;
    done.push_back(m);
    const size_t g = m->grid_size();
    if (member_stride < 3 * g)
      throw Error(PSV_ERR_INVALID_ARGUMENT, "member stride shorter than a member's fields");
    const double *p = fields + k * member_stride;
    m->set_parameter_fields(p, p + g, p + 2 * g, true);
  }
}

int Batch::autotune(int n_steps) {
  if (members_.empty()) return tile_cfg_;
  // Every (launch scheme, tile shape) pair on n_steps steps of the members
  // currently active, each timed on its third run (after the build and the
  // graph capture), and the cluster-resident scheme when the members fit;
  // the fastest is kept.
  float best = 0;
  int best_cfg = tile_cfg_;
  bool best_persistent = persistent_, first = true;
  cudaEvent_t a, b;
  cuda_check(cudaEventCreate(&a), "cudaEventCreate");
  cuda_check(cudaEventCreate(&b), "cudaEventCreate");
  for (bool p : {false, true}) {
    for (int cfg = 0; cfg < tma::kNumTileCfgs; ++cfg) {
      set_persistent(p);
      set_tile_cfg(cfg);
      forward(false, n_steps);  // eager run (also builds)
      forward(false, n_steps);  // graph capture
      cudaEventRecord(a, stream_);
      forward(false, n_steps);
      cudaEventRecord(b, stream_);
      cudaEventSynchronize(b);
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      if (first || ms < best) {
        best = ms;
        best_cfg = cfg;
        best_persistent = p;
        first = false;
      }
    }
  }
  bool best_cluster = false;
  if (cluster_fits()) {
    set_cluster(true);
    forward(false, n_steps);
    forward(false, n_steps);
    cudaEventRecord(a, stream_);
    forward(false, n_steps);
    cudaEventRecord(b, stream_);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best) best_cluster = true;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  set_persistent(best_persistent);
  set_tile_cfg(best_cfg);
  if (best_cluster) set_cluster(true);
  return best_cfg;
}

}  // namespace psv
