// Host orchestration of one P-SV model: setup tables, device memory, the
// calls of the reference's fdModel API (src/fdModel.cpp), and text I/O.
#include "psv_model.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <sstream>

#include "../../include/psvwave.h"
#include "psv_cluster.hpp"
#include "psv_exact_tma.hpp"
#include "psv_fast.hpp"

namespace psv {

namespace {

// The reference's degrees-to-radians constant (src/fdModel.cpp:14) and the
// M_PI its Ricker wavelet uses (src/fdModel.cpp:227).
constexpr double kRefPi = 3.14159265;
constexpr double kMPi = 3.14159265358979323846;

std::string pad5(int n) {
  std::ostringstream ss;
  ss << std::setw(5) << std::setfill('0') << n;
  return ss.str();
}

}  // namespace

void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(PSV_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

DeviceBuffer::~DeviceBuffer() { release(); }

void DeviceBuffer::allocate(size_t bytes) {
  release();
  if (bytes == 0) bytes = 16;
  cuda_check(cudaMalloc(&ptr_, bytes), "cudaMalloc");
  bytes_ = bytes;
  cuda_check(cudaMemset(ptr_, 0, bytes), "cudaMemset");
}

void DeviceBuffer::release() {
  if (ptr_) cudaFree(ptr_);
  ptr_ = nullptr;
  bytes_ = 0;
}

// ---------------------------------------------------------------- setup --

Model::Model(const Config &cfg, int precision, int device)
    : cfg_(cfg), geo_(validate(cfg)), prec_(precision), device_(device) {
  if (prec_ != PSV_FP32 && prec_ != PSV_FP64)
    throw Error(PSV_ERR_INVALID_ARGUMENT, "precision must be PSV_FP32 or PSV_FP64");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    throw Error(PSV_ERR_CUDA, "no CUDA device is available");
  }
  if (device_ < 0 || device_ >= count)
    throw Error(PSV_ERR_INVALID_ARGUMENT, "CUDA device index out of range");
  DeviceGuard guard(device_);
  cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  variant_ = prec_ == PSV_FP32 ? kFused : kTwoKernel;
  pitch_ = (geo_.nz + 3) / 4 * 4;
  build_tables();
  allocate();
  // Homogeneous background medium (src/fdModel.cpp:249-261).
  std::vector<double> v(grid_size());
  const double scal[3] = {cfg_.scalar_vp, cfg_.scalar_vs, cfg_.scalar_rho};
  DeviceBuffer *dst[3] = {&vp_, &vs_, &rho_};
  for (int k = 0; k < 3; ++k) {
    std::fill(v.begin(), v.end(), scal[k]);
    cuda_check(cudaMemcpy(dst[k]->get(), v.data(), v.size() * sizeof(double),
                          cudaMemcpyHostToDevice),
               "upload medium");
  }
  update_from_velocity();
  build_plans();
  // Tile shape. Grids with at least a full wave of 32 x 60 tiles keep them
  // (and run persistent, below); smaller ones take 16 x 28 tiles. At
  // 1100 x 500: 32 x 60 tiles (315, against 456 resident) 12.0 us per step,
  // 16 x 28 (1242) 8.9 us, 20 x 28 (990, one wave of 1216 resident) 9.3 us.
  // autotune() times every shape.
  if (prec_ == PSV_FP32) {
    const int big_slots = tma::resident_ctas(tma::kTile32x60, false);
    if (big_slots > 0 ? tma::tile_count(tma::kTile32x60, geo_.nx, geo_.nz) < big_slots
                      : static_cast<double>(geo_.nx) * geo_.nz < 4.0e5)
      tile_cfg_ = tma::kTile16x28;
  }
  build_descs();
  if (tma_ok_) {
    // One launch per step, or the persistent launch when a step has at least
    // a full wave of 32 x 60 tiles (measured faster there; smaller grids are
    // latency-bound and keep the per-step launches). autotune() times both.
    variant_ = kFusedTma;
    const int slots = tma::resident_ctas(tile_cfg_, false);
    if (tile_cfg_ == tma::kTile32x60 && slots > 0 &&
        tma::tile_count(tile_cfg_, geo_.nx, geo_.nz) >= slots)
      variant_ = kFusedTmaPersistent;
    // Grids that one thread-block cluster holds in shared memory run
    // cluster-resident (up to kClusterCells points).
    if (cluster_nc_ > 0 && static_cast<double>(geo_.nx) * geo_.nz <= kClusterCells)
      variant_ = kFusedCluster;
  }
  synchronize();
}

Model::Model(const Model &o)
    : cfg_(o.cfg_), geo_(o.geo_), prec_(o.prec_), device_(o.device_), async_(o.async_),
      misfit_(o.misfit_), pitch_(o.pitch_), variant_(o.variant_), cur_(o.cur_) {
  DeviceGuard guard(device_);
  cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  tile_cfg_ = o.tile_cfg_;
  build_tables();
  allocate();
  build_plans();
  const_cast<Model &>(o).synchronize();
  auto copy = [&](DeviceBuffer &d, const DeviceBuffer &s) {
    if (!s.get()) return;
    if (d.bytes() != s.bytes()) d.allocate(s.bytes());
    cuda_check(cudaMemcpy(d.get(), s.get(), s.bytes(), cudaMemcpyDeviceToDevice), "clone");
  };
  for (int k = 0; k < 5; ++k) copy(fields_[k], o.fields_[k]);
  for (int k = 0; k < 5; ++k) copy(fields2_[k], o.fields2_[k]);
  copy(lm_, o.lm_);
  copy(la_, o.la_);
  copy(mu_, o.mu_);
  copy(b_, o.b_);
  copy(vp_, o.vp_);
  copy(vs_, o.vs_);
  copy(rho_, o.rho_);
  for (int k = 0; k < 5; ++k) copy(accu_[k], o.accu_[k]);
  for (int k = 0; k < 2; ++k) {
    copy(rtf_[k], o.rtf_[k]);
    copy(rtf_true_[k], o.rtf_true_[k]);
    copy(a_stf_[k], o.a_stf_[k]);
  }
  copy(rec_raw_, o.rec_raw_);
  for (int k = 0; k < 3; ++k) {
    copy(klame_[k], o.klame_[k]);
    copy(kvel_[k], o.kvel_[k]);
  }
  build_descs();
}

Model::~Model() {
  DeviceGuard guard(device_);
  clear_graphs();
  destroy_lanes();
  if (stream_) {
    cudaStreamSynchronize(stream_);
    cudaStreamDestroy(stream_);
  }
}

void Model::build_tables() {
  const int np = cfg_.np_boundary;
  // Source/receiver positions in the padded grid (src/fdModel.cpp:197-212).
  ix_src_.clear();
  iz_src_.clear();
  ix_rec_.clear();
  iz_rec_.clear();
  for (int i = 0; i < cfg_.n_sources; ++i) {
    ix_src_.push_back(cfg_.ix_sources[i] + np);
    iz_src_.push_back(cfg_.iz_sources[i] + np);
  }
  for (int i = 0; i < cfg_.nr; ++i) {
    ix_rec_.push_back(cfg_.ix_receivers[i] + np);
    iz_rec_.push_back(cfg_.iz_receivers[i] + np);
  }
  // Ricker wavelets, each delayed by delay_cycles_per_shot periods per
  // position in its shot (src/fdModel.cpp:215-231).
  const int nt = cfg_.nt;
  stf_.assign(static_cast<size_t>(cfg_.n_sources) * nt, 0.0);
  for (const auto &shot : cfg_.shots) {
    for (size_t pos = 0; pos < shot.size(); ++pos) {
      const int src = shot[pos];
      for (int it = 0; it < nt; ++it) {
        const double t = static_cast<double>(static_cast<unsigned>(it)) * cfg_.dt;
        const double f = 1.0 / geo_.alpha;
        const double shifted =
            t - 1.4 / f - cfg_.delay_cycles_per_shot * static_cast<int>(pos) / f;
        const double a = kMPi * f * shifted;
        stf_[static_cast<size_t>(src) * nt + it] = (1 - 2 * (a * a)) * std::exp(-(a * a));
      }
    }
  }
  // Moment tensors of reverse faults rotated by their dip (src/fdModel.cpp:234-246).
  moment_.assign(static_cast<size_t>(cfg_.n_sources) * 4, 0.0);
  for (int i = 0; i < cfg_.n_sources; ++i) {
    const double r = cfg_.moment_angles[i] * kRefPi / 180.0;
    moment_[4 * i + 0] = std::cos(r) * 1e15;
    moment_[4 * i + 1] = -std::sin(r) * 1e15;
    moment_[4 * i + 2] = -std::sin(r) * 1e15;
    moment_[4 * i + 3] = -std::cos(r) * 1e15;
  }
  // Cerjan taper as a function of the nested-frame count c in [0, np]
  // (src/fdModel.cpp:263-298): exp(-(np_factor (np - c))^2).
  taper_tab_.assign(static_cast<size_t>(np) + 1, 1.0);
  for (int c = 0; c <= np; ++c) {
    const double a = cfg_.np_factor * (static_cast<double>(np) - static_cast<double>(c));
    taper_tab_[c] = std::exp(-(a * a));
  }
}

void Model::allocate() {
  const size_t g = grid_size(), gp = padded_size(), e = elem(), d = data_size();
  for (auto &f : fields_) f.allocate(gp * e);
  if (prec_ == PSV_FP32)
    for (auto &f : fields2_) f.allocate(gp * e);
  lm_.allocate(gp * e);
  la_.allocate(gp * e);
  mu_.allocate(gp * e);
  b_.allocate(gp * e);
  vp_.allocate(g * sizeof(double));
  vs_.allocate(g * sizeof(double));
  rho_.allocate(g * sizeof(double));
  for (int k = 0; k < 2; ++k) {
    rtf_[k].allocate(d * sizeof(double));
    rtf_true_[k].allocate(d * sizeof(double));
    a_stf_[k].allocate(d * sizeof(double));
  }
  rec_raw_.allocate(2 * static_cast<size_t>(cfg_.nr) * cfg_.nt * e);
  rec_cell_.allocate(static_cast<size_t>(cfg_.nr) * sizeof(int));
  for (auto &k : klame_) k.allocate(g * sizeof(double));
  for (auto &k : kvel_) k.allocate(g * sizeof(double));
  partials_.allocate(kPartials * sizeof(double));
  err_flag_.allocate(sizeof(int));
  scalar_.allocate(sizeof(double));
  stf_d_.allocate(stf_.size() * sizeof(double));
  if (!stf_.empty())
    cuda_check(cudaMemcpy(stf_d_.get(), stf_.data(), stf_.size() * sizeof(double),
                          cudaMemcpyHostToDevice),
               "upload stf");
  std::vector<int> cells(cfg_.nr);
  for (int r = 0; r < cfg_.nr; ++r) cells[r] = ix_rec_[r] * pitch_ + iz_rec_[r];
  if (cfg_.nr)
    cuda_check(cudaMemcpy(rec_cell_.get(), cells.data(), cells.size() * sizeof(int),
                          cudaMemcpyHostToDevice),
               "upload receivers");
  {
    // Receivers grouped by cell, groups in order of first appearance and
    // receivers in increasing index within a group.
    std::vector<int> start, order;
    std::vector<char> done(cfg_.nr, 0);
    for (int r = 0; r < cfg_.nr; ++r) {
      if (done[r]) continue;
      start.push_back(static_cast<int>(order.size()));
      for (int q = r; q < cfg_.nr; ++q)
        if (!done[q] && cells[q] == cells[r]) {
          order.push_back(q);
          done[q] = 1;
        }
    }
    n_rec_groups_ = static_cast<int>(start.size());
    start.push_back(static_cast<int>(order.size()));
    rec_start_.allocate(start.size() * sizeof(int));
    rec_order_.allocate(std::max<size_t>(order.size(), 1) * sizeof(int));
    cuda_check(cudaMemcpy(rec_start_.get(), start.data(), start.size() * sizeof(int),
                          cudaMemcpyHostToDevice),
               "upload receiver groups");
    if (!order.empty())
      cuda_check(cudaMemcpy(rec_order_.get(), order.data(), order.size() * sizeof(int),
                            cudaMemcpyHostToDevice),
                 "upload receiver groups");
  }
  {
    // Receivers by tile of the exact adjoint's TMA step, increasing index
    // within a tile.
    const int n_tiles = exact_tma::tile_count(geo_.nx, geo_.nz);
    std::vector<int> start(n_tiles + 1, 0), list(std::max(cfg_.nr, 1));
    for (int r = 0; r < cfg_.nr; ++r) ++start[1 + exact_tma::tile_of(geo_.nz, ix_rec_[r], iz_rec_[r])];
    for (int t = 0; t < n_tiles; ++t) start[t + 1] += start[t];
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int r = 0; r < cfg_.nr; ++r) list[fill[exact_tma::tile_of(geo_.nz, ix_rec_[r], iz_rec_[r])]++] = r;
    exrec_start_.allocate(start.size() * sizeof(int));
    exrec_list_.allocate(list.size() * sizeof(int));
    cuda_check(cudaMemcpy(exrec_start_.get(), start.data(), start.size() * sizeof(int),
                          cudaMemcpyHostToDevice),
               "upload receiver tiles");
    cuda_check(cudaMemcpy(exrec_list_.get(), list.data(), list.size() * sizeof(int),
                          cudaMemcpyHostToDevice),
               "upload receiver tiles");
  }
  taper_tab_d_.allocate(taper_tab_.size() * e);
  if (prec_ == PSV_FP64) {
    cuda_check(cudaMemcpy(taper_tab_d_.get(), taper_tab_.data(),
                          taper_tab_.size() * sizeof(double), cudaMemcpyHostToDevice),
               "upload taper");
  } else {
    std::vector<float> t(taper_tab_.begin(), taper_tab_.end());
    cuda_check(cudaMemcpy(taper_tab_d_.get(), t.data(), t.size() * sizeof(float),
                          cudaMemcpyHostToDevice),
               "upload taper");
  }
}

// Injection terms in the reference's serial order, grouped by point.
void Model::build_plans() {
  const int nz = geo_.nz, n_shots = cfg_.n_shots;
  const double dx = cfg_.dx, dz = cfg_.dz;
  const double dx4 = dx * dx * dx * dx, dz4 = dz * dz * dz * dz;
  plans_.assign(n_shots + 1, InjPlan());
  plan_terms_.clear();
  plan_maps_.clear();
  plan_terms_.resize(n_shots + 1);
  plan_maps_.resize(n_shots + 1);
  for (int p = 0; p <= n_shots; ++p) {
    std::vector<InjTerm> terms;
    auto add = [&](int cell, int field, int index, int kind, double coef, double div) {
      terms.push_back(InjTerm{cell, field, index, kind, coef, div});
    };
    if (p < n_shots) {
      // src/fdModel.cpp:681-751
      for (int s : cfg_.shots[p]) {
        const int c = ix_src_[s] * nz + iz_src_[s];
        const double *M = &moment_[4 * s];
        const double q01 = 0.25 * M[1], q10 = 0.25 * M[2];
        add(c - nz, 0, s, 0, -M[0], dx4);
        add(c, 0, s, 0, M[0], dx4);
        add(c - 1, 1, s, 0, -M[3], dz4);
        add(c, 1, s, 0, M[3], dz4);
        add(c - nz + 1, 0, s, 0, q01, dx4);
        add(c + 1, 0, s, 0, q01, dx4);
        add(c - nz - 1, 0, s, 0, -q01, dx4);
        add(c - 1, 0, s, 0, -q01, dx4);
        add(c + nz - 1, 1, s, 0, q10, dz4);
        add(c + nz, 1, s, 0, q10, dz4);
        add(c - nz - 1, 1, s, 0, -q10, dz4);
        add(c - nz, 1, s, 0, -q10, dz4);
      }
    } else {
      // src/fdModel.cpp:951-958
      for (int r = 0; r < cfg_.nr; ++r) {
        const int c = ix_rec_[r] * nz + iz_rec_[r];
        add(c, 0, r, 1, 0.0, dx * dz);
        add(c, 1, r, 1, 0.0, dx * dz);
      }
    }
    std::stable_sort(terms.begin(), terms.end(),
                     [](const InjTerm &a, const InjTerm &b) { return a.cell < b.cell; });
    InjPlan plan;
    plan.n = static_cast<int>(terms.size());
    if (plan.n) {
      int x0 = geo_.nx, x1 = -1, z0 = nz, z1 = -1;
      for (const auto &t : terms) {
        x0 = std::min(x0, t.cell / nz);
        x1 = std::max(x1, t.cell / nz);
        z0 = std::min(z0, t.cell % nz);
        z1 = std::max(z1, t.cell % nz);
      }
      plan.x0 = x0;
      plan.z0 = z0;
      plan.w = x1 - x0 + 1;
      plan.h = z1 - z0 + 1;
      std::vector<int> map(static_cast<size_t>(plan.w) * plan.h, -1);
      for (int k = plan.n - 1; k >= 0; --k) {
        const int cx = terms[k].cell / nz - x0, cz = terms[k].cell % nz - z0;
        map[static_cast<size_t>(cx) * plan.h + cz] = k;
      }
      plan_terms_[p].allocate(terms.size() * sizeof(InjTerm));
      plan_maps_[p].allocate(map.size() * sizeof(int));
      cuda_check(cudaMemcpy(plan_terms_[p].get(), terms.data(), terms.size() * sizeof(InjTerm),
                            cudaMemcpyHostToDevice),
                 "upload injection terms");
      cuda_check(cudaMemcpy(plan_maps_[p].get(), map.data(), map.size() * sizeof(int),
                            cudaMemcpyHostToDevice),
                 "upload injection map");
      plan.terms = plan_terms_[p].as<InjTerm>();
      plan.map = plan_maps_[p].as<int>();
    }
    plans_[p] = plan;
  }
}

void Model::build_descs() {
  tma_ok_ = false;
  if (prec_ != PSV_FP32 || !tma::supported(geo_.nx, geo_.nz, pitch_)) return;
  const int n_shots = cfg_.n_shots;
  const size_t gsz = grid_size();
  std::vector<tma::SimDesc> descs(static_cast<size_t>(2 * std::max(n_shots, 1)));
  for (int k = 0; k < 2 * n_shots; ++k) {
    const bool adjoint = k >= n_shots;
    const int shot = adjoint ? k - n_shots : k;
    tma::SimDesc &d = descs[k];
    d.set[0] = fast::Fields{fields_[0].as<float>(), fields_[1].as<float>(), fields_[2].as<float>(),
                            fields_[3].as<float>(), fields_[4].as<float>()};
    d.set[1] = fast::Fields{fields2_[0].as<float>(), fields2_[1].as<float>(),
                            fields2_[2].as<float>(), fields2_[3].as<float>(),
                            fields2_[4].as<float>()};
    d.nx = geo_.nx;
    d.nz = geo_.nz;
    d.pitch = pitch_;
    d.np = cfg_.np_boundary;
    d.nt = cfg_.nt;
    d.nr = cfg_.nr;
    d.si = cfg_.snapshot_interval;
    d.dt = static_cast<float>(cfg_.dt);
    d.idx = static_cast<float>(1.0 / cfg_.dx);
    d.idz = static_cast<float>(1.0 / cfg_.dz);
    d.dt_d = cfg_.dt;
    d.lm = lm_.as<float>();
    d.mu = mu_.as<float>();
    d.b = b_.as<float>();
    d.taper_tab = taper_tab_d_.as<float>();
    for (int f = 0; f < 5; ++f)
      d.accu[f] = accu_[f].get()
                      ? accu_[f].as<float>() + static_cast<size_t>(shot) * geo_.snapshots * gsz
                      : nullptr;
    d.krho = klame_[2].as<double>();
    d.klam = klame_[0].as<double>();
    d.kmu = klame_[1].as<double>();
    d.sidt = cfg_.snapshot_interval * cfg_.dt;
    d.fx0 = geo_.fx0;
    d.fx1 = geo_.fx1;
    d.fz0 = geo_.fz0;
    d.fz1 = geo_.fz1;
    d.rec_cell = rec_cell_.as<int>();
    d.rec_vx = cfg_.nr ? rec_raw_.as<float>() : nullptr;
    d.rec_vz = cfg_.nr ? rec_raw_.as<float>() + static_cast<size_t>(cfg_.nr) * cfg_.nt : nullptr;
    if (!adjoint) {
      d.plan = plans_[shot];
      d.stf = stf_d_.as<double>();
    } else {
      d.plan = plans_[n_shots];
      d.a_ux = a_stf_[0].as<double>() + static_cast<size_t>(shot) * cfg_.nr * cfg_.nt;
      d.a_uz = a_stf_[1].as<double>() + static_cast<size_t>(shot) * cfg_.nr * cfg_.nt;
    }
    if (!tma::make_maps(d, mu_.as<float>(), tile_cfg_)) return;
  }
  // Receivers by tile (persistent step) and the persistent step's schedule.
  {
    const int n_tiles = tma::tile_count(tile_cfg_, geo_.nx, geo_.nz);
    std::vector<int> start(n_tiles + 1, 0), list(std::max(cfg_.nr, 1));
    for (int r = 0; r < cfg_.nr; ++r)
      ++start[1 + tma::tile_of(tile_cfg_, geo_.nz, ix_rec_[r], iz_rec_[r])];
    for (int t = 0; t < n_tiles; ++t) start[t + 1] += start[t];
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int r = 0; r < cfg_.nr; ++r)
      list[fill[tma::tile_of(tile_cfg_, geo_.nz, ix_rec_[r], iz_rec_[r])]++] = r;
    rec_tile_start_.allocate(start.size() * sizeof(int));
    rec_tile_list_.allocate(list.size() * sizeof(int));
    cuda_check(cudaMemcpy(rec_tile_start_.get(), start.data(), start.size() * sizeof(int),
                          cudaMemcpyHostToDevice),
               "receiver tiles");
    cuda_check(cudaMemcpy(rec_tile_list_.get(), list.data(), list.size() * sizeof(int),
                          cudaMemcpyHostToDevice),
               "receiver tiles");
    sched_.allocate(tma::sched_words(tile_cfg_, geo_.nx, geo_.nz) * sizeof(unsigned));
    for (int k = 0; k < n_shots; ++k) {
      descs[k].rec_start = rec_tile_start_.as<int>();
      descs[k].rec_list = rec_tile_list_.as<int>();
    }
  }
  descs_h_ = std::move(descs);
  cluster_nc_ = cluster::plan(geo_.nx, geo_.nz, cfg_.np_boundary);
  tma_ok_ = true;
}

cudaError_t Model::tma_forward(int shot, bool store, int it0, int it1, bool zero, bool finish,
                               cudaEvent_t *events, bool allow_cluster) {
  cudaStream_t s = stream();
  if (zero) {
    const size_t bytes = padded_size() * sizeof(float);
    for (int f = 0; f < 5; ++f) {
      cudaError_t e = cudaMemsetAsync(fields_[f].get(), 0, bytes, s);
      if (e == cudaSuccess) e = cudaMemsetAsync(fields2_[f].get(), 0, bytes, s);
      if (e != cudaSuccess) return e;
    }
    cur_ = 0;
  }
  const tma::SimDesc &h = descs_h_[shot];
  const int cfg = tile_cfg_;
  if (variant_ == kFusedCluster && allow_cluster && it1 > it0) {
    cudaError_t e = cluster::steps(h, false, it0, it1 - it0, cur_, store, cluster_nc_, s);
    if (e != cudaSuccess) return e;
    cur_ ^= (it1 - it0) & 1;
    it0 = it1;  // done; falls through to the seismograms
  }
  if (variant_ == kFusedTmaPersistent && it1 > it0) {
    cudaError_t e = cudaMemsetAsync(sched_.get(), 0, sched_.bytes(), s);
    if (e == cudaSuccess)
      e = tma::steps_persistent(h, cfg, false, it0, it1 - it0, cur_, store, err_flag_.as<int>(),
                                sched_.as<unsigned>(), s);
    if (e != cudaSuccess) return e;
    cur_ ^= (it1 - it0) & 1;
    it0 = it1;  // done; falls through to the seismograms
  }
  for (int it = it0; it < it1; ++it) {
    cudaEvent_t *ev = events ? events + 2 * (it - it0) : nullptr;
    if (ev) cudaEventRecord(ev[0], s);
    cudaError_t e = tma::step_single(h, cfg, false, it, cur_, store, err_flag_.as<int>(), s);
    if (ev) cudaEventRecord(ev[1], s);
    if (e != cudaSuccess) return e;
    cur_ ^= 1;
  }
  if (finish && cfg_.nr) {
    const size_t off = static_cast<size_t>(shot) * cfg_.nr * cfg_.nt;
    const float *raw = rec_raw_.as<float>();
    cudaError_t e = receiver_cumsum_f32(cfg_.nr, cfg_.nt, it1, cfg_.dt, cfg_.dx * cfg_.dz, raw,
                                        raw + static_cast<size_t>(cfg_.nr) * cfg_.nt,
                                        rtf_[0].as<double>() + off, rtf_[1].as<double>() + off, s);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

cudaError_t Model::tma_adjoint(int shot) {
  cudaStream_t s = stream();
  const size_t bytes = padded_size() * sizeof(float);
  for (int f = 0; f < 5; ++f) {
    cudaError_t e = cudaMemsetAsync(fields_[f].get(), 0, bytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(fields2_[f].get(), 0, bytes, s);
    if (e != cudaSuccess) return e;
  }
  cur_ = 0;
  const tma::SimDesc &h = descs_h_[cfg_.n_shots + shot];
  const int cfg = tile_cfg_;
  if (variant_ == kFusedCluster) {
    cudaError_t e = cluster::steps(h, true, cfg_.nt - 1, cfg_.nt, 0, false, cluster_nc_, s);
    if (e != cudaSuccess) return e;
    cur_ = cfg_.nt & 1;
    return cudaGetLastError();
  }
  if (variant_ == kFusedTmaPersistent) {
    cudaError_t e = cudaMemsetAsync(sched_.get(), 0, sched_.bytes(), s);
    if (e == cudaSuccess)
      e = tma::steps_persistent(h, cfg, true, cfg_.nt - 1, cfg_.nt, 0, false, err_flag_.as<int>(),
                                sched_.as<unsigned>(), s);
    if (e != cudaSuccess) return e;
    cur_ = cfg_.nt & 1;
    return cudaGetLastError();
  }
  for (int it = cfg_.nt - 1; it >= 0; --it) {
    cudaError_t e = tma::step_single(h, cfg, true, it, cur_, false, err_flag_.as<int>(), s);
    if (e != cudaSuccess) return e;
    cur_ ^= 1;
  }
  return cudaGetLastError();
}

size_t Model::exact_lane_bytes(int C) const {
  const int nt = cfg_.nt;
  if (C <= 0 || C > nt) C = nt;
  const size_t state = 5 * padded_size() * elem();
  const size_t n_ck = (nt + C - 1) / C;
  return n_ck * state + (C + 1) * state + kLamPlanes * padded_size() * elem() +
         2 * static_cast<size_t>(cfg_.nr) * nt * sizeof(float) +
         padded_size() * (sizeof(float2) + sizeof(float));
}

int Model::exact_lane_count(int C, int n_list) const {
  // As many lanes as shots, at most kMaxExactLanes, within 60 % of the device
  // memory that is free or already held by lanes.
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 1;
  for (const auto &l : lanes_)
    free_b += l->ckpt.bytes() + l->slots.bytes() + l->lam.bytes() + l->raw.bytes() +
              l->part.bytes();
  const size_t per = std::max<size_t>(exact_lane_bytes(C), 1);
  const size_t fit = static_cast<size_t>(0.6 * static_cast<double>(free_b)) / per;
  return static_cast<int>(std::max<size_t>(1, std::min<size_t>(
      fit, static_cast<size_t>(std::min(n_list, kMaxExactLanes)))));
}

size_t Model::exact_bytes(int C) const {
  const int nt = cfg_.nt;
  if (C <= 0 || C > nt) C = nt;
  if (prec_ == PSV_FP32 && tma_ok_ && is_tma())
    return static_cast<size_t>(exact_lane_count(C, cfg_.n_shots)) * exact_lane_bytes(C) +
           static_cast<size_t>(cfg_.n_shots) * 4 * grid_size() * sizeof(float2) +
           7 * grid_size() * sizeof(double);
  const size_t state = 5 * padded_size() * elem();
  const size_t n_ck = (nt + C - 1) / C;
  return n_ck * state + (C + 1) * state + 13 * padded_size() * elem() +
         7 * grid_size() * sizeof(double);
}

double Model::exact_gradient(int C) {
  std::vector<int> all(cfg_.n_shots);
  for (int s = 0; s < cfg_.n_shots; ++s) all[s] = s;
  return exact_gradient(C, all);
}

double Model::exact_gradient(int C, const std::vector<int> &shot_list) {
  DeviceGuard guard(device_);
  {
    std::vector<char> seen(cfg_.n_shots, 0);
    for (int s : shot_list) {
      if (s < 0 || s >= cfg_.n_shots) throw Error(PSV_ERR_INVALID_ARGUMENT, "i_shot out of range");
      if (seen[s]++) throw Error(PSV_ERR_INVALID_ARGUMENT, "a shot is listed twice");
    }
  }
  if (prec_ == PSV_FP32 && tma_ok_ && is_tma()) return exact_gradient_lanes(C, shot_list);
  const int nt = cfg_.nt, n_shots = cfg_.n_shots, nr = cfg_.nr;
  if (C <= 0 || C > nt) C = nt;
  const int n_ck = (nt + C - 1) / C;
  const size_t gp = padded_size(), g = grid_size(), e = elem();
  const size_t field_bytes = gp * e, state_bytes = 5 * field_bytes;
  cudaStream_t s = stream();
  // Scratch grows only; captured pipelines hold its addresses, so a
  // reallocation drops them.
  bool grown = false;
  auto ensure = [&](DeviceBuffer &b, size_t bytes) {
    if (b.bytes() < bytes) {
      synchronize();
      b.allocate(bytes);
      grown = true;
    }
  };
  for (auto &b : gex_) ensure(b, g * sizeof(double));
  for (auto &b : kexact_) ensure(b, g * sizeof(double));
  for (auto &b : adj_) ensure(b, data_size() * sizeof(double));
  ensure(lam_, kLamPlanes * field_bytes);
  const bool etma = prec_ == PSV_FP32 && tma_ok_;
  if (etma)
    for (auto &b : gff_) ensure(b, g * sizeof(float2));
  ensure(ckpt_, n_ck * state_bytes);
  ensure(slots_, (C + 1) * state_bytes);
  if (grown) clear_graphs();
  for (auto &b : gex_) cuda_check(cudaMemsetAsync(b.get(), 0, b.bytes(), s), "exact zero");
  if (etma)
    for (auto &b : gff_) cuda_check(cudaMemsetAsync(b.get(), 0, b.bytes(), s), "exact zero");
  // FP32: the exact step reads its tiles through tensor maps over the
  // adjoint planes, the state slots and the medium, and sums the gradient
  // in float-float pairs (gff_), turned into FP64 (gex_) at the end.
  exact_tma::Maps emaps;
  if (etma &&
      !exact_tma::encode(emaps, lam_.as<float>(), kLamPlanes, slots_.as<float>(), 5 * (C + 1),
                         field_bytes, lm_.as<float>(), la_.as<float>(), mu_.as<float>(),
                         b_.as<float>(), geo_.nx, geo_.nz, pitch_))
    throw Error(PSV_ERR_CUDA, "tensor-map encoding failed for the exact adjoint");

  const SolverArgs a = solver_args();
  unsigned char *ck = ckpt_.as<unsigned char>(), *sl = slots_.as<unsigned char>();
  void *fields[5];
  for (int f = 0; f < 5; ++f) fields[f] = fields_[f].get();
  auto state = [&](unsigned char *base, void *out[5]) {
    for (int f = 0; f < 5; ++f) out[f] = base + f * field_bytes;
  };
  // dst <- src (and dst2 <- src), whole states.
  auto copy = [&](void *const src[5], void *const dst[5], void *const *dst2) {
    cuda_check(copy_state(src, dst, dst2, field_bytes, s), "copy state");
  };
  auto fwd = [&](int shot, int it0, int it1, bool finish) {
    cudaError_t err = prec_ == PSV_FP64
                          ? forward_f64(a, plans_[shot], shot, false, it0, it1, false, finish, s)
                          : forward_f32(a, plans_[shot], shot, false, it0, it1, false, finish, s);
    cuda_check(err, "exact forward");
  };
  // FP32 with the TMA step: the forward runs ping-pong in the model's two
  // field sets (checkpoint pass) and from state slot j straight into slot
  // j + 1 (recompute), so no state is copied per step. The slots' input
  // tensor maps are encoded once per call, when first needed.
  const bool tma = prec_ == PSV_FP32 && tma_ok_ && is_tma();
  std::vector<tma::Maps> slot_maps;
  auto slot_fields = [&](int j) {
    void *p[5];
    state(sl + j * state_bytes, p);
    return fast::Fields{static_cast<float *>(p[0]), static_cast<float *>(p[1]),
                        static_cast<float *>(p[2]), static_cast<float *>(p[3]),
                        static_cast<float *>(p[4])};
  };
  // Steps it0 .. it1-1 of `shot` from slot 0 (state it0) into slots 1 ..
  // it1-it0; receivers are recorded when `record`.
  auto tma_slots = [&](int shot, int it0, int it1, bool record) {
    if (slot_maps.empty()) {
      slot_maps.resize(C + 1);
      for (int j = 0; j <= C; ++j)
        if (!tma::encode_input_maps(slot_maps[j], slot_fields(j), lm_.as<float>(), mu_.as<float>(),
                                    geo_.nx, geo_.nz, pitch_, tile_cfg_))
          throw Error(PSV_ERR_CUDA, "tensor-map encoding failed for a state slot");
    }
    for (int n = it0; n < it1; ++n) {
      const int j = n - it0;
      tma::SimDesc d = descs_h_[shot];
      d.set[0] = slot_fields(j);
      d.set[1] = slot_fields(j + 1);
      d.maps[0] = slot_maps[j];
      if (!record) d.nr = 0;
      cuda_check(tma::step_single(d, tile_cfg_, false, n, 0, false, err_flag_.as<int>(), s),
                 "exact forward");
    }
  };
  // One shot: checkpointed forward (which also gives the shot's seismograms
  // and, from them, its adjoint receiver terms), then the segments
  // backwards: each is recomputed from its checkpoint into C + 1 state slots
  // and transposed step by step. Deterministic in (shot, C) and the scratch
  // addresses, so it is captured once as a CUDA graph and replayed.
  auto one_shot = [&](int shot) {
    if (tma) {
      // Checkpoint pass; its last segment writes its states into the slots
      // directly, and the reverse pass starts from them.
      const int last0 = (n_ck - 1) * C;
      // The checkpoint pass runs the TMA step, as the recompute does, so that
      // every state is the same whatever the checkpoint interval (the
      // cluster scheme agrees with it to FP32 rounding, not bit for bit).
      if (last0 > 0)
        cuda_check(tma_forward(shot, false, 0, 0, true, false, nullptr, false), "zero");
      for (int k = 0; k + 1 < n_ck; ++k) {
        void *src[5], *dst[5];
        for (int f = 0; f < 5; ++f) src[f] = (cur_ ? fields2_ : fields_)[f].get();
        state(ck + k * state_bytes, dst);
        copy(src, dst, nullptr);
        cuda_check(tma_forward(shot, false, k * C, (k + 1) * C, false, false, nullptr, false),
                   "exact forward");
      }
      if (last0 > 0) {
        void *src[5], *dst[5];
        for (int f = 0; f < 5; ++f) src[f] = (cur_ ? fields2_ : fields_)[f].get();
        state(sl, dst);
        copy(src, dst, nullptr);
      } else {
        cuda_check(cudaMemsetAsync(sl, 0, state_bytes, s), "zero state");
      }
      tma_slots(shot, last0, nt, true);
      if (nr) {
        const size_t off = static_cast<size_t>(shot) * nr * nt;
        const float *raw = rec_raw_.as<float>();
        cuda_check(receiver_cumsum_f32(nr, nt, nt, cfg_.dt, cfg_.dx * cfg_.dz, raw,
                                       raw + static_cast<size_t>(nr) * nt,
                                       rtf_[0].as<double>() + off, rtf_[1].as<double>() + off, s),
                   "seismograms");
      }
    } else {
      for (auto &f : fields_) cuda_check(cudaMemsetAsync(f.get(), 0, f.bytes(), s), "zero");
      for (int k = 0; k < n_ck; ++k) {
        void *dst[5];
        state(ck + k * state_bytes, dst);
        copy(fields, dst, nullptr);
        fwd(shot, k * C, std::min(nt, (k + 1) * C), k + 1 == n_ck);
      }
    }
    const size_t off = static_cast<size_t>(shot) * nr * nt;
    for (int c = 0; c < 2; ++c)
      cuda_check(exact_receiver_terms(nr, nt, cfg_.dt, cfg_.dx * cfg_.dz, rtf_[c].as<double>() + off,
                                      rtf_true_[c].as<double>() + off, adj_[c].as<double>() + off,
                                      s),
                 "receiver terms");
    cuda_check(cudaMemsetAsync(lam_.get(), 0, lam_.bytes(), s), "zero adjoint");
    // Adjoint state planes: l^{n+1} in (lv, lt), l^n out (ov, ot), swapped
    // after every step.
    int lv[2] = {0, 1}, ov[2] = {8, 9}, lt[3] = {2, 3, 4}, ot[3] = {5, 6, 7};
    auto plane = [&](int k) { return lam_.as<unsigned char>() + k * field_bytes; };
    for (int k = n_ck - 1; k >= 0; --k) {
      const int s0 = k * C, s1 = std::min(nt, s0 + C);
      void *src[5], *slot0[5];
      state(ck + k * state_bytes, src);
      state(sl, slot0);
      if (tma) {
        if (k + 1 < n_ck) {  // the last segment's states are already in the slots
          copy(src, slot0, nullptr);
          tma_slots(shot, s0, s1, false);
        }
      } else {
        copy(src, fields, slot0);
        for (int n = s0; n < s1; ++n) {
          void *dst[5];
          state(sl + (n + 1 - s0) * state_bytes, dst);
          fwd(shot, n, n + 1, false);
          copy(fields, dst, nullptr);
        }
      }
      for (int n = s1 - 1; n >= s0; --n) {
        if (etma) {
          exact_tma::Step x;
          x.nx = geo_.nx;
          x.nz = geo_.nz;
          x.pitch = pitch_;
          x.np = cfg_.np_boundary;
          x.nt = nt;
          x.it = n;
          x.dt = static_cast<float>(cfg_.dt);
          x.idx = static_cast<float>(1.0 / cfg_.dx);
          x.idz = static_cast<float>(1.0 / cfg_.dz);
          x.dt_d = cfg_.dt;
          x.taper_tab = taper_tab_d_.as<float>();
          for (int f = 0; f < 2; ++f) {
            x.lv[f] = lv[f];
            x.olv[f] = reinterpret_cast<float *>(plane(ov[f]));
          }
          for (int f = 0; f < 3; ++f) {
            x.lt[f] = lt[f];
            x.olt[f] = reinterpret_cast<float *>(plane(ot[f]));
          }
          x.sv = 5 * (n - s0);
          x.st = 5 * (n + 1 - s0);
          x.g_lm = gff_[0].as<float2>();
          x.g_la = gff_[1].as<float2>();
          x.g_mu = gff_[2].as<float2>();
          x.g_b = gff_[3].as<float2>();
          x.plan = plans_[shot];
          x.stf = stf_d_.as<double>();
          x.rec_cell = rec_cell_.as<int>();
          x.rec_start = exrec_start_.as<int>();
          x.rec_list = exrec_list_.as<int>();
          x.adj_x = adj_[0].as<double>() + off;
          x.adj_z = adj_[1].as<double>() + off;
          x.err = err_flag_.as<int>();
          cuda_check(exact_tma::step(emaps, x, s), "exact step");
          for (int f = 0; f < 2; ++f) std::swap(lv[f], ov[f]);
          for (int f = 0; f < 3; ++f) std::swap(lt[f], ot[f]);
          continue;
        }
        ExactStepArgs x;
        x.nx = geo_.nx;
        x.nz = geo_.nz;
        x.pitch = pitch_;
        x.np = cfg_.np_boundary;
        x.nt = nt;
        x.it = n;
        x.nr = nr;
        x.dt = cfg_.dt;
        x.dx = cfg_.dx;
        x.dz = cfg_.dz;
        x.lm = lm_.get();
        x.la = la_.get();
        x.mu = mu_.get();
        x.b = b_.get();
        x.taper_tab = taper_tab_d_.get();
        for (int f = 0; f < 2; ++f) {
          x.lv[f] = plane(lv[f]);
          x.ov[f] = plane(ov[f]);
        }
        for (int f = 0; f < 3; ++f) {
          x.lt[f] = plane(lt[f]);
          x.ot[f] = plane(ot[f]);
        }
        const unsigned char *sv = sl + (n - s0) * state_bytes;      // v^n
        const unsigned char *st = sl + (n + 1 - s0) * state_bytes;  // tau^(n+1)
        x.fv[0] = sv;
        x.fv[1] = sv + field_bytes;
        x.ft[0] = st + 2 * field_bytes;
        x.ft[1] = st + 3 * field_bytes;
        x.ft[2] = st + 4 * field_bytes;
        x.g_lm = gex_[0].as<double>();
        x.g_la = gex_[1].as<double>();
        x.g_mu = gex_[2].as<double>();
        x.g_b = gex_[3].as<double>();
        x.plan = plans_[shot];
        x.stf = stf_d_.as<double>();
        x.rec_cell = rec_cell_.as<int>();
        x.n_rec_groups = n_rec_groups_;
        x.rec_start = rec_start_.as<int>();
        x.rec_order = rec_order_.as<int>();
        x.adj_x = adj_[0].as<double>() + off;
        x.adj_z = adj_[1].as<double>() + off;
        cuda_check(prec_ == PSV_FP64 ? exact_step_f64(x, s) : exact_step_f32(x, s), "exact step");
        for (int f = 0; f < 2; ++f) std::swap(lv[f], ov[f]);
        for (int f = 0; f < 3; ++f) std::swap(lt[f], ot[f]);
      }
    }
  };
  cur_ = 0;
  for (int shot : shot_list) run_loop(2, shot, false, C, [&] { one_shot(shot); });
  double misfit = 0;
  if (static_cast<int>(shot_list.size()) == n_shots) {
    misfit = calculate_l2_misfit();
  } else {
    // Misfit of the listed shots: the same reduction over each shot's slice.
    const size_t per = static_cast<size_t>(nr) * nt;
    for (int shot : shot_list) {
      if (!per) break;
      const size_t off = static_cast<size_t>(shot) * per;
      int parts = static_cast<int>(std::min<size_t>(kPartials, (per + 255) / 256));
      if (parts < 1) parts = 1;
      cuda_check(misfit_l2(per, cfg_.dt, rtf_true_[0].as<double>() + off, rtf_[0].as<double>() + off,
                           rtf_true_[1].as<double>() + off, rtf_[1].as<double>() + off,
                           partials_.as<double>(), parts, scalar_.as<double>(), s),
                 "shot misfit");
      double v = 0;
      cuda_check(cudaMemcpyAsync(&v, scalar_.get(), sizeof(double), cudaMemcpyDeviceToHost, s),
                 "misfit copy");
      synchronize();
      misfit += v;
    }
    misfit_ = misfit;
  }
  if (etma) {
    float2 *ff[4] = {gff_[0].as<float2>(), gff_[1].as<float2>(), gff_[2].as<float2>(),
                     gff_[3].as<float2>()};
    double *out[4] = {gex_[0].as<double>(), gex_[1].as<double>(), gex_[2].as<double>(),
                      gex_[3].as<double>()};
    cuda_check(exact_tma::finish(g, ff, out, s), "exact sums");
  }
  // Chain rule to (vp, vs, rho).
  cuda_check(exact_chain(g, vp_.as<double>(), vs_.as<double>(), rho_.as<double>(),
                         gex_[0].as<double>(), gex_[1].as<double>(), gex_[2].as<double>(),
                         gex_[3].as<double>(), kexact_[0].as<double>(), kexact_[1].as<double>(),
                         kexact_[2].as<double>(), s),
             "exact chain");
  synchronize();
  if (tma || etma) check_device_error();
  return misfit;
}

void Model::destroy_lanes() {
  for (auto &l : lanes_) {
    if (l->stream) {
      cudaStreamSynchronize(l->stream);
      cudaStreamDestroy(l->stream);
    }
    if (l->done) cudaEventDestroy(l->done);
  }
  lanes_.clear();
  if (lanes_start_) {
    cudaEventDestroy(lanes_start_);
    lanes_start_ = nullptr;
  }
}

// FP32 exact gradient with the TMA steps, the shots in concurrent lanes.
// Per shot, in its lane (stream order), the same pipeline as the serial
// path: a checkpoint pass (the forward run slot to slot, its state saved
// every C steps, its receivers recorded), the seismograms and adjoint
// receiver terms, then the segments backwards, each recomputed from its
// checkpoint into the C + 1 state slots and transposed step by step into
// the shot's own gradient sums. Every forward step, in either pass, is the
// same TMA step kernel from slot j into slot j + 1, so every state is the
// same whatever C. Each shot's pipeline is captured once as a CUDA graph on
// its lane's stream and replayed. At the end the shots' sums are added in
// shot order, and the chain rule maps them to (vp, vs, rho).
int Model::ensure_lanes(int K) {
  int changed = 0;
  // Lanes beyond K give their memory back.
  while (static_cast<int>(lanes_.size()) > K) {
    auto &l = lanes_.back();
    if (l->stream) {
      cuda_check(cudaStreamSynchronize(l->stream), "lane sync");
      cudaStreamDestroy(l->stream);
    }
    if (l->done) cudaEventDestroy(l->done);
    lanes_.pop_back();
    changed = 1;
  }
  while (static_cast<int>(lanes_.size()) < K) {
    auto l = std::make_unique<ExactLane>();
    if (!lanes_.empty())
      cuda_check(cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking), "lane stream");
    cuda_check(cudaEventCreateWithFlags(&l->done, cudaEventDisableTiming), "lane event");
    lanes_.push_back(std::move(l));
    changed = 1;
  }
  if (!lanes_start_)
    cuda_check(cudaEventCreateWithFlags(&lanes_start_, cudaEventDisableTiming), "lane event");
  return changed;
}

double Model::exact_gradient_lanes(int C, const std::vector<int> &shot_list) {
  const int nt = cfg_.nt, n_shots = cfg_.n_shots, nr = cfg_.nr;
  if (C <= 0 || C > nt) C = nt;
  const int n_ck = (nt + C - 1) / C;
  const size_t gp = padded_size(), g = grid_size();
  const size_t field_bytes = gp * sizeof(float), state_bytes = 5 * field_bytes;
  cudaStream_t ms = stream();
  const int n_list = static_cast<int>(shot_list.size());
  const int K = std::max(1, exact_lane_count(C, std::max(n_list, 1)));
  // Forward steps of the lanes: the 32 x 60 shape (the vectorised tile
  // path, fewest instructions per point) when the lanes' tiles fill at
  // least two waves of resident CTAs between them; else the model's shape.
  // Measured at c3 (1100 x 500): eight lanes 1.07 s with 32 x 60 against
  // 1.14 s with 16 x 28; two lanes (every state kept) 0.88 s against 0.84 s.
  // (Four lanes now: 4 x 315 tiles, still 32 x 60.)
  int ecfg = tile_cfg_;
  {
    const int big = tma::resident_ctas(tma::kTile32x60, false);
    if (big > 0 && static_cast<long long>(K) *
                           tma::tile_count(tma::kTile32x60, geo_.nx, geo_.nz) >= 2LL * big)
      ecfg = tma::kTile32x60;
  }

  bool grown = false;
  auto ensure = [&](DeviceBuffer &b, size_t bytes) {
    if (b.bytes() < bytes) {
      synchronize();
      for (auto &l : lanes_)
        if (l->stream) cuda_check(cudaStreamSynchronize(l->stream), "lane sync");
      b.allocate(bytes);
      grown = true;
    }
  };
  if (ensure_lanes(K)) grown = true;
  for (auto &l : lanes_) {
    ensure(l->ckpt, n_ck * state_bytes);
    ensure(l->slots, (C + 1) * state_bytes);
    ensure(l->lam, kLamPlanes * field_bytes);
    ensure(l->raw, std::max<size_t>(2 * static_cast<size_t>(nr) * nt * sizeof(float), 16));
    ensure(l->part, gp * (sizeof(float2) + sizeof(float)));
  }
  for (auto &b : gex_) ensure(b, g * sizeof(double));
  for (auto &b : kexact_) ensure(b, g * sizeof(double));
  for (auto &b : adj_) ensure(b, data_size() * sizeof(double));
  ensure(gff_shots_, static_cast<size_t>(n_shots) * 4 * g * sizeof(float2));
  if (grown) clear_graphs();

  // Tensor maps of each lane's slots (forward steps) and of its adjoint
  // planes, slots and the medium (exact steps); encoded when the buffers,
  // C or the tile shape change.
  auto slot_fields = [&](ExactLane &l, int j) {
    float *b = reinterpret_cast<float *>(l.slots.as<unsigned char>() + j * state_bytes);
    const size_t n = gp;
    return fast::Fields{b, b + n, b + 2 * n, b + 3 * n, b + 4 * n};
  };
  for (auto &lp : lanes_) {
    ExactLane &l = *lp;
    if (l.maps_slots == l.slots.get() && l.maps_lam == l.lam.get() && l.maps_C == C &&
        l.maps_cfg == ecfg)
      continue;
    l.slot_maps.assign(C + 1, tma::Maps{});
    for (int j = 0; j <= C; ++j)
      if (!tma::encode_input_maps(l.slot_maps[j], slot_fields(l, j), lm_.as<float>(),
                                  mu_.as<float>(), geo_.nx, geo_.nz, pitch_, ecfg))
        throw Error(PSV_ERR_CUDA, "tensor-map encoding failed for a state slot");
    if (!exact_tma::encode(l.emaps, l.lam.as<float>(), kLamPlanes, l.slots.as<float>(),
                           5 * (C + 1), field_bytes, lm_.as<float>(), la_.as<float>(),
                           mu_.as<float>(), b_.as<float>(), geo_.nx, geo_.nz, pitch_))
      throw Error(PSV_ERR_CUDA, "tensor-map encoding failed for the exact adjoint");
    l.maps_slots = l.slots.get();
    l.maps_lam = l.lam.get();
    l.maps_C = C;
    l.maps_cfg = ecfg;
  }

  auto one_shot = [&](ExactLane &l, int shot, cudaStream_t s) {
    unsigned char *ck = l.ckpt.as<unsigned char>(), *sl = l.slots.as<unsigned char>();
    float2 *gs = gff_shots_.as<float2>() + static_cast<size_t>(shot) * 4 * g;
    cuda_check(cudaMemsetAsync(gs, 0, 4 * g * sizeof(float2), s), "exact zero");
    cuda_check(cudaMemsetAsync(l.part.get(), 0, gp * (sizeof(float2) + sizeof(float)), s),
               "exact zero");
    auto state = [&](unsigned char *base, void *out[5]) {
      for (int f = 0; f < 5; ++f) out[f] = base + f * field_bytes;
    };
    auto copy = [&](unsigned char *from, unsigned char *to) {
      void *src[5], *dst[5];
      state(from, src);
      state(to, dst);
      cuda_check(copy_state(src, dst, nullptr, field_bytes, s), "copy state");
    };
    float *raw = l.raw.as<float>();
    // Step n from slot j_in into slot j_out.
    auto step = [&](int n, int j_in, int j_out, bool record) {
      tma::SimDesc d = descs_h_[shot];
      d.set[0] = slot_fields(l, j_in);
      d.set[1] = slot_fields(l, j_out);
      d.maps[0] = l.slot_maps[j_in];
      d.rec_vx = raw;
      d.rec_vz = raw + static_cast<size_t>(nr) * nt;
      if (!record) d.nr = 0;
      cuda_check(tma::step_single(d, ecfg, false, n, 0, false, err_flag_.as<int>(), s),
                 "exact forward");
    };
    // Steps it0 .. it1-1 from slot 0 (state it0) into slots 1 .. it1-it0.
    auto slots_forward = [&](int it0, int it1, bool record) {
      for (int n = it0; n < it1; ++n) step(n, n - it0, n - it0 + 1, record);
    };
    // Checkpoint pass. Every segment but the last runs back and forth
    // between slots 0 and 1 (two states that stay in L2, where C + 1 slots
    // would stream through DRAM); the last one runs into slots 1 .. for the
    // reverse sweep. The same step kernel either way, so the same states.
    cuda_check(cudaMemsetAsync(sl, 0, state_bytes, s), "zero state");
    int cur = 0;  // slot holding the current state
    for (int k = 0; k < n_ck; ++k) {
      const int s0 = k * C, s1 = std::min(nt, s0 + C);
      copy(sl + cur * state_bytes, ck + k * state_bytes);
      if (k + 1 < n_ck) {
        for (int n = s0; n < s1; ++n) {
          step(n, cur, cur ^ 1, true);
          cur ^= 1;
        }
      } else {
        if (cur != 0) copy(sl + cur * state_bytes, sl);
        slots_forward(s0, s1, true);
      }
    }
    const size_t off = static_cast<size_t>(shot) * nr * nt;
    if (nr) {
      cuda_check(receiver_cumsum_f32(nr, nt, nt, cfg_.dt, cfg_.dx * cfg_.dz, raw,
                                     raw + static_cast<size_t>(nr) * nt,
                                     rtf_[0].as<double>() + off, rtf_[1].as<double>() + off, s),
                 "seismograms");
      for (int c = 0; c < 2; ++c)
        cuda_check(exact_receiver_terms(nr, nt, cfg_.dt, cfg_.dx * cfg_.dz,
                                        rtf_[c].as<double>() + off,
                                        rtf_true_[c].as<double>() + off,
                                        adj_[c].as<double>() + off, s),
                   "receiver terms");
    }
    cuda_check(cudaMemsetAsync(l.lam.get(), 0, l.lam.bytes(), s), "zero adjoint");
    // Adjoint state planes: l^{n+1} in (lv, lt), l^n out (ov, ot), swapped
    // after every step.
    int lv[2] = {0, 1}, ov[2] = {8, 9}, lt[3] = {2, 3, 4}, ot[3] = {5, 6, 7};
    auto plane = [&](int k) { return l.lam.as<unsigned char>() + k * field_bytes; };
    for (int k = n_ck - 1; k >= 0; --k) {
      const int s0 = k * C, s1 = std::min(nt, s0 + C);
      if (k + 1 < n_ck) {  // the last segment's states are still in the slots
        copy(ck + k * state_bytes, sl);
        slots_forward(s0, s1, false);
      }
      for (int n = s1 - 1; n >= s0; --n) {
        exact_tma::Step x;
        x.nx = geo_.nx;
        x.nz = geo_.nz;
        x.pitch = pitch_;
        x.np = cfg_.np_boundary;
        x.nt = nt;
        x.it = n;
        x.dt = static_cast<float>(cfg_.dt);
        x.idx = static_cast<float>(1.0 / cfg_.dx);
        x.idz = static_cast<float>(1.0 / cfg_.dz);
        x.dt_d = cfg_.dt;
        x.taper_tab = taper_tab_d_.as<float>();
        for (int f = 0; f < 2; ++f) {
          x.lv[f] = lv[f];
          x.olv[f] = reinterpret_cast<float *>(plane(ov[f]));
        }
        for (int f = 0; f < 3; ++f) {
          x.lt[f] = lt[f];
          x.olt[f] = reinterpret_cast<float *>(plane(ot[f]));
        }
        x.sv = 5 * (n - s0);
        x.st = 5 * (n + 1 - s0);
        x.g_lm = gs;
        x.g_la = gs + g;
        x.g_mu = gs + 2 * g;
        x.g_b = gs + 3 * g;
        // Terms go into FP32 partial sums (lambda's folded into lm's and
        // mu's), added into the float-float pairs every kFlushSteps steps
        // and at step 0.
        x.g_part_lmu = l.part.as<float2>();
        x.g_part_b = reinterpret_cast<float *>(l.part.as<unsigned char>() + gp * sizeof(float2));
        x.flush = (n % kFlushSteps == 0) ? 1 : 0;
        x.plan = plans_[shot];
        x.stf = stf_d_.as<double>();
        x.rec_cell = rec_cell_.as<int>();
        x.rec_start = exrec_start_.as<int>();
        x.rec_list = exrec_list_.as<int>();
        x.adj_x = adj_[0].as<double>() + off;
        x.adj_z = adj_[1].as<double>() + off;
        x.err = err_flag_.as<int>();
        cuda_check(exact_tma::step(l.emaps, x, s), "exact step");
        for (int f = 0; f < 2; ++f) std::swap(lv[f], ov[f]);
        for (int f = 0; f < 3; ++f) std::swap(lt[f], ot[f]);
      }
    }
  };

  // Lanes start after the work already queued on the model's stream.
  cuda_check(cudaEventRecord(lanes_start_, ms), "lane start");
  for (int k = 1; k < K; ++k)
    cuda_check(cudaStreamWaitEvent(lanes_[k]->stream, lanes_start_, 0), "lane wait");
  for (int i = 0; i < n_list; ++i) {
    const int shot = shot_list[i];
    const int li = i % K;
    ExactLane &l = *lanes_[li];
    cudaStream_t s = li == 0 ? ms : l.stream;
    auto enqueue = [&] { one_shot(l, shot, s); };
    if (!use_graphs_) {
      enqueue();
      continue;
    }
    GraphEntry &ge = graphs_[std::make_tuple(3 + li, shot, K, C)];
    if (ge.exec) {
      cuda_check(cudaGraphLaunch(ge.exec, s), "cudaGraphLaunch");
      continue;
    }
    if (ge.uses++ == 0) {  // first run: eager
      enqueue();
      continue;
    }
    cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
               "cudaStreamBeginCapture");
    try {
      enqueue();
    } catch (...) {
      cudaGraph_t broken = nullptr;
      cudaStreamEndCapture(s, &broken);
      if (broken) cudaGraphDestroy(broken);
      throw;
    }
    cudaGraph_t graph = nullptr;
    cuda_check(cudaStreamEndCapture(s, &graph), "cudaStreamEndCapture");
    cudaError_t e = cudaGraphInstantiate(&ge.exec, graph, 0);
    cudaGraphDestroy(graph);
    cuda_check(e, "cudaGraphInstantiate");
    cuda_check(cudaGraphLaunch(ge.exec, s), "cudaGraphLaunch");
  }
  for (int k = 1; k < K; ++k) {
    cuda_check(cudaEventRecord(lanes_[k]->done, lanes_[k]->stream), "lane done");
    cuda_check(cudaStreamWaitEvent(ms, lanes_[k]->done, 0), "lane join");
  }

  double misfit = 0;
  if (n_list == n_shots) {
    misfit = calculate_l2_misfit();
  } else {
    const size_t per = static_cast<size_t>(nr) * nt;
    for (int shot : shot_list) {
      if (!per) break;
      const size_t off = static_cast<size_t>(shot) * per;
      int parts = static_cast<int>(std::min<size_t>(kPartials, (per + 255) / 256));
      if (parts < 1) parts = 1;
      cuda_check(misfit_l2(per, cfg_.dt, rtf_true_[0].as<double>() + off, rtf_[0].as<double>() + off,
                           rtf_true_[1].as<double>() + off, rtf_[1].as<double>() + off,
                           partials_.as<double>(), parts, scalar_.as<double>(), ms),
                 "shot misfit");
      double v = 0;
      cuda_check(cudaMemcpyAsync(&v, scalar_.get(), sizeof(double), cudaMemcpyDeviceToHost, ms),
                 "misfit copy");
      synchronize();
      misfit += v;
    }
    misfit_ = misfit;
  }
  // The shots' sums in increasing shot order (independent of the lanes).
  std::vector<int> order(shot_list);
  std::sort(order.begin(), order.end());
  double *out[4] = {gex_[0].as<double>(), gex_[1].as<double>(), gex_[2].as<double>(),
                    gex_[3].as<double>()};
  if (order.empty())
    for (auto &b : gex_) cuda_check(cudaMemsetAsync(b.get(), 0, b.bytes(), ms), "exact zero");
  for (size_t i = 0; i < order.size(); ++i) {
    const float2 *gs = gff_shots_.as<float2>() + static_cast<size_t>(order[i]) * 4 * g;
    const float2 *ff[4] = {gs, gs + g, gs + 2 * g, gs + 3 * g};
    cuda_check(exact_tma::accumulate(g, ff, out, i == 0, ms), "exact sums");
  }
  cuda_check(exact_chain(g, vp_.as<double>(), vs_.as<double>(), rho_.as<double>(),
                         gex_[0].as<double>(), gex_[1].as<double>(), gex_[2].as<double>(),
                         gex_[3].as<double>(), kexact_[0].as<double>(), kexact_[1].as<double>(),
                         kexact_[2].as<double>(), ms),
             "exact chain");
  synchronize();
  check_device_error();
  return misfit;
}

bool Model::run_model_lanes_ok() const {
  return prec_ == PSV_FP32 && tma_ok_ && cfg_.n_shots > 1 &&
         (variant_ == kFusedTma || variant_ == kFusedTmaPersistent);
}

// run_model with the shots in concurrent lanes (FP32, per-step TMA
// launches; the persistent scheme's steps are the same tile arithmetic, so
// the same states). Forward phase: each shot, in lane k % K, advances from
// zero fields in the lane's two state slots (ping-pong), storing its
// snapshots and recording its receivers into the lane's raw series, then
// its seismograms. The misfit and adjoint sources follow on the model's
// stream. Adjoint phase: each shot's adjoint in its lane, correlating into
// the shot's own kernel sums, which are added to the kernels in shot order.
// The last shot's final fields are copied into the model's fields, where
// the serial run leaves them.
void Model::run_model_lanes(bool simulate_adjoint) {
  DeviceGuard guard(device_);
  ensure_snapshots();
  const int n_shots = cfg_.n_shots, nr = cfg_.nr, nt = cfg_.nt;
  const int K = std::min(n_shots, kMaxLanes);
  const size_t gp = padded_size(), g = grid_size();
  const size_t field_bytes = gp * sizeof(float), state_bytes = 5 * field_bytes;
  cudaStream_t ms = stream();
  bool grown = ensure_lanes(K) != 0;
  auto ensure = [&](DeviceBuffer &b, size_t bytes) {
    if (b.bytes() < bytes) {
      synchronize();
      for (auto &l : lanes_)
        if (l->stream) cuda_check(cudaStreamSynchronize(l->stream), "lane sync");
      b.allocate(bytes);
      grown = true;
    }
  };
  for (auto &l : lanes_) {
    ensure(l->slots, 2 * state_bytes);
    ensure(l->raw, std::max<size_t>(2 * static_cast<size_t>(nr) * nt * sizeof(float), 16));
  }
  ensure(kshots_, static_cast<size_t>(n_shots) * 3 * g * sizeof(double));
  if (grown) clear_graphs();
  auto slot_fields = [&](ExactLane &l, int j) {
    float *b = reinterpret_cast<float *>(l.slots.as<unsigned char>() + j * state_bytes);
    return fast::Fields{b, b + gp, b + 2 * gp, b + 3 * gp, b + 4 * gp};
  };
  for (auto &lp : lanes_) {
    ExactLane &l = *lp;
    if (l.rm_slots == l.slots.get() && l.rm_cfg == tile_cfg_) continue;
    for (int j = 0; j < 2; ++j)
      if (!tma::encode_input_maps(l.rm_maps[j], slot_fields(l, j), lm_.as<float>(),
                                  mu_.as<float>(), geo_.nx, geo_.nz, pitch_, tile_cfg_))
        throw Error(PSV_ERR_CUDA, "tensor-map encoding failed for a lane's state");
    l.rm_slots = l.slots.get();
    l.rm_cfg = tile_cfg_;
  }
  // One shot's forward (adjoint = false) or adjoint, in lane l on stream s.
  auto one = [&](ExactLane &l, int shot, bool adjoint, cudaStream_t s) {
    cuda_check(cudaMemsetAsync(l.slots.get(), 0, 2 * state_bytes, s), "zero state");
    tma::SimDesc d = descs_h_[adjoint ? n_shots + shot : shot];
    for (int j = 0; j < 2; ++j) {
      d.set[j] = slot_fields(l, j);
      d.maps[j] = l.rm_maps[j];
    }
    float *raw = l.raw.as<float>();
    d.rec_vx = nr ? raw : nullptr;
    d.rec_vz = nr ? raw + static_cast<size_t>(nr) * nt : nullptr;
    if (adjoint) {
      double *k = kshots_.as<double>() + static_cast<size_t>(shot) * 3 * g;
      cuda_check(cudaMemsetAsync(k, 0, 3 * g * sizeof(double), s), "zero kernels");
      d.klam = k;
      d.kmu = k + g;
      d.krho = k + 2 * g;
    }
    int cur = 0;
    for (int n = 0; n < nt; ++n) {
      const int it = adjoint ? nt - 1 - n : n;
      cuda_check(tma::step_single(d, tile_cfg_, adjoint, it, cur, !adjoint, err_flag_.as<int>(), s),
                 adjoint ? "adjoint_simulate" : "forward_simulate");
      cur ^= 1;
    }
    if (!adjoint && nr) {
      const size_t off = static_cast<size_t>(shot) * nr * nt;
      cuda_check(receiver_cumsum_f32(nr, nt, nt, cfg_.dt, cfg_.dx * cfg_.dz, raw,
                                     raw + static_cast<size_t>(nr) * nt,
                                     rtf_[0].as<double>() + off, rtf_[1].as<double>() + off, s),
                 "seismograms");
    }
  };
  auto phase = [&](bool adjoint) {
    cuda_check(cudaEventRecord(lanes_start_, ms), "lane start");
    for (int k = 1; k < K; ++k)
      cuda_check(cudaStreamWaitEvent(lanes_[k]->stream, lanes_start_, 0), "lane wait");
    for (int shot = 0; shot < n_shots; ++shot) {
      const int li = shot % K;
      ExactLane &l = *lanes_[li];
      cudaStream_t s = li == 0 ? ms : l.stream;
      auto enqueue = [&] { one(l, shot, adjoint, s); };
      if (!use_graphs_) {
        enqueue();
        continue;
      }
      GraphEntry &ge = graphs_[std::make_tuple(20 + li, shot, K, adjoint ? 1 : 0)];
      if (ge.exec) {
        cuda_check(cudaGraphLaunch(ge.exec, s), "cudaGraphLaunch");
        continue;
      }
      if (ge.uses++ == 0) {
        enqueue();
        continue;
      }
      cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                 "cudaStreamBeginCapture");
      try {
        enqueue();
      } catch (...) {
        cudaGraph_t broken = nullptr;
        cudaStreamEndCapture(s, &broken);
        if (broken) cudaGraphDestroy(broken);
        throw;
      }
      cudaGraph_t graph = nullptr;
      cuda_check(cudaStreamEndCapture(s, &graph), "cudaStreamEndCapture");
      cudaError_t e = cudaGraphInstantiate(&ge.exec, graph, 0);
      cudaGraphDestroy(graph);
      cuda_check(e, "cudaGraphInstantiate");
      cuda_check(cudaGraphLaunch(ge.exec, s), "cudaGraphLaunch");
    }
    for (int k = 1; k < K; ++k) {
      cuda_check(cudaEventRecord(lanes_[k]->done, lanes_[k]->stream), "lane done");
      cuda_check(cudaStreamWaitEvent(ms, lanes_[k]->done, 0), "lane join");
    }
    // The last shot's final state into the model's fields (nt steps from
    // slot 0 end in slot nt % 2).
    ExactLane &last = *lanes_[(n_shots - 1) % K];
    void *src[5], *dst[5];
    for (int f = 0; f < 5; ++f) {
      src[f] = last.slots.as<unsigned char>() + (nt & 1) * state_bytes + f * field_bytes;
      dst[f] = fields_[f].get();
    }
    cuda_check(copy_state(src, dst, nullptr, field_bytes, ms), "final state");
    cur_ = 0;
  };
  phase(false);
  calculate_l2_misfit();
  if (simulate_adjoint) {
    calculate_l2_adjoint_sources();
    reset_kernels();
    phase(true);
    double *dst[3] = {klame_[0].as<double>(), klame_[1].as<double>(), klame_[2].as<double>()};
    for (int shot = 0; shot < n_shots; ++shot) {
      const double *k = kshots_.as<double>() + static_cast<size_t>(shot) * 3 * g;
      const double *src[3] = {k, k + g, k + 2 * g};
      cuda_check(add_into3(g, src, dst, ms), "kernel sums");
    }
    map_kernels_to_velocity();
  }
  synchronize();
  check_device_error();
}

void Model::get_exact_gradient(double *g_vp, double *g_vs, double *g_rho, bool device_pointers) {
  DeviceGuard guard(device_);
  if (!kexact_[0].get()) throw Error(PSV_ERR_INVALID_ARGUMENT, "no exact gradient computed yet");
  const size_t bytes = grid_size() * sizeof(double);
  double *out[3] = {g_vp, g_vs, g_rho};
  for (int k = 0; k < 3; ++k)
    if (out[k])
      cuda_check(cudaMemcpyAsync(out[k], kexact_[k].get(), bytes,
                                 device_pointers ? cudaMemcpyDeviceToDevice
                                                 : cudaMemcpyDeviceToHost,
                                 stream()),
                 "get_exact_gradient");
  synchronize();
}

void Model::set_tile_cfg(int cfg) {
  if (cfg < 0 || cfg >= tma::kNumTileCfgs) throw Error(PSV_ERR_INVALID_ARGUMENT, "unknown tile shape");
  if (cfg == tile_cfg_) return;
  DeviceGuard guard(device_);
  clear_graphs();
  tile_cfg_ = cfg;
  if (tma_ok_) {
    synchronize();
    build_descs();
  }
}

int Model::autotune(int n_steps) {
  if (!(prec_ == PSV_FP32 && is_tma())) return tile_cfg_;
  if (cfg_.n_shots < 1) return tile_cfg_;
  DeviceGuard guard(device_);
  n_steps = std::max(1, std::min(n_steps, cfg_.nt));
  // Every (launch scheme, tile shape) pair, timed as forward_simulate runs
  // it: the time loop replayed as a CUDA graph, over n_steps steps.
  cudaEvent_t a, b;
  cuda_check(cudaEventCreate(&a), "cudaEventCreate");
  cuda_check(cudaEventCreate(&b), "cudaEventCreate");
  float best = 0;
  int best_cfg = tile_cfg_, best_variant = variant_;
  bool first = true;
  std::vector<int> variants = {kFusedTma, kFusedTmaPersistent};
  if (cluster_nc_ > 0) variants.push_back(kFusedCluster);
  for (int v : variants) {
    for (int c = 0; c < tma::kNumTileCfgs; ++c) {
      if (v == kFusedCluster && c > 0) break;  // no tiles: timed once
      set_variant(v);
      set_tile_cfg(c);
      forward_simulate(0, false, false, false, n_steps);  // eager
      forward_simulate(0, false, false, false, n_steps);  // captured
      cuda_check(cudaEventRecord(a, stream()), "cudaEventRecord");
      forward_simulate(0, false, false, false, n_steps);
      cuda_check(cudaEventRecord(b, stream()), "cudaEventRecord");
      cuda_check(cudaEventSynchronize(b), "cudaEventSynchronize");
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      if (first || ms < best) {
        best = ms;
        best_cfg = c;
        best_variant = v;
        first = false;
      }
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  set_variant(best_variant);
  set_tile_cfg(best_cfg);
  return best_cfg;
}

void Model::check_device_error() {
  int flag = 0;
  cuda_check(cudaMemcpyAsync(&flag, err_flag_.get(), sizeof(int), cudaMemcpyDeviceToHost, stream()),
             "error flag");
  cuda_check(cudaStreamSynchronize(stream()), "error flag");
  if (flag) {
    cudaMemsetAsync(err_flag_.get(), 0, sizeof(int), stream());
    cudaStreamSynchronize(stream());
    throw Error(PSV_ERR_CUDA, "a CTA timed out waiting for its TMA tile copies");
  }
}

void Model::clear_graphs() {
  for (auto &kv : graphs_)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  graphs_.clear();
}

void Model::run_loop(int direction, int shot, bool store, int n_steps,
                     const std::function<void()> &enqueue) {
  if (!use_graphs_) {
    enqueue();
    return;
  }
  GraphEntry &g = graphs_[std::make_tuple(direction, shot, store ? 1 : 0, n_steps)];
  if (g.exec) {
    cuda_check(cudaGraphLaunch(g.exec, stream()), "cudaGraphLaunch");
    cur_ = g.cur_after;
    return;
  }
  if (g.uses++ == 0) {  // first run: eager (also sets per-device kernel attributes)
    enqueue();
    return;
  }
  cuda_check(cudaStreamBeginCapture(stream(), cudaStreamCaptureModeThreadLocal),
             "cudaStreamBeginCapture");
  try {
    enqueue();
  } catch (...) {
    cudaGraph_t broken = nullptr;
    cudaStreamEndCapture(stream(), &broken);
    if (broken) cudaGraphDestroy(broken);
    throw;
  }
  cudaGraph_t graph = nullptr;
  cuda_check(cudaStreamEndCapture(stream(), &graph), "cudaStreamEndCapture");
  cudaError_t e = cudaGraphInstantiate(&g.exec, graph, 0);
  cudaGraphDestroy(graph);
  cuda_check(e, "cudaGraphInstantiate");
  g.cur_after = cur_;
  cuda_check(cudaGraphLaunch(g.exec, stream()), "cudaGraphLaunch");
}

void Model::ensure_snapshots() {
  if (accu_[0].get()) return;
  const size_t n = static_cast<size_t>(cfg_.n_shots) * geo_.snapshots * grid_size();
  synchronize();
  for (auto &a : accu_) a.allocate(n * elem());
  if (tma_ok_) build_descs();
}

size_t Model::device_bytes() const {
  size_t total = 0;
  auto add = [&](const DeviceBuffer &b) { total += b.bytes(); };
  for (auto &b : fields_) add(b);
  for (auto &b : fields2_) add(b);
  for (auto &b : accu_) add(b);
  for (auto &b : klame_) add(b);
  for (auto &b : kvel_) add(b);
  for (int k = 0; k < 2; ++k) {
    add(rtf_[k]);
    add(rtf_true_[k]);
    add(a_stf_[k]);
  }
  add(lm_);
  add(la_);
  add(mu_);
  add(b_);
  add(vp_);
  add(vs_);
  add(rho_);
  add(rec_raw_);
  add(stf_d_);
  for (auto &b : plan_terms_) add(b);
  for (auto &b : plan_maps_) add(b);
  return total;
}

SolverArgs Model::solver_args() {
  SolverArgs a;
  a.nx = geo_.nx;
  a.nz = geo_.nz;
  a.pitch = pitch_;
  a.nt = cfg_.nt;
  a.np = cfg_.np_boundary;
  a.si = cfg_.snapshot_interval;
  a.snapshots = geo_.snapshots;
  a.nr = cfg_.nr;
  a.dt = cfg_.dt;
  a.dx = cfg_.dx;
  a.dz = cfg_.dz;
  a.vx = fields_[0].get();
  a.vz = fields_[1].get();
  a.txx = fields_[2].get();
  a.tzz = fields_[3].get();
  a.txz = fields_[4].get();
  a.lm = lm_.get();
  a.la = la_.get();
  a.mu = mu_.get();
  a.b = b_.get();
  a.taper_tab = taper_tab_d_.get();
  for (int k = 0; k < 5; ++k) a.accu[k] = accu_[k].get();
  a.rec_cell = rec_cell_.as<int>();
  a.rec_raw = rec_raw_.get();
  a.rtf_ux = rtf_[0].as<double>();
  a.rtf_uz = rtf_[1].as<double>();
  a.a_stf_ux = a_stf_[0].as<double>();
  a.a_stf_uz = a_stf_[1].as<double>();
  a.stf = stf_d_.as<double>();
  a.k_lam = klame_[0].as<double>();
  a.k_mu = klame_[1].as<double>();
  a.k_rho = klame_[2].as<double>();
  a.fx0 = geo_.fx0;
  a.fx1 = geo_.fx1;
  a.fz0 = geo_.fz0;
  a.fz1 = geo_.fz1;
  return a;
}

void Model::synchronize() {
  DeviceGuard guard(device_);
  cuda_check(cudaStreamSynchronize(stream()), "cudaStreamSynchronize");
}

void Model::finish(const char *what) {
  cuda_check(cudaGetLastError(), what);
  if (!async_) synchronize();
}

void Model::widen(size_t n, const void *src, double *dst) {
  cuda_check(prec_ == PSV_FP64 ? widen_f64(n, src, dst, stream()) : widen_f32(n, src, dst, stream()),
             "widen");
}

// ----------------------------------------------------------- simulation --

void Model::forward_simulate(int shot, bool store, bool verbose, bool output_wavefields,
                             int n_steps) {
  if (shot < 0 || shot >= cfg_.n_shots) throw Error(PSV_ERR_INVALID_ARGUMENT, "i_shot out of range");
  if (n_steps < 0 || n_steps > cfg_.nt) n_steps = cfg_.nt;
  DeviceGuard guard(device_);
  if (store) ensure_snapshots();
  SolverArgs a = solver_args();
  const InjPlan &plan = plans_[shot];
  auto t0 = std::chrono::steady_clock::now();
  void *second[5] = {fields2_[0].get(), fields2_[1].get(), fields2_[2].get(), fields2_[3].get(),
                     fields2_[4].get()};
  auto run = [&](int it0, int it1, bool zero, bool fin) {
    cudaError_t e;
    if (prec_ == PSV_FP64)
      e = forward_f64(a, plan, shot, store, it0, it1, zero, fin, stream());
    else if (is_tma())
      e = tma_forward(shot, store, it0, it1, zero, fin, nullptr);
    else if (variant_ == kFused)
      e = fast::forward(a, second, &cur_, plan, shot, store, it0, it1, zero, fin, stream());
    else
      e = forward_f32(a, plan, shot, store, it0, it1, zero, fin, stream());
    if (zero && (prec_ == PSV_FP64 || variant_ == kTwoKernel)) cur_ = 0;
    cuda_check(e, "forward_simulate");
  };
  if (!output_wavefields) {
    run_loop(0, shot, store, n_steps, [&] { run(0, n_steps, true, true); });
  } else {
    // Text dumps of vx, vz after every 10th step (src/fdModel.cpp:753-776).
    for (int it0 = 0; it0 < n_steps; it0 += 10) {
      const int it1 = std::min(n_steps, it0 + 1);
      run(it0, it1, it0 == 0, false);
      dump_wavefields_text(it0);
      if (it1 < std::min(n_steps, it0 + 10)) run(it1, std::min(n_steps, it0 + 10), false, false);
    }
    run(n_steps, n_steps, false, true);
  }
  finish("forward_simulate");
  if (!async_ && is_tma()) check_device_error();
  if (verbose) {
    synchronize();
    double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::cout << "Seconds elapsed for forward wave simulation: " << s << std::endl;
  }
}

int Model::profile_forward(int shot, int n_steps, double *per_step_ms, double *kernel_ms,
                           int max_kernels) {
  if (shot < 0 || shot >= cfg_.n_shots) throw Error(PSV_ERR_INVALID_ARGUMENT, "i_shot out of range");
  if (n_steps <= 0 || n_steps > cfg_.nt) n_steps = cfg_.nt;
  DeviceGuard guard(device_);
  const int kps = kernels_per_step();
  const int per = kps + 1;
  std::vector<cudaEvent_t> ev(static_cast<size_t>(per) * n_steps);
  for (auto &e : ev) cuda_check(cudaEventCreate(&e), "cudaEventCreate");
  SolverArgs a = solver_args();
  a.events = ev.data();
  void *second[5] = {fields2_[0].get(), fields2_[1].get(), fields2_[2].get(), fields2_[3].get(),
                     fields2_[4].get()};
  cudaError_t err;
  if (variant_ == kFusedTmaPersistent || variant_ == kFusedCluster) {
    // One launch for all steps: time it whole; the per-step figure is its
    // share.
    cudaEventRecord(ev.front(), stream());
    err = tma_forward(shot, false, 0, n_steps, true, false, nullptr);
    cudaEventRecord(ev.back(), stream());
    cudaError_t sync = cudaStreamSynchronize(stream());
    float ms = 0;
    if (err == cudaSuccess && sync == cudaSuccess) cudaEventElapsedTime(&ms, ev.front(), ev.back());
    for (auto &e : ev) cudaEventDestroy(e);
    cuda_check(err, "profile_forward");
    cuda_check(sync, "profile_forward");
    if (per_step_ms) *per_step_ms = ms / n_steps;
    if (kernel_ms && max_kernels > 0) kernel_ms[0] = ms / n_steps;
    return 1;
  }
  if (prec_ == PSV_FP64)
    err = forward_f64(a, plans_[shot], shot, false, 0, n_steps, true, false, stream());
  else if (variant_ == kFusedTma)
    err = tma_forward(shot, false, 0, n_steps, true, false, a.events);
  else if (variant_ == kFused)
    err = fast::forward(a, second, &cur_, plans_[shot], shot, false, 0, n_steps, true, false,
                        stream());
  else
    err = forward_f32(a, plans_[shot], shot, false, 0, n_steps, true, false, stream());
  cudaError_t sync = cudaStreamSynchronize(stream());
  std::vector<double> sums(kps, 0.0);
  double total = 0;
  if (err == cudaSuccess && sync == cudaSuccess) {
    for (int s = 0; s < n_steps; ++s) {
      for (int k = 0; k < kps; ++k) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ev[per * s + k], ev[per * s + k + 1]);
        sums[k] += ms;
      }
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, ev.front(), ev.back());
    total = ms;
  }
  for (auto &e : ev) cudaEventDestroy(e);
  cuda_check(err, "profile_forward");
  cuda_check(sync, "profile_forward");
  if (per_step_ms) *per_step_ms = total / n_steps;
  for (int k = 0; k < kps && k < max_kernels; ++k)
    if (kernel_ms) kernel_ms[k] = sums[k] / n_steps;
  return kps;
}

void Model::set_variant(int v) {
  if (v != kFused && v != kTwoKernel && v != kFusedTma && v != kFusedTmaPersistent &&
      v != kFusedCluster)
    throw Error(PSV_ERR_INVALID_ARGUMENT, "unknown kernel variant");
  if (prec_ == PSV_FP64 && v != kTwoKernel)
    throw Error(PSV_ERR_INVALID_ARGUMENT, "the fused variants are FP32 only");
  if ((v == kFusedTma || v == kFusedTmaPersistent || v == kFusedCluster) && !tma_ok_)
    throw Error(PSV_ERR_INVALID_ARGUMENT, "the TMA variant needs driver tensor-map support");
  if (v == kFusedCluster && cluster_nc_ == 0)
    throw Error(PSV_ERR_INVALID_ARGUMENT,
                "the grid does not fit in the shared memory of one thread-block cluster");
  DeviceGuard guard(device_);
  if ((v == kTwoKernel) != (variant_ == kTwoKernel) && cur_ == 1) {
    // Bring the current state back into the primary buffers.
    for (int f = 0; f < 5; ++f)
      cuda_check(cudaMemcpyAsync(fields_[f].get(), fields2_[f].get(), fields_[f].bytes(),
                                 cudaMemcpyDeviceToDevice, stream()),
                 "set_variant");
    cur_ = 0;
  }
  variant_ = v;
  clear_graphs();
  synchronize();
}

const char *Model::step_kernel_name(int k) const {
  if (variant_ == kFused) return k == 0 ? "fused_step" : "";
  if (variant_ == kFusedTma) return k == 0 ? "fused_step_tma" : "";
  if (variant_ == kFusedTmaPersistent) return k == 0 ? "fused_steps_tma" : "";
  if (variant_ == kFusedCluster) return k == 0 ? "cluster_steps" : "";
  return k == 0 ? "stress_step" : (k == 1 ? "velocity_step" : "");
}

void Model::adjoint_simulate(int shot, bool verbose) {
  if (shot < 0 || shot >= cfg_.n_shots) throw Error(PSV_ERR_INVALID_ARGUMENT, "i_shot out of range");
  DeviceGuard guard(device_);
  ensure_snapshots();
  SolverArgs a = solver_args();
  auto t0 = std::chrono::steady_clock::now();
  void *second[5] = {fields2_[0].get(), fields2_[1].get(), fields2_[2].get(), fields2_[3].get(),
                     fields2_[4].get()};
  run_loop(1, shot, true, cfg_.nt, [&] {
    cudaError_t e;
    if (prec_ == PSV_FP64) {
      e = adjoint_f64(a, plans_[cfg_.n_shots], shot, stream());
      cur_ = 0;
    } else if (is_tma()) {
      e = tma_adjoint(shot);
    } else if (variant_ == kFused) {
      e = fast::adjoint(a, second, &cur_, plans_[cfg_.n_shots], shot, stream());
    } else {
      e = adjoint_f32(a, plans_[cfg_.n_shots], shot, stream());
      cur_ = 0;
    }
    cuda_check(e, "adjoint_simulate");
  });
  finish("adjoint_simulate");
  if (!async_ && is_tma()) check_device_error();
  if (verbose) {
    synchronize();
    double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::cout << "Seconds elapsed for adjoint wave simulation: " << s << std::endl;
  }
}

double Model::calculate_l2_misfit() {
  DeviceGuard guard(device_);
  const size_t n = data_size();
  int parts = static_cast<int>(std::min<size_t>(kPartials, (n + 255) / 256));
  if (parts < 1) parts = 1;
  cuda_check(misfit_l2(n, cfg_.dt, rtf_true_[0].as<double>(), rtf_[0].as<double>(),
                       rtf_true_[1].as<double>(), rtf_[1].as<double>(), partials_.as<double>(),
                       parts, scalar_.as<double>(), stream()),
             "calculate_l2_misfit");
  double out = 0;
  cuda_check(cudaMemcpyAsync(&out, scalar_.get(), sizeof(double), cudaMemcpyDeviceToHost, stream()),
             "misfit copy");
  synchronize();
  misfit_ = out;
  return out;
}

void Model::calculate_l2_adjoint_sources() {
  DeviceGuard guard(device_);
  cuda_check(adjoint_sources_l2(data_size(), rtf_[0].as<double>(), rtf_true_[0].as<double>(),
                                rtf_[1].as<double>(), rtf_true_[1].as<double>(),
                                a_stf_[0].as<double>(), a_stf_[1].as<double>(), stream()),
             "calculate_l2_adjoint_sources");
  finish("calculate_l2_adjoint_sources");
}

void Model::reset_kernels() {
  DeviceGuard guard(device_);
  for (auto &k : klame_)
    cuda_check(cudaMemsetAsync(k.get(), 0, k.bytes(), stream()), "reset_kernels");
  finish("reset_kernels");
}

void Model::map_kernels_to_velocity() {
  DeviceGuard guard(device_);
  cuda_check(map_kernels(grid_size(), vp_.as<double>(), vs_.as<double>(), rho_.as<double>(),
                         klame_[0].as<double>(), klame_[1].as<double>(), klame_[2].as<double>(),
                         kvel_[0].as<double>(), kvel_[1].as<double>(), kvel_[2].as<double>(),
                         stream()),
             "map_kernels_to_velocity");
  finish("map_kernels_to_velocity");
}

void Model::run_model(bool verbose, bool simulate_adjoint) {
  if (!verbose && run_model_lanes_ok()) {
    run_model_lanes(simulate_adjoint);
    return;
  }
  const bool was_async = async_;
  async_ = true;
  try {
    for (int s = 0; s < cfg_.n_shots; ++s) forward_simulate(s, true, verbose, false);
    calculate_l2_misfit();
    if (simulate_adjoint) {
      calculate_l2_adjoint_sources();
      reset_kernels();
      for (int s = 0; s < cfg_.n_shots; ++s) adjoint_simulate(s, verbose);
      map_kernels_to_velocity();
    }
  } catch (...) {
    async_ = was_async;
    throw;
  }
  async_ = was_async;
  finish("run_model");
}

void Model::update_from_velocity() {
  DeviceGuard guard(device_);
  cudaError_t e =
      prec_ == PSV_FP64
          ? medium_f64(geo_.nx, geo_.nz, pitch_, vp_.as<double>(), vs_.as<double>(),
                       rho_.as<double>(), lm_.get(), la_.get(), mu_.get(), b_.get(), stream())
          : medium_f32(geo_.nx, geo_.nz, pitch_, vp_.as<double>(), vs_.as<double>(),
                       rho_.as<double>(), lm_.get(), la_.get(), mu_.get(), b_.get(), stream());
  cuda_check(e, "update_from_velocity");
  finish("update_from_velocity");
}

// ------------------------------------------------------------ transfers --

void Model::get_parameter_fields(double *vp, double *vs, double *rho) {
  DeviceGuard guard(device_);
  const size_t bytes = grid_size() * sizeof(double);
  double *out[3] = {vp, vs, rho};
  DeviceBuffer *src[3] = {&vp_, &vs_, &rho_};
  for (int k = 0; k < 3; ++k)
    if (out[k])
      cuda_check(cudaMemcpyAsync(out[k], src[k]->get(), bytes, cudaMemcpyDeviceToHost, stream()),
                 "get_parameter_fields");
  synchronize();
}

void Model::set_parameter_fields(const double *vp, const double *vs, const double *rho,
                                 bool device_pointers) {
  DeviceGuard guard(device_);
  const size_t bytes = grid_size() * sizeof(double);
  const double *in[3] = {vp, vs, rho};
  DeviceBuffer *dst[3] = {&vp_, &vs_, &rho_};
  for (int k = 0; k < 3; ++k)
    cuda_check(cudaMemcpyAsync(dst[k]->get(), in[k], bytes,
                               device_pointers ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               stream()),
               "set_parameter_fields");
  update_from_velocity();
}

void Model::load_model(const std::string &de_path, const std::string &vp_path,
                       const std::string &vs_path, bool verbose) {
  std::ifstream de(de_path), vp(vp_path), vs(vs_path);
  if (verbose) {
    std::cout << "Loading models." << std::endl;
    std::cout << "File: " << de_path << std::endl
              << "File for density is " << (de.good() ? "good (exists at least)." : "ungood.")
              << std::endl;
    std::cout << "File: " << vp_path << std::endl
              << "File for P-wave velocity is "
              << (vp.good() ? "good (exists at least)." : "ungood.") << std::endl;
    std::cout << "File: " << vs_path << std::endl
              << "File for S-wave velocity is "
              << (vs.good() ? "good (exists at least)." : "ungood.") << std::endl;
  }
  if (!de.good() || !vp.good() || !vs.good())
    throw Error(PSV_ERR_IO, "The files for target models don't seem to exist.\r\nPaths:\r\n"
                            "\tDensity target: " + de_path + "\r\n\tP-wave target : " + vp_path +
                                "\r\n\tS-wave target : " + vs_path + "\r\n");
  const size_t n = grid_size();
  std::vector<double> r(n), p(n), s(n);
  for (size_t i = 0; i < n; ++i) {
    de >> r[i];
    vp >> p[i];
    vs >> s[i];
    if (!de.good() || !vp.good() || !vs.good())
      throw Error(PSV_ERR_IO,
                  "Received bad state of one of the files at end of reading. Does the data match "
                  "the domain?");
  }
  double extra;
  de >> extra;
  vp >> extra;
  vs >> extra;
  if (de.good() || vp.good() || vs.good()) throw Error(PSV_ERR_IO, "Too much data is present!");
  set_parameter_fields(p.data(), s.data(), r.data(), false);
  synchronize();
}

void Model::get_kernels(double *vp_k, double *vs_k, double *rho_k, bool device_pointers) {
  DeviceGuard guard(device_);
  const size_t bytes = grid_size() * sizeof(double);
  double *out[3] = {vp_k, vs_k, rho_k};
  for (int k = 0; k < 3; ++k)
    if (out[k])
      cuda_check(cudaMemcpyAsync(out[k], kvel_[k].get(), bytes,
                                 device_pointers ? cudaMemcpyDeviceToDevice
                                                 : cudaMemcpyDeviceToHost,
                                 stream()),
                 "get_kernels");
  if (!device_pointers) synchronize();
}

void Model::get_lame_kernels(double *lam, double *mu, double *rho) {
  DeviceGuard guard(device_);
  const size_t bytes = grid_size() * sizeof(double);
  double *out[3] = {lam, mu, rho};
  for (int k = 0; k < 3; ++k)
    if (out[k])
      cuda_check(cudaMemcpyAsync(out[k], klame_[k].get(), bytes, cudaMemcpyDeviceToHost, stream()),
                 "get_lame_kernels");
  synchronize();
}

void Model::get_data(int which, double *ux, double *uz, bool device_pointers) {
  DeviceGuard guard(device_);
  DeviceBuffer *src = which == kSynthetic ? rtf_ : which == kObserved ? rtf_true_ : a_stf_;
  const size_t bytes = data_size() * sizeof(double);
  double *out[2] = {ux, uz};
  for (int k = 0; k < 2; ++k)
    if (out[k] && bytes)
      cuda_check(cudaMemcpyAsync(out[k], src[k].get(), bytes,
                                 device_pointers ? cudaMemcpyDeviceToDevice
                                                 : cudaMemcpyDeviceToHost,
                                 stream()),
                 "get data");
  if (!device_pointers) synchronize();
}

void Model::set_data(int which, const double *ux, const double *uz, bool device_pointers) {
  DeviceGuard guard(device_);
  DeviceBuffer *dst = which == kSynthetic ? rtf_ : which == kObserved ? rtf_true_ : a_stf_;
  const size_t bytes = data_size() * sizeof(double);
  const double *in[2] = {ux, uz};
  for (int k = 0; k < 2; ++k)
    if (bytes)
      cuda_check(cudaMemcpyAsync(dst[k].get(), in[k], bytes,
                                 device_pointers ? cudaMemcpyDeviceToDevice
                                                 : cudaMemcpyHostToDevice,
                                 stream()),
                 "set data");
  finish("set data");
}

void Model::get_snapshots(double *out[5]) {
  DeviceGuard guard(device_);
  ensure_snapshots();
  const size_t n = static_cast<size_t>(cfg_.n_shots) * geo_.snapshots * grid_size();
  const size_t chunk = std::min<size_t>(n, size_t(1) << 24);
  DeviceBuffer tmp;
  if (prec_ != PSV_FP64) tmp.allocate(chunk * sizeof(double));
  for (int f = 0; f < 5; ++f) {
    if (!out[f]) continue;
    for (size_t off = 0; off < n; off += chunk) {
      const size_t m = std::min(chunk, n - off);
      if (prec_ == PSV_FP64) {
        cuda_check(cudaMemcpyAsync(out[f] + off, accu_[f].as<double>() + off, m * sizeof(double),
                                   cudaMemcpyDeviceToHost, stream()),
                   "get_snapshots");
      } else {
        widen(m, accu_[f].as<float>() + off, tmp.as<double>());
        cuda_check(cudaMemcpyAsync(out[f] + off, tmp.get(), m * sizeof(double),
                                   cudaMemcpyDeviceToHost, stream()),
                   "get_snapshots");
      }
      synchronize();
    }
  }
}

void Model::get_wavefields(double *out[5]) {
  DeviceGuard guard(device_);
  const size_t n = grid_size();
  DeviceBuffer *cur = (prec_ == PSV_FP32 && cur_ == 1) ? fields2_ : fields_;
  DeviceBuffer tmp;
  tmp.allocate(n * sizeof(double));
  for (int f = 0; f < 5; ++f) {
    if (!out[f]) continue;
    cudaError_t e = prec_ == PSV_FP64
                        ? unpad_f64(geo_.nx, geo_.nz, pitch_, cur[f].get(), tmp.as<double>(), stream())
                        : unpad_f32(geo_.nx, geo_.nz, pitch_, cur[f].get(), tmp.as<double>(), stream());
    cuda_check(e, "get_wavefields");
    cuda_check(cudaMemcpyAsync(out[f], tmp.get(), n * sizeof(double), cudaMemcpyDeviceToHost,
                               stream()),
               "get_wavefields");
    synchronize();
  }
}

void Model::get_stf(double *out) const { std::copy(stf_.begin(), stf_.end(), out); }
void Model::get_moment(double *out) const { std::copy(moment_.begin(), moment_.end(), out); }

void Model::set_stf(const double *stf) {
  DeviceGuard guard(device_);
  for (size_t i = 0; i < stf_.size(); ++i)
    if (!std::isfinite(stf[i])) throw Error(PSV_ERR_INVALID_ARGUMENT, "stf must be finite");
  synchronize();  // work in flight reads the device copy
  std::copy(stf, stf + stf_.size(), stf_.begin());
  if (!stf_.empty())
    cuda_check(cudaMemcpy(stf_d_.get(), stf_.data(), stf_.size() * sizeof(double),
                          cudaMemcpyHostToDevice),
               "upload stf");
}

void Model::set_moment(const double *moment) {
  DeviceGuard guard(device_);
  for (size_t i = 0; i < moment_.size(); ++i)
    if (!std::isfinite(moment[i])) throw Error(PSV_ERR_INVALID_ARGUMENT, "moment must be finite");
  synchronize();
  std::copy(moment, moment + moment_.size(), moment_.begin());
  // The injection terms carry the tensor: rebuild them, and everything that
  // holds their device addresses (descriptors, captured pipelines).
  clear_graphs();
  build_plans();
  if (tma_ok_) build_descs();
}

void Model::get_taper(double *out) const {
  const int nx = geo_.nx, nz = geo_.nz, np = cfg_.np_boundary;
  for (int ix = 0; ix < nx; ++ix)
    for (int iz = 0; iz < nz; ++iz) {
      int c = std::min(std::min(ix + 1, iz + 1), std::min(nx - ix, nz - iz));
      c = std::min(c, np);
      out[static_cast<size_t>(ix) * nz + iz] = taper_tab_[c];
    }
}

// ------------------------------------------------------ model vectors ---

void Model::get_model_vector(double *out) {
  std::vector<double> vp(grid_size()), vs(grid_size()), rho(grid_size());
  get_parameter_fields(vp.data(), vs.data(), rho.data());
  const int npx = cfg_.npx, npz = cfg_.npz, nz = geo_.nz;
  const int bx = geo_.nx_free / npx, bz = geo_.nz_free / npz, per = bx * bz;
  for (int ix = 0; ix < bx; ++ix)
    for (int iz = 0; iz < bz; ++iz) {
      const int p = ix + iz * geo_.nx_free / npx;
      const int gx = ix * npx + cfg_.nx_inner_boundary + cfg_.np_boundary;
      const int gz = iz * npz + cfg_.nz_inner_boundary + cfg_.np_boundary;
      out[p] = out[p + per] = out[p + 2 * per] = 0;
      for (int sx = 0; sx < npx; ++sx)
        for (int sz = 0; sz < npz; ++sz) {
          const size_t i = static_cast<size_t>(gx + sx) * nz + gz + sz;
          out[p] += vp[i] / (npx * npz);
          out[p + per] += vs[i] / (npx * npz);
          out[p + 2 * per] += rho[i] / (npx * npz);
        }
    }
}

void Model::set_model_vector(const double *in) {
  std::vector<double> vp(grid_size()), vs(grid_size()), rho(grid_size());
  get_parameter_fields(vp.data(), vs.data(), rho.data());
  const int npx = cfg_.npx, npz = cfg_.npz, nz = geo_.nz;
  const int bx = geo_.nx_free / npx, bz = geo_.nz_free / npz, per = bx * bz;
  for (int ix = 0; ix < bx; ++ix)
    for (int iz = 0; iz < bz; ++iz) {
      const int p = ix + iz * geo_.nx_free / npx;
      const int gx = ix * npx + cfg_.nx_inner_boundary + cfg_.np_boundary;
      const int gz = iz * npz + cfg_.nz_inner_boundary + cfg_.np_boundary;
      for (int sx = 0; sx < npx; ++sx)
        for (int sz = 0; sz < npz; ++sz) {
          const size_t i = static_cast<size_t>(gx + sx) * nz + gz + sz;
          vp[i] = in[p];
          vs[i] = in[p + per];
          rho[i] = in[p + 2 * per];
        }
    }
  set_parameter_fields(vp.data(), vs.data(), rho.data(), false);
  synchronize();
}

void Model::get_gradient_vector(double *out) {
  std::vector<double> kp(grid_size()), ks(grid_size()), kr(grid_size());
  get_kernels(kp.data(), ks.data(), kr.data(), false);
  const int npx = cfg_.npx, npz = cfg_.npz, nz = geo_.nz;
  const int bx = geo_.nx_free / npx, bz = geo_.nz_free / npz, per = bx * bz;
  for (int ix = 0; ix < bx; ++ix)
    for (int iz = 0; iz < bz; ++iz) {
      const int p = ix + iz * geo_.nx_free / npx;
      const int gx = ix * npx + cfg_.nx_inner_boundary + cfg_.np_boundary;
      const int gz = iz * npz + cfg_.nz_inner_boundary + cfg_.np_boundary;
      out[p] = out[p + per] = out[p + 2 * per] = 0;
      for (int sx = 0; sx < npx; ++sx)
        for (int sz = 0; sz < npz; ++sz) {
          const size_t i = static_cast<size_t>(gx + sx) * nz + gz + sz;
          out[p] += kp[i];
          out[p + per] += ks[i];
          out[p + 2 * per] += kr[i];
        }
    }
}

void Model::load_vector(const std::string &path, bool verbose, double *out) const {
  const int n = 3 * geo_.nx_free * geo_.nz_free;
  std::ifstream f(path);
  if (verbose)
    std::cout << "Loading model vector." << std::endl
              << "File: " << path << std::endl
              << "File is " << (f.good() ? "good (exists at least)." : "ungood.") << std::endl;
  if (!f.good())
    throw Error(PSV_ERR_IO, "The files for target models don't seem to exist.\r\nPaths:\r\n"
                            "\tDensity target: " + path + "\r\n");
  for (int i = 0; i < n; ++i) f >> out[i];
  if (!f.good()) throw Error(PSV_ERR_IO, "Not enough data is present!");
  double extra;
  f >> extra;
  if (f.good()) throw Error(PSV_ERR_IO, "Too much data is present!");
}

// ------------------------------------------------------------ geometry --

void Model::get_sources(bool in_units, bool include_boundary, double *x, double *z) const {
  for (int i = 0; i < cfg_.n_sources; ++i) {
    x[i] = ix_src_[i];
    z[i] = iz_src_[i];
    if (!include_boundary || in_units) {
      x[i] -= cfg_.np_boundary;
      z[i] -= cfg_.np_boundary;
      if (in_units) {
        x[i] *= cfg_.dx;
        z[i] *= cfg_.dz;
      }
    }
  }
}

void Model::get_receivers(bool in_units, bool include_boundary, double *x, double *z) const {
  for (int i = 0; i < cfg_.nr; ++i) {
    x[i] = ix_rec_[i];
    z[i] = iz_rec_[i];
    if (!include_boundary || in_units) {
      x[i] -= cfg_.np_boundary;
      z[i] -= cfg_.np_boundary;
      if (in_units) {
        x[i] *= cfg_.dx;
        z[i] *= cfg_.dz;
      }
    }
  }
}

void Model::get_coordinates(bool in_units, double *ix_out, double *iz_out) const {
  const int nx = geo_.nx, nz = geo_.nz, np = cfg_.np_boundary;
  for (int ix = 0; ix < nx; ++ix)
    for (int iz = 0; iz < nz; ++iz) {
      const size_t i = static_cast<size_t>(ix) * nz + iz;
      if (in_units) {
        ix_out[i] = (ix - np) * cfg_.dx;
        iz_out[i] = (iz - np) * cfg_.dz;
      } else {
        ix_out[i] = ix;
        iz_out[i] = iz;
      }
    }
}

void Model::get_extent(bool include_boundary, double *o) const {
  if (include_boundary) {
    o[0] = -cfg_.np_boundary;
    o[1] = cfg_.dx * (cfg_.nx_inner + cfg_.np_boundary);
    o[2] = -cfg_.np_boundary;
    o[3] = cfg_.dz * (cfg_.nz_inner + cfg_.np_boundary);
  } else {
    o[0] = 0;
    o[1] = cfg_.dx * cfg_.nx_inner;
    o[2] = 0;
    o[3] = cfg_.dz * cfg_.nz_inner;
  }
}

// ------------------------------------------------------------ text I/O --

void Model::write_receivers(const std::string &) {
  // The reference accepts a prefix but writes to the same names regardless
  // (src/fdModel.cpp:973-1006).
  std::vector<double> ux(data_size()), uz(data_size());
  get_data(kSynthetic, ux.data(), uz.data(), false);
  const int nr = cfg_.nr, nt = cfg_.nt;
  for (int s = 0; s < cfg_.n_shots; ++s) {
    std::ofstream fx(cfg_.observed_data_folder + "/rtf_ux" + std::to_string(s) + ".txt");
    std::ofstream fz(cfg_.observed_data_folder + "/rtf_uz" + std::to_string(s) + ".txt");
    if (!fx.good() || !fz.good()) throw Error(PSV_ERR_IO, "cannot write receiver files");
    fx.precision(std::numeric_limits<double>::digits10 + 10);
    fz.precision(std::numeric_limits<double>::digits10 + 10);
    for (int r = 0; r < nr; ++r) {
      fx << std::endl;
      fz << std::endl;
      for (int it = 0; it < nt; ++it) {
        const size_t i = (static_cast<size_t>(s) * nr + r) * nt + it;
        fx << ux[i] << " ";
        fz << uz[i] << " ";
      }
    }
  }
}

void Model::load_receivers(bool verbose) {
  const int nr = cfg_.nr, nt = cfg_.nt;
  std::vector<double> ux(data_size()), uz(data_size());
  for (int s = 0; s < cfg_.n_shots; ++s) {
    std::ifstream fx(cfg_.observed_data_folder + "/rtf_ux" + std::to_string(s) + ".txt");
    std::ifstream fz(cfg_.observed_data_folder + "/rtf_uz" + std::to_string(s) + ".txt");
    if (verbose) {
      std::cout << "File for ux data at shot " << s << " is "
                << (fx.good() ? "good (exists at least)." : "ungood.") << std::endl;
      std::cout << "File for uz data at shot " << s << " is "
                << (fz.good() ? "good (exists at least)." : "ungood.") << std::endl;
    }
    if (!fx.good() || !fz.good()) throw Error(PSV_ERR_IO, "Not all data is present!");
    for (int r = 0; r < nr; ++r)
      for (int it = 0; it < nt; ++it) {
        const size_t i = (static_cast<size_t>(s) * nr + r) * nt + it;
        fx >> ux[i];
        fz >> uz[i];
      }
    if (!fx.good() || !fz.good()) throw Error(PSV_ERR_IO, "Not enough data is present!");
    double extra;
    fx >> extra;
    fz >> extra;
    if (fx.good() || fz.good()) throw Error(PSV_ERR_IO, "Too much data is present!");
  }
  set_data(kObserved, ux.data(), uz.data(), false);
  synchronize();
}

void Model::write_sources() const {
  const int nt = cfg_.nt;
  for (int s = 0; s < cfg_.n_shots; ++s) {
    std::ofstream f(cfg_.stf_folder + "/sources_shot_" + std::to_string(s) + ".txt");
    if (!f.good()) throw Error(PSV_ERR_IO, "cannot write source files");
    f.precision(std::numeric_limits<double>::digits10 + 10);
    for (int src : cfg_.shots[s]) {
      f << std::endl;
      for (int it = 0; it < nt; ++it) f << stf_[static_cast<size_t>(src) * nt + it] << " ";
    }
  }
}

void Model::write_kernels() {
  const size_t n = grid_size();
  std::vector<double> kp(n), ks(n), kr(n);
  get_kernels(kp.data(), ks.data(), kr.data(), false);
  std::ofstream fp("kernel_vp.txt"), fs("kernel_vs.txt"), fr("kernel_density.txt");
  if (!fp.good() || !fs.good() || !fr.good()) throw Error(PSV_ERR_IO, "cannot write kernel files");
  for (int ix = 0; ix < geo_.nx; ++ix) {
    for (int iz = 0; iz < geo_.nz; ++iz) {
      const size_t i = static_cast<size_t>(ix) * geo_.nz + iz;
      fp << kp[i] << " ";
      fs << ks[i] << " ";
      fr << kr[i] << " ";
    }
    fp << std::endl;
    fs << std::endl;
    fr << std::endl;
  }
}

void Model::dump_wavefields_text(int it) {
  std::vector<double> vx(grid_size()), vz(grid_size());
  double *out[5] = {vx.data(), vz.data(), nullptr, nullptr, nullptr};
  get_wavefields(out);
  std::ofstream fx("snapshots/vx" + pad5(it) + ".txt"), fz("snapshots/vz" + pad5(it) + ".txt");
  for (int ix = 0; ix < geo_.nx; ++ix) {
    for (int iz = 0; iz < geo_.nz; ++iz) {
      const size_t i = static_cast<size_t>(ix) * geo_.nz + iz;
      fx << vx[i] << " ";
      fz << vz[i] << " ";
    }
    fx << std::endl;
    fz << std::endl;
  }
}

}  // namespace psv
