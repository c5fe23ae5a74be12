#!/usr/bin/env python
"""Benchmark of the P-SV forward solver: Gcell-updates/s on the 2100 x 900
grid (2000 x 800 inner cells + 50-cell Cerjan boundary), 5000 time steps,
400 receivers, one explosive + dip source, FP32 wave fields, seeded layered
Gaussian-random medium (psvwave_gb300/workloads.py, c1).

A step is one complete forward simulation (forward_simulate of shot 0, no
snapshot storage): nx * nz * nt cell-updates. One cell-update is both
half-steps at one grid point, counted over the full grid incl. boundary.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Under torchrun (N > 1) every rank advances its own copy of the model
(independent shots of the same survey; no data-path collective), so the
scaling is weak and `value` sums the ranks' cell-updates over the slowest
rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gcell-updates/s"
# FP32 algorithmic bytes per cell-update of each step kernel: reads and writes
# of the fields, medium and buoyancy per point and step, at one visit each
BYTES_PER_CELL = {"stress_step": 48, "velocity_step": 36, "fused_step": 56, "fused_step_tma": 52,
                  "fused_steps_tma": 52}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-secondary", action="store_true",
                   help="skip the FWI-gradient and batching measurements")
    p.add_argument("--ncu-case", type=int, default=0, metavar="NT",
                   help="run one NT-step forward of the c1 workload and exit (for ncu captures)")
    p.add_argument("--ncu-case-small", type=int, default=0, metavar="NT",
                   help="run one NT-step forward of the c0 workload (the default scheme there: "
                        "cluster-resident), launch by launch, and exit (for ncu captures)")
    p.add_argument("--ncu-case-exact", type=int, default=0, metavar="NT",
                   help="run one exact gradient of one NT-step shot of the c3 workload, launch by "
                        "launch, and exit (for ncu captures)")
    p.add_argument("--ncu-case-c4judge", type=int, default=0, metavar="SHAPE",
                   help="run one batched forward of the c4 judge (128 members) with the tile "
                        "shape given by index (0 32x60, 1 16x28, 2 20x28, 3 16x60; one launch "
                        "per step) and exit (for ncu captures)")
    p.add_argument("--ncu-case-cnn", type=int, default=0, metavar="B",
                   help="run two surrogate-network predictions and one training step at B states "
                        "and exit (for ncu captures)")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def measured_traffic(kernel):
    """DRAM bytes (read + write) per launch of `kernel` from the warm-cache
    ncu capture summarised in profiles/<kernel>_c1.json, or None."""
    path = os.path.join(ROOT, "profiles", "%s_c1.json" % kernel)
    try:
        with open(path) as f:
            return float(json.load(f)["dram_bytes_per_launch"])
    except Exception:
        return None


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def cpu_baseline(params_fn, media, seconds=12.0, moment=None):
    """The oracle port (the reference's algorithm in C/OpenMP) on a bounded
    sample of the workload: the same grid, source and medium, fewer time
    steps."""
    from oracle import portbind

    def run(n):
        p = params_fn(nt=n)
        p["snapshot_interval"] = n
        o = portbind.OracleModel(params=p)
        if moment is not None:
            o.view("moment")[...] = moment
        o.set_parameter_fields(*media)
        t = time.perf_counter()
        o.forward_simulate(0, False)
        return time.perf_counter() - t, o.nx, o.nz

    dt0, nx, nz = run(20)
    cells = nx * nz
    rate = cells * 20 / dt0
    n = int(max(20, min(5000, seconds * rate / cells)))
    n -= n % 10
    dt, nx, nz = run(n)
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": cells * n / dt / 1e9, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": "oracle port (C, OpenMP) forward on the c1 grid %dx%d and medium, "
                      "%d of 5000 time steps, %.1f s" % (nx, nz, n, dt)}


def fwi_gradients(steps, warmup, with_cpu):
    """FWI gradients/s on the c0 workload: observed data from the target
    medium, then each step is one full gradient at the start medium
    (run_model: forward with snapshots, misfit, adjoint sources, kernel
    reset, adjoint with kernel correlation, velocity mapping; FP32 wave fields,
    FP64 misfit and kernels), timed end to end with the model's stream
    synchronised, plus the gradient vector read back to the host."""
    import psvwave_gb300 as psv
    from psvwave_gb300 import workloads

    p = workloads.c0_params()
    target, start = workloads.c0_media()

    def rate(precision):
        m = psv.fdModel.from_parameters(p, precision=precision)
        m.set_parameter_fields(*target)
        for s_ in range(m.n_shots):
            m.forward_simulate(s_, False)
        m.set_observed_data(*m.get_synthetic_data())
        m.set_parameter_fields(*start)
        for _ in range(warmup):
            m.run_model(False, True)
        t0 = time.perf_counter()
        for _ in range(steps):
            m.run_model(False, True)
            m.get_gradient_vector()
        return m, time.perf_counter() - t0

    m, dt = rate("fp32")
    m64, dt64 = rate("fp64")
    out = {"value": steps / dt, "unit": "FWI gradients/s",
           "workload": "c0: 250x150 grid, nt=4000, 2 sources in 1 shot, 19 receivers, "
                       "snapshot interval 10; forward + misfit + adjoint + kernels per gradient",
           "ms_per_gradient": 1e3 * dt / steps, "misfit": m.misfit,
           "tile_shape": m.tile_shape, "kernel_variant": m.kernel_variant,
           "fp64": {"value": steps / dt64, "ms_per_gradient": 1e3 * dt64 / steps,
                    "misfit": m64.misfit,
                    "note": "the reference's precision, bit-identical to it"}}
    if with_cpu:
        from oracle import portbind
        o = portbind.OracleModel(params=p)
        o.set_parameter_fields(*target)
        o.forward_simulate(0, False)
        o.set_observed_data(*o.get_synthetic_data())
        o.set_parameter_fields(*start)
        t0 = time.perf_counter()
        o.run_model(True)
        cdt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / cdt, "unit": "FWI gradients/s",
                               "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
                               "kind": "port", "sample": "one full c0 gradient, %.2f s" % cdt}
        out["cpu_misfit"] = o.misfit
    return out


def fwi_gradients_c3(steps, with_cpu=False):
    """FWI gradients/s on the differentiation workload (1000 x 400 inner
    cells, 8 shots, nt = 6000, FP32 wave fields, FP64 kernel sums): the
    gradient of the L2 misfit through the torch.autograd layer, as the exact
    discrete adjoint with checkpoints every 100 steps and with every state
    kept, and the reference's own adjoint kernels (snapshots every 10 steps).
    Each timed gradient starts from CUDA tensors and ends with the gradient
    in CUDA tensors."""
    import torch

    import psvwave_gb300 as psv
    from psvwave_gb300 import workloads
    from psvwave_gb300.torch_ops import l2_misfit

    p = workloads.c3_params()
    true, start = workloads.c3_media(p)
    m = psv.fdModel.from_parameters(p)
    m.set_parameter_fields(*true)
    for s_ in range(m.n_shots):
        m.forward_simulate(s_, False)
    m.set_observed_data(*m.get_synthetic_data())
    out = {"unit": "FWI gradients/s",
           "workload": "c3: 1100x500 grid (1000x400 inner + 50), 8 shots, nt=6000, 200 receivers, "
                       "Ricker 25 Hz; layered + 3 elliptic vs anomalies, start = 20-cell smoothing"}
    runs = (("checkpoint_100", dict(checkpoint_every=100, mode="exact")),
            ("store_all", dict(checkpoint_every=p["nt"], mode="exact")),
            ("reference_kernels", dict(checkpoint_every=100, mode="reference")))
    for name, kw in runs:
        def one():
            t = [torch.tensor(a, dtype=torch.float64, device="cuda", requires_grad=True)
                 for a in start]
            chi = l2_misfit(m, *t, **kw)
            chi.backward()
            torch.cuda.synchronize()
            return float(chi.detach())

        one()  # warm-up: allocations, eager first run
        one()  # warm-up: per-shot pipelines captured as CUDA graphs
        t0 = time.perf_counter()
        for _ in range(steps):
            chi = one()
        dt = (time.perf_counter() - t0) / steps
        res = {"value": 1.0 / dt, "ms_per_gradient": 1e3 * dt, "misfit": chi}
        if kw["mode"] == "exact":
            res["device_bytes"] = m.exact_bytes(kw["checkpoint_every"])
        out[name] = res
    out["value"] = out["checkpoint_100"]["value"]
    # Algorithmic bytes of one checkpointed gradient: per shot and step two
    # forward steps (checkpoint pass, recompute; 52 B per cell each) and one
    # exact step (98.4 B per cell: 18 words of fields and medium, three FP32
    # partial sums read and written, three float-float pairs on one step in
    # 20).
    cells = float(m.nx * m.nz)
    per_grad = m.n_shots * m.nt * cells * (2 * 52.0 + 98.4)
    peak, kind = measured_peaks()
    t = out["checkpoint_100"]["ms_per_gradient"] / 1e3
    out["roofline"] = {"bound": "hbm", "bytes_per_gradient": per_grad,
                       "achieved": per_grad / t / 1e9, "peak": peak, "unit": "GB/s",
                       "frac": per_grad / t / 1e9 / peak, "peak_source": kind,
                       "note": "whole checkpointed gradient, all kernels, 8 shots in "
                               "concurrent lanes"}
    if with_cpu:
        out["cpu_baseline"] = cpu_baseline_c3()
    return out


def cpu_baseline_c3(n_steps=600):
    """The oracle port (C, OpenMP, all host threads) on a bounded sample of
    the differentiation workload: the reference's gradient (run_model:
    forward with snapshots every 10 steps, misfit, adjoint sources, adjoint
    with kernel correlation, velocity kernels) of one shot over n_steps
    steps on the full 1100 x 500 grid, scaled to a full gradient (8 shots x
    6000 steps)."""
    from oracle import portbind
    from psvwave_gb300 import workloads

    p = workloads.c3_params(nt=n_steps, n_shots=1)
    true, start = workloads.c3_media(workloads.c3_params())
    o = portbind.OracleModel(params=p)
    o.set_parameter_fields(*true)
    o.forward_simulate(0, False)
    o.set_observed_data(*o.get_synthetic_data())
    o.set_parameter_fields(*start)
    t0 = time.perf_counter()
    o.run_model(True)
    t = time.perf_counter() - t0
    full = t * 8 * (6000 / n_steps)
    return {"value": 1.0 / full, "unit": "FWI gradients/s",
            "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)), "kind": "port",
            "sample": "oracle port run_model (reference adjoint kernels), 1 shot x %d steps on "
                      "the c3 grid in %.2f s, scaled x8 shots x%g steps" % (n_steps, t,
                                                                       6000 / n_steps)}


def mc_samples_c4():
    """Accepted MC samples/s on the surrogate workload at its stated size (c0
    grid, 600 coarse parameters): the network trained on 20000 exact
    (model, misfit, gradient) triples plus 1024 local ones, then
    delayed-acceptance HMC over 128 chains x 400 iterations (51200
    proposals) screened by the network, against the same sampler screened
    by the prior alone and against HMC with the solver's exact gradients
    (16 chains x 32 iterations, 512 samples), with posterior summaries of
    the exact samplers (psvwave_gb300.c4)."""
    from psvwave_gb300 import c4

    out = c4.run(n_train=20000, n_local=1024, n_chains=128, n_iter=400, plain_chains=16,
                 plain_iter=32)
    out["unit"] = "accepted samples/s"
    out["workload"] = ("c4: 250x150 grid, nt=2000, Ricker 15 Hz, 600 coarse parameters "
                       "(20x10 vp/vs/rho, prior sigma 10%), s2 = misfit(prior mean)/20; "
                       "20000 training triples, 128 chains x 400 iterations")
    return out


def batched(steps, warmup, rank=0, world=1, with_cpu=False):
    """Aggregate Gcell-updates/s of the batching workload (256 models of
    uneven sizes, 1-4 shots each, nt = 1000): all shots of all models in one
    launch per time step (one CUDA graph), versus the same models run one
    after another, each shot its own forward_simulate. Under torchrun the
    models are split round-robin across the ranks (model k on rank
    k % world, psvwave_gb300.distributed.shard), each rank advancing its
    share in one batch; the rate is the whole set's cell-updates over the
    slowest rank's time (a fixed workload: strong scaling)."""
    import psvwave_gb300 as psv
    from psvwave_gb300 import workloads
    from psvwave_gb300.distributed import shard

    pairs = workloads.c2_models()
    mine = shard(len(pairs), rank, world)
    models = []
    for k in mine:
        p, media = pairs[k]
        m = psv.fdModel.from_parameters(p)
        m.set_parameter_fields(*media)
        models.append(m)
    b = psv.Batch()
    for m in models:
        b.add_all_shots(m)
    shape = b.autotune(50)
    info = b.info()  # after the build, so the tile count is known
    nt = models[0].nt
    for _ in range(max(2, warmup)):
        b.forward()
    b_times = []
    for _ in range(steps):
        if world > 1:
            import torch
            torch.distributed.barrier()
        t0 = time.perf_counter()
        b.forward()
        b_times.append(time.perf_counter() - t0)
    mean_t = sum(b_times) / len(b_times)
    cells = info["cells"]
    if world > 1:
        import torch
        t = torch.tensor([mean_t, cells], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t[:1], op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(t[1:], op=torch.distributed.ReduceOp.SUM)
        mean_t, cells = float(t[0]), float(t[1])
    batched_rate = cells * nt / mean_t / 1e9
    out = {"value": batched_rate, "unit": "Gcell-updates/s",
           "workload": "c2: 256 seeded models, nx_inner U[200,800], nz_inner U[100,400], "
                       "25-cell boundary, 1-4 shots, Ricker 20-50 Hz, nt=1000, forward only",
           "members": info["members"], "cells_per_step": cells, "tiles": info["tiles"],
           "tile_shape": shape, "persistent": b.persistent}
    if world > 1:
        out["parallelism"] = "models round-robin over %d ranks, no collective on the data path" % world
        return out
    for m in models:  # warm the per-model graphs
        for _ in range(2):
            for s_ in range(m.n_shots):
                m.forward_simulate(s_, False)
    t0 = time.perf_counter()
    for m in models:
        for s_ in range(m.n_shots):
            m.forward_simulate(s_, False)
    seq = time.perf_counter() - t0
    seq_rate = cells * nt / seq / 1e9
    out["one_launch_per_model"] = seq_rate
    out["speedup_vs_one_launch_per_model"] = batched_rate / seq_rate
    if with_cpu:
        out["cpu_baseline"] = cpu_baseline_c2(pairs)
    return out


def cpu_baseline_c2(pairs, n_models=4, n_steps=200):
    """The oracle port (C, OpenMP, all host threads) on a bounded sample of
    the batching workload: every shot of the first n_models models, n_steps
    of their 1000 time steps, in Gcell-updates/s."""
    from oracle import portbind

    cells = 0.0
    t = 0.0
    for p, media in pairs[:n_models]:
        q = dict(p)
        q.update(nt=n_steps, snapshot_interval=n_steps)
        o = portbind.OracleModel(params=q)
        o.set_parameter_fields(*media)
        t0 = time.perf_counter()
        for s_ in range(o.n_shots):
            o.forward_simulate(s_, False)
        t += time.perf_counter() - t0
        cells += float(o.nx * o.nz) * n_steps * o.n_shots
    return {"value": cells / t / 1e9, "unit": "Gcell-updates/s",
            "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)), "kind": "port",
            "sample": "oracle port forward, every shot of the first %d c2 models, %d of 1000 "
                      "steps, %.1f s" % (n_models, n_steps, t)}


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return
    from psvwave_gb300 import workloads

    media = workloads.c1_media()
    samples = []
    base = None
    for i in range(args.warmup + args.steps):
        b = cpu_baseline(workloads.c1_params, media, seconds=5.0, moment=workloads.c1_moment())
        if i >= args.warmup:
            samples.append(b["value"])
            base = b
    value = sum(samples) / len(samples)
    base["value"] = value
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded layered medium)",
            "config": {"workload": "c1: 2100x900 grid, nt=5000 (bounded sample per step), "
                                   "400 receivers, forward only"},
            "cpu_baseline": base,
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def ncu_case(nt):
    """A short forward run of the c1 workload, for ncu captures."""
    import psvwave_gb300 as psv
    from psvwave_gb300 import workloads

    m = workloads.c1_model(nt=nt)
    m.forward_simulate(0, False)
    print("ncu case: %s, %s tiles, seismogram sum %.6e" % (
        m.kernel_variant, m.tile_shape, m.get_synthetic_data()[0].sum()))


def ncu_case_small(nt):
    """A short forward of the c0 workload with its default scheme, kernels
    launched one by one (no graph), for ncu captures."""
    import psvwave_gb300 as psv
    from psvwave_gb300 import workloads

    p = workloads.c0_params()
    p["nt"] = nt
    m = psv.fdModel.from_parameters(p)
    m.set_graph_capture(False)
    m.set_parameter_fields(*workloads.c0_media()[0])
    m.forward_simulate(0, False)
    print("ncu small case: %s, seismogram sum %.6e" % (m.kernel_variant,
                                                      m.get_synthetic_data()[0].sum()))


def ncu_case_exact(nt):
    """One exact gradient (checkpoints every 100 steps) of a one-shot, NT-step
    version of the c3 workload, kernels launched one by one (no graph), for
    ncu captures."""
    import psvwave_gb300 as psv
    from psvwave_gb300 import workloads

    true, start = workloads.c3_media(workloads.c3_params())
    m = psv.fdModel.from_parameters(workloads.c3_params(nt=nt, n_shots=1))
    m.set_parameter_fields(*true)
    m.forward_simulate(0, False)
    m.set_observed_data(*m.get_synthetic_data())
    m.set_parameter_fields(*start)
    m.set_graph_capture(False)
    mis, _ = m.exact_gradient(100)
    print("ncu exact case: %s tiles, misfit %.9e" % (m.tile_shape, mis))


def ncu_case_c4judge(shape):
    """One batched forward (2000 steps) of the c4 posterior's judge over its
    128 members at seeded prior states, with tile shape index SHAPE and one
    launch per step, for ncu captures (set-up and tuning launches come
    first)."""
    import torch
    from psvwave_gb300 import surrogate as sg

    S = sg.c4_setup(128, s2=1.0)
    post = S["posterior"]
    post.batch.persistent = False
    post.batch.tile_shape = {0: "32x60", 1: "16x28", 2: "20x28", 3: "16x60"}[shape]
    gen = torch.Generator(device="cuda").manual_seed(0)
    z = 0.5 * torch.randn((128, 3, 20, 10), device="cuda", generator=gen)
    mis = post.misfits(z)
    print("ncu c4 judge case: %s tiles, misfit sum %.9e" % (post.batch.tile_shape, mis.sum()))


def ncu_case_cnn(batch):
    """Two predictions (four tensor-core convolutions and the head each) and
    one Adam step of the c4 surrogate network at BATCH seeded random
    states, for ncu captures."""
    import torch
    from psvwave_gb300 import surrogate as sg

    gen = torch.Generator(device="cuda").manual_seed(0)
    net = sg.SurrogateNet(max_batch=batch, seed=1)
    x = torch.randn(batch, 5, 20, 10, device="cuda", generator=gen)
    m = torch.randn(batch, device="cuda", generator=gen)
    g = torch.randn(batch, 3, 20, 10, device="cuda", generator=gen)
    for _ in range(2):
        mp, _ = net.predict_features(x)
    net.train_step(x, m, g)
    torch.cuda.synchronize()
    print("ncu cnn case: %d states, misfit sum %.6e" % (batch, float(mp.sum())))


def main():
    args = parse()
    if args.ncu_case_cnn:
        ncu_case_cnn(args.ncu_case_cnn)
        return
    if args.ncu_case_c4judge:
        ncu_case_c4judge(args.ncu_case_c4judge)
        return
    if args.ncu_case:
        ncu_case(args.ncu_case)
        return
    if args.ncu_case_exact:
        ncu_case_exact(args.ncu_case_exact)
        return
    if args.ncu_case_small:
        ncu_case_small(args.ncu_case_small)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    import numpy as np
    import torch

    import psvwave_gb300 as psv
    from psvwave_gb300 import workloads

    rank, local_rank, world = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)

    media = workloads.c1_media(seed=1 + rank)
    model = workloads.c1_model(precision=args.precision, device=local_rank, seed=1 + rank)
    stream = torch.cuda.Stream(device=dev)
    model.set_stream(stream.cuda_stream)
    cells = model.nx * model.nz
    nt = model.nt
    work = cells * nt

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        model.forward_simulate(0, False)
    torch.cuda.synchronize()

    sampler = ClockSampler(local_rank)
    sampler.start()
    barrier()
    torch.cuda.synchronize()
    total_ms = 0.0
    for k in range(args.steps):
        flush.fill_(k & 0xFF)  # evict L2 between timed iterations (outside the timed span)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        model.forward_simulate(0, False)
        e.record(stream)
        e.synchronize()
        total_ms += s.elapsed_time(e)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()

    t = torch.tensor([total_ms], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    max_ms = float(t.item())
    value = world * work * args.steps / (max_ms / 1e3) / 1e9

    # End to end through the public API: host inputs from pinned memory,
    # seismograms back to the host, every step.
    pinned = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in media]
    host_in = [p.numpy() for p in pinned]
    for _ in range(max(1, args.warmup // 2)):
        model.set_parameter_fields(*host_in)
        model.forward_simulate(0, False)
        model.get_synthetic_data()
    # At least 10 steps (under a second here): single host-side hiccups on
    # a shared machine moved a 5-step figure by several per cent.
    e2e_steps = max(args.steps, 10)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        model.set_parameter_fields(*host_in)
        model.forward_simulate(0, False)
        ux, uz = model.get_synthetic_data()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    e2e_value = world * work * e2e_steps / float(t.item()) / 1e9
    h2d = 3 * cells * 8
    d2h = 2 * model.n_shots * model.nr * model.nt * 8

    # The FP32 answer against the FP64 solve of the same run (outside every
    # timed region): relative L2 error of both seismogram components.
    parity = None
    if rank == 0 and args.precision == "fp32":
        m64 = workloads.c1_model(precision="fp64", device=local_rank, seed=1 + rank)
        m64.forward_simulate(0, False)
        errs = [float(np.linalg.norm(a - b) / np.linalg.norm(b))
                for a, b in zip((ux, uz), m64.get_synthetic_data())]
        parity = {"against": "FP64 GPU solve of the same 5000-step run",
                  "seismogram_rel_l2": {"ux": errs[0], "uz": errs[1]}, "tolerance": 1e-4}
        del m64

    # Roofline of the dominant kernel, per time step: the timed region's
    # device time divided by its time steps (each timed forward also holds
    # one field memset and the receiver prefix sum, so the figure is
    # slightly pessimistic), against the algorithmic bytes of one step. With
    # one launch per step, consecutive launches overlap their prologue with
    # the previous step's tail (programmatic dependent launch); with the
    # persistent scheme all steps are one launch whose tiles start a step as
    # soon as their neighbours have finished the previous one. The isolated
    # time (CUDA events around each of 500 per-step launches, or around one
    # 500-step persistent launch) is reported beside it.
    per_step_ms, kernel_ms = model.profile_forward(0, 500)
    dominant = max(kernel_ms, key=kernel_ms.get)
    # Kernels of ours per timed forward: the time-step launches (all steps in
    # one launch for the persistent scheme) and the receiver prefix sum.
    persistent = model.kernel_variant == "fused_tma_persistent"
    launches_per_forward = 2 if persistent else len(kernel_ms) * nt + 1
    words = 2 if args.precision == "fp64" else 1
    if dominant in ("stress_step", "velocity_step"):  # two launches per time step
        dominant = "stress_step+velocity_step"
        bpc = (BYTES_PER_CELL["stress_step"] + BYTES_PER_CELL["velocity_step"]) * words
    else:
        bpc = BYTES_PER_CELL[dominant] * words
    kernel_avg_ms = max_ms / args.steps / nt
    achieved = bpc * cells / (kernel_avg_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = measured_traffic(dominant)
    roofline = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": traffic,
                # measured DRAM bytes per step (warm-cache ncu capture) over
                # this run's time per step, against the same peak
                "dram_frac": (traffic / (kernel_avg_ms / 1e3) / 1e9 / peak
                              if traffic else None),
                "bytes_per_launch": bpc * cells,
                "kernel_avg_ms_timed_region": kernel_avg_ms,
                "launch_scheme": model.kernel_variant,
                "isolated_kernel_ms": kernel_ms, "isolated_step_ms": per_step_ms,
                "achieved_gcells_per_launch": cells / (kernel_avg_ms / 1e3) / 1e9}

    base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        base = cpu_baseline(workloads.c1_params, media, moment=workloads.c1_moment())
    secondary = None
    if not args.no_secondary:
        with_cpu = world == 1 and not args.no_cpu_baseline
        # Every rank takes its share of the c2 models; the rest runs on rank 0.
        sharded = batched(args.steps, args.warmup, rank, world, with_cpu)
        if rank == 0:
            secondary = {"fwi_gradients": fwi_gradients(args.steps, args.warmup, with_cpu),
                         "batched": sharded,
                         "fwi_gradients_c3": fwi_gradients_c3(min(args.steps, 2), with_cpu),
                         "mc_samples_c4": mc_samples_c4()}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": max_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == "fp32" else "f64",
            "data": "synthetic (seeded layered + Gaussian-random medium)",
            "config": {"workload": "c1: 2000x800 inner + 50-cell boundary (2100x900), nt=5000, "
                                   "400 receivers, 1 source, forward only",
                       "cells": cells, "nt": nt, "l2": "flushed between timed iterations",
                       "parallelism": "replicas" if world > 1 else "single"},
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_steps},
            "gpu_launches": launches_per_forward * args.steps,
            "roofline": roofline,
            "cpu_baseline": base,
            "clocks": clocks,
            "parity": parity,
            "secondary": secondary,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
