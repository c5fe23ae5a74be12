"""Shot-sharded gradients across ranks (psvwave_gb300.distributed) on CPU:
world_size 2 and 3 gloo ranks, each driving the oracle port as its engine,
reproduce the single-process gradient (the reference's run_model) of the
two-shot golden configuration."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from tests.conftest import SMALL_INI, rel_l2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _oracle(target, start):
    from oracle.portbind import OracleModel

    o = OracleModel(SMALL_INI)
    o.dt = o.scalars()["dt"]
    o.set_parameter_fields(*target)
    for s in range(o.n_shots):
        o.forward_simulate(s, False)
    o.set_observed_data(*o.get_synthetic_data())
    o.set_parameter_fields(*start)
    return o


def _rank(rank, world, port, target, start, queue):
    import torch.distributed as dist

    from psvwave_gb300.distributed import shard, sharded_gradient

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        o = _oracle(target, start)
        mis, g = sharded_gradient(o, "reference")
        queue.put((rank, shard(o.n_shots, rank, world), mis, [np.asarray(x) for x in g]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_gradient_matches_single_process(golden, world):
    target = [np.array(a) for a in golden["target"]]
    start = [np.array(a) for a in golden["start"]]
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, target, start, queue))
             for r in range(world)]
    for p in procs:
        p.start()
    results = [queue.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    results.sort(key=lambda r: r[0])
    # Every shot is simulated by exactly one rank.
    assert sorted(s for r in results for s in r[1]) == [0, 1]
    o = _oracle(target, start)
    o.run_model(True)
    ref = o.get_kernels()
    for _, _, mis, g in results:  # every rank holds the same total
        assert abs(mis - o.misfit) <= 1e-12 * abs(o.misfit)
        for a, b in zip(g, ref):
            assert rel_l2(a, b) <= 1e-12


# ---- models of a batch (c2) and chains of the sampler (c4) ---------------

def _models(n):
    """n small models (the golden configuration) with different seeded media."""
    from oracle.portbind import OracleModel

    out = []
    for k in range(n):
        o = OracleModel(SMALL_INI)
        rng = np.random.default_rng(100 + k)
        shape = (o.nx, o.nz)
        o.set_parameter_fields(2000 * (1 + 0.03 * rng.standard_normal(shape)),
                               800 * (1 + 0.03 * rng.standard_normal(shape)),
                               1500 * (1 + 0.03 * rng.standard_normal(shape)))
        out.append(o)
    return out


def _run_all_shots(models):
    for m in models:
        for s in range(m.n_shots):
            m.forward_simulate(s, False)


def _forward_rank(rank, world, port, n_models, queue):
    import torch.distributed as dist

    from psvwave_gb300.distributed import sharded_forward

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        models = _models(n_models)
        ran = []

        def runner(ms):
            ran.extend(id(m) for m in ms)
            _run_all_shots(ms)

        out = sharded_forward(models, runner=runner)
        mine = [k for k, m in enumerate(models) if id(m) in ran]
        queue.put((rank, mine, out))
    finally:
        dist.destroy_process_group()


def _spawn(fn, world, *args):
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=fn, args=(r, world, port) + args + (queue,))
             for r in range(world)]
    for p in procs:
        p.start()
    results = [queue.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return sorted(results, key=lambda r: r[0])


def test_sharded_forward_gathers_every_model_once():
    """Three models over two ranks: each model runs on exactly one rank
    (round-robin) and every rank ends with every model's seismograms,
    identical to running all models in one process."""
    n = 3
    results = _spawn(_forward_rank, 2, n)
    assert [r[1] for r in results] == [[0, 2], [1]]
    ref = _models(n)
    _run_all_shots(ref)
    for _, _, out in results:
        assert len(out) == n
        for m, (ux, uz) in zip(ref, out):
            rx, rz = m.get_synthetic_data()
            assert np.array_equal(ux, rx) and np.array_equal(uz, rz)


def _hmc_problem():
    from tests.test_hmc_exactness import Judge, Net, problem

    q, wrong, _, _ = problem()
    return Judge(q), Net(wrong)


def _hmc_rank(rank, world, port, n_chains, queue):
    import torch
    import torch.distributed as dist

    from psvwave_gb300.distributed import sharded_da_hmc

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        judge, net = _hmc_problem()
        z0 = torch.zeros((n_chains, 4), dtype=torch.float32)
        res = sharded_da_hmc(judge, net, z0, 60, 0.15, 8, seed=3)
        queue.put((rank, res["samples"].numpy(), res["accepted"], res["proposals"]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_da_hmc_chains_match_one_process(world):
    """Delayed-acceptance chains split round-robin over ranks follow the
    trajectories they follow in one process: every rank draws all chains'
    random numbers from the same seed and keeps its chains' share."""
    import torch

    from psvwave_gb300.surrogate import da_hmc

    n_chains = 7
    results = _spawn(_hmc_rank, world, n_chains)
    judge, net = _hmc_problem()
    ref = da_hmc(judge, net, torch.zeros((n_chains, 4), dtype=torch.float32), 60, 0.15, 8, seed=3)
    for _, samples, acc, props in results:
        assert props == ref["proposals"]
        assert acc == ref["accepted"]
        np.testing.assert_allclose(samples, ref["samples"].numpy(), rtol=0, atol=1e-6)
