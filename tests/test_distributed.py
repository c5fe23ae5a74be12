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
