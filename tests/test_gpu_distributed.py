"""The sharding helpers on the GPU path (psvwave_gb300.distributed) in a
one-rank NCCL group on one GPU: the device-resident all-reduce of
sharded_gradient (kernels from the solver's device buffers, CUDA tensors
back), the batched runner of sharded_forward, and sharded_da_hmc over the
real solver judge (NCCL object gathers) all give what one process gives. The multi-rank splits
themselves are covered by the gloo tests (tests/test_distributed.py); a box
here has one GPU."""
import os
import socket

import numpy as np
import pytest
import torch

import psvwave_gb300 as psv
from psvwave_gb300 import distributed
from tests.conftest import SMALL_INI, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nccl_group():
    import torch.distributed as dist

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    torch.cuda.set_device(0)
    dist.init_process_group("nccl", init_method="tcp://127.0.0.1:%d" % port, rank=0,
                            world_size=1, device_id=torch.device("cuda", 0))
    yield dist.group.WORLD
    dist.destroy_process_group()


def observed(golden, precision):
    m = psv.fdModel(SMALL_INI, precision=precision)
    m.set_parameter_fields(*golden["target"])
    for s in range(m.n_shots):
        m.forward_simulate(s, False)
    m.set_observed_data(*m.get_synthetic_data())
    m.set_parameter_fields(*golden["start"])
    return m


@pytest.mark.parametrize("mode", ["reference", "exact"])
def test_sharded_gradient_device_path_matches_one_process(golden, nccl_group, mode):
    m = observed(golden, "fp64")
    mis, g = distributed.sharded_gradient(m, mode=mode, group=nccl_group)
    assert all(isinstance(x, torch.Tensor) and x.is_cuda for x in g)
    ref = observed(golden, "fp64")
    if mode == "reference":
        ref.compute_gradients()
        want = ref.get_kernels()
        ref.calculate_l2_misfit()
        want_mis = ref.misfit
    else:
        want_mis, want = ref.exact_gradient(100)
    assert abs(mis - want_mis) <= 1e-12 * abs(want_mis)
    for a, b in zip(g, want):
        assert rel_l2(a.cpu().numpy(), b) <= 1e-12


def test_sharded_forward_batch_runner(nccl_group):
    from psvwave_gb300 import workloads

    pairs = workloads.c2_models(n_models=3, nt=300, seed=5)
    models = []
    for p, media in pairs:
        m = psv.fdModel.from_parameters(p)
        m.set_parameter_fields(*media)
        models.append(m)
    out = distributed.sharded_forward(models, group=nccl_group)
    for (p, media), (ux, uz) in zip(pairs, out):
        m = psv.fdModel.from_parameters(p)
        m.kernel_variant = "fused_tma"
        m.tile_shape = "16x28"  # the batch's default shape
        m.set_parameter_fields(*media)
        for s in range(m.n_shots):
            m.forward_simulate(s, False)
        rx, rz = m.get_synthetic_data()
        assert np.array_equal(ux, rx) and np.array_equal(uz, rz)


def test_sharded_da_hmc_matches_one_process(nccl_group):
    from psvwave_gb300 import surrogate as sg

    S = sg.c4_setup(4, s2=1.0)
    post = S["posterior"]
    post.s2 = float(post.misfits(torch.zeros((1, 3, 20, 10), device="cuda"))[0]) / 20.0
    net = sg.SurrogateNet(max_batch=64, seed=2)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)
    z0 = 0.5 * torch.randn((4, 3, 20, 10), device="cuda", generator=gen)
    kw = dict(screen=0.5, force=0.0)
    got = distributed.sharded_da_hmc(post, net, z0, 3, 0.03, 4, seed=7, group=nccl_group, **kw)
    want = sg.da_hmc(post, net, z0, 3, 0.03, 4, seed=7, **kw)
    assert got["proposals"] == want["proposals"] == 12
    assert got["stage1_accepted"] == want["stage1_accepted"]
    assert got["accepted"] == want["accepted"]
    assert torch.equal(got["samples"], want["samples"].cpu())
    assert torch.equal(got["z"], want["z"].cpu())
