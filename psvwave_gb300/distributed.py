"""FWI gradients sharded by shot across torch.distributed ranks, one GPU per
rank.

Shots are independent in the forward and adjoint runs
(src/fdModel.cpp:1293-1305). Each rank takes the shots k with
k % world == rank, and the ranks then add their per-shot sums. That is one
all-reduce (sum) of 3 nx nz FP64 values plus the misfit, with NCCL between
GPUs and gloo for CPU-side tests. Nothing else crosses ranks: no halo
exchange, because each rank holds whole grids.

The velocity kernels are linear in the per-shot Lame kernels
(src/fdModel.cpp:1164-1183), so summing mapped kernels across ranks equals
mapping the summed Lame kernels, up to rounding.
"""
import numpy as np
import torch
import torch.distributed as dist


def shard(n_shots, rank, world):
    """The shots this rank simulates: round-robin."""
    return list(range(rank, n_shots, world))


def shot_misfit(model, shots):
    """The reference's L2 misfit restricted to `shots`
    (0.5 dt sum (obs - syn)^2 over both components, src/fdModel.cpp:1128-1145),
    from the model's synthetic and observed data, in FP64 on the host."""
    sx, sz = model.get_synthetic_data()
    ox, oz = model.get_observed_data()
    tot = 0.0
    for s in shots:
        tot += 0.5 * model.dt * (float(np.sum((ox[s] - sx[s]) ** 2)) +
                                 float(np.sum((oz[s] - sz[s]) ** 2)))
    return tot


def _all_reduce(values, group):
    backend = dist.get_backend(group)
    device = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else "cpu"
    buf = torch.tensor(values, dtype=torch.float64, device=device)
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    return buf.cpu().numpy()


def sharded_gradient(model, mode="reference", checkpoint_every=100, group=None):
    """(misfit, (g_vp, g_vs, g_rho)) over all shots of `model`, each rank
    simulating its shard. mode "reference": the reference's adjoint kernels
    (forward with snapshots, adjoint sources, adjoint, velocity mapping);
    mode "exact": the exact discrete adjoint. Every rank must hold the same
    medium and observed data. Every rank returns the same total."""
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    shots = shard(model.n_shots, rank, world)
    shape = (model.nx, model.nz)
    if mode == "reference":
        for s in shots:
            model.forward_simulate(s, True)
        model.calculate_l2_adjoint_sources()
        model.reset_kernels()
        for s in shots:
            model.adjoint_simulate(s)
        model.map_kernels_to_velocity()
        g = np.stack(model.get_kernels()) if shots else np.zeros((3,) + shape)
        mis = shot_misfit(model, shots)
    elif mode == "exact":
        if shots:
            mis, g = model.exact_gradient(checkpoint_every, shots=shots)
            g = np.stack(g)
        else:
            mis, g = 0.0, np.zeros((3,) + shape)
    else:
        raise ValueError("mode must be 'reference' or 'exact'")
    total = _all_reduce(np.concatenate([g.reshape(-1), [mis]]), group)
    g = total[:-1].reshape((3,) + shape)
    return float(total[-1]), (g[0], g[1], g[2])
