"""Independent units of the P-SV workloads spread across torch.distributed
ranks, one GPU per rank.

Shots are independent in the forward and adjoint runs
(src/fdModel.cpp:1293-1305), and so are the models of a batch and the chains
of a Monte Carlo sampler. Each is assigned round-robin: unit k goes to rank
k % world. Nothing crosses ranks on the time-stepping path (no halo
exchange: every rank holds whole grids); the only exchanges are at the end:

* sharded_gradient -- shots of one model (the c3 gradient): one sum
  all-reduce of the 3 nx nz FP64 velocity kernels plus the misfit. On NCCL
  the kernels stay in device memory from the solver to the reduction.
* sharded_forward -- models of a batch (c2): each rank advances its models'
  shots in one batched launch per time step; the seismograms are gathered.
* sharded_da_hmc -- chains of the delayed-acceptance sampler (c4): each rank
  runs its chains; every rank draws the random numbers of all chains from
  the same seed and uses its own chains' share, so the samples do not
  depend on the number of ranks. The samples are gathered.

The velocity kernels are linear in the per-shot Lame kernels
(src/fdModel.cpp:1164-1183), so summing mapped kernels across ranks equals
mapping the summed Lame kernels, up to rounding.
"""
import numpy as np
import torch
import torch.distributed as dist


def shard(n, rank, world):
    """The units (shots, models, chains) this rank takes: round-robin."""
    return list(range(rank, n, world))


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


def _on_device(model, group):
    """True when the reduction runs over NCCL and the model is a GPU
    fdModel whose kernels can be read as CUDA tensors."""
    return dist.get_backend(group) == "nccl" and hasattr(model, "get_kernels_device")


def sharded_gradient(model, mode="reference", checkpoint_every=100, group=None):
    """(misfit, (g_vp, g_vs, g_rho)) over all shots of `model`, each rank
    simulating its shard. mode "reference": the reference's adjoint kernels
    (forward with snapshots, adjoint sources, adjoint, velocity mapping);
    mode "exact": the exact discrete adjoint. Every rank must hold the same
    medium and observed data, and every rank returns the same total: CUDA
    tensors when the group runs NCCL over GPU models (the kernels never
    leave device memory), numpy arrays otherwise."""
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    shots = shard(model.n_shots, rank, world)
    shape = (model.nx, model.nz)
    device = _on_device(model, group)
    if mode not in ("reference", "exact"):
        raise ValueError("mode must be 'reference' or 'exact'")
    if device:
        dev = torch.device("cuda", model.device)
        g = torch.zeros((3,) + shape, dtype=torch.float64, device=dev)
        mis = 0.0
        if shots and mode == "reference":
            for s in shots:
                model.forward_simulate(s, True)
            model.calculate_l2_adjoint_sources()
            model.reset_kernels()
            for s in shots:
                model.adjoint_simulate(s)
            model.map_kernels_to_velocity()
            for k, t in enumerate(model.get_kernels_device()):
                g[k].copy_(t)
            mis = shot_misfit(model, shots)
        elif shots:
            mis, gd = model.exact_gradient(checkpoint_every, on_device=True, shots=shots)
            for k, t in enumerate(gd):
                g[k].copy_(t)
        flat = torch.cat([g.reshape(-1), torch.tensor([mis], dtype=torch.float64, device=dev)])
        dist.all_reduce(flat, op=dist.ReduceOp.SUM, group=group)
        g = flat[:-1].reshape((3,) + shape)
        return float(flat[-1].item()), (g[0], g[1], g[2])
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
    else:
        if shots:
            mis, g = model.exact_gradient(checkpoint_every, shots=shots)
            g = np.stack(g)
        else:
            mis, g = 0.0, np.zeros((3,) + shape)
    buf = torch.tensor(np.concatenate([g.reshape(-1), [mis]]), dtype=torch.float64)
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    total = buf.numpy()
    g = total[:-1].reshape((3,) + shape)
    return float(total[-1]), (g[0], g[1], g[2])


def _batch_runner(models, store_fields=False):
    """The GPU runner: every shot of `models` in one psvwave_gb300.Batch
    (one launch per time step, replayed as a CUDA graph)."""
    from .batch import Batch

    if not models:
        return
    b = Batch(device=models[0].device)
    for m in models:
        b.add_all_shots(m)
    b.forward(store_fields)


def sharded_forward(models, group=None, runner=None):
    """Advance every shot of every model, each rank taking the models k with
    k % world == rank, then gather the seismograms. Returns, on every rank,
    a list with each model's (ux, uz) [shots][nr][nt] FP64 arrays in model
    order. `runner(models)` advances the given models (default: one batch
    of all their shots on this rank's GPU); models on other ranks are left
    untouched."""
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    mine = shard(len(models), rank, world)
    (runner or _batch_runner)([models[k] for k in mine])
    local = {k: tuple(np.asarray(a) for a in models[k].get_synthetic_data()) for k in mine}
    parts = [None] * world
    dist.all_gather_object(parts, local, group=group)
    out = {}
    for p in parts:
        out.update(p)
    return [out[k] for k in range(len(models))]


def sharded_da_hmc(post, net, z0, n_iter, eps, n_leap, seed=0, group=None, **kw):
    """Delayed-acceptance HMC (surrogate.da_hmc) of the chains z0 [B, ...],
    each rank running the chains k with k % world == rank against its own
    posterior (`post` and `net` local to the rank). Every rank draws the
    momenta and acceptance numbers of all B chains from `seed` and uses its
    chains' share, so a chain's trajectory is the same whatever the number
    of ranks. Returns, on every rank, the gathered samples [n_iter][B][...]
    (host tensors), the final states and the summed acceptance counts, plus
    this rank's own timing."""
    from .surrogate import da_hmc

    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    B = z0.shape[0]
    mine = shard(B, rank, world)
    record = kw.get("record", True)
    if mine:
        idx = torch.tensor(mine, dtype=torch.long, device=z0.device)
        res = da_hmc(post, net, z0[idx], n_iter, eps, n_leap, seed=seed, chains=(mine, B), **kw)
    else:  # more ranks than chains
        res = {"samples": None, "z": z0[:0], "proposals": 0, "stage1_accepted": 0,
               "accepted": 0, "seconds": 0.0}
    local = {"chains": mine, "samples": res["samples"].cpu() if res["samples"] is not None
             else None, "z": res["z"].cpu(), "proposals": res["proposals"],
             "stage1_accepted": res["stage1_accepted"], "accepted": res["accepted"]}
    parts = [None] * world
    dist.all_gather_object(parts, local, group=group)
    z = torch.empty((B,) + tuple(z0.shape[1:]), dtype=torch.float32)
    samples = None
    if record:
        samples = torch.empty((n_iter, B) + tuple(z0.shape[1:]), dtype=torch.float32)
    for p in parts:
        if not p["chains"]:
            continue
        ci = torch.tensor(p["chains"], dtype=torch.long)
        z[ci] = p["z"]
        if samples is not None:
            samples[:, ci] = p["samples"]
    return {"samples": samples, "z": z,
            "proposals": sum(p["proposals"] for p in parts),
            "stage1_accepted": sum(p["stage1_accepted"] for p in parts),
            "accepted": sum(p["accepted"] for p in parts),
            "seconds": res["seconds"]}
