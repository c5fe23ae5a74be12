"""The surrogate-screened Monte Carlo workload end to end: training triples
from the solver, the network trained on them, local refinement, then
delayed-acceptance HMC against HMC with the solver's gradients.

    python -m psvwave_gb300.c4 --train 20000      # the full configuration

prints one JSON object. bench.py calls run() with a smaller training set.
"""
import argparse
import json
import time

import torch

from . import surrogate as sg


def _r2(pred, true):
    pred, true = pred.double(), true.double()
    return float(1.0 - ((pred - true) ** 2).mean() / true.var())


def _rel(pred, true):
    return float(((pred - true) ** 2).mean().sqrt() / (true ** 2).mean().sqrt())


def run(n_train=2048, n_local=512, n_chains=128, n_iter=40, burn_in=20, eps=0.03, n_leap=10,
        plain_chains=16, plain_iter=3, s2_div=20.0, epochs=None, seed=0, log=None):
    """Runs the workload; returns a dict of measurements.

    The posterior's noise scale is s2 = misfit(prior mean) / s2_div. Chains
    start from 0.5 x prior draws; a burn-in screened by the prior alone
    provides the states at which n_local more exact triples refine the
    network. Timed: n_iter iterations of every sampler from the burn-in's
    final states."""
    def say(msg):
        if log:
            log(msg)

    if epochs is None:  # about 4500 Adam steps whatever the set size, at least 60 epochs
        epochs = max(60, (4500 * 256) // max(n_train, 1))
    out = {}
    S = sg.c4_setup(n_chains, s2=1.0)
    post = S["posterior"]
    dev = S["z_true"].device
    chi0 = float(post.misfits(torch.zeros((1, 3, 20, 10), device=dev))[0])
    post.s2 = chi0 / s2_div
    out["s2"] = post.s2
    out["misfit_prior_mean"] = chi0

    t0 = time.perf_counter()
    z, mis, grads = sg.generate_training_set(post, n_train, seed=seed + 1)
    torch.cuda.synchronize()
    out["train_set"] = {"triples": n_train, "seconds": time.perf_counter() - t0}
    hold = max(1, n_train // 16)
    net = sg.SurrogateNet(max_batch=512, seed=seed)
    t0 = time.perf_counter()
    hist = sg.train(net, z[:-hold], mis[:-hold], grads[:-hold], epochs=epochs, batch=256, lr=1e-3,
                    seed=seed)
    torch.cuda.synchronize()
    out["training"] = {"seconds": time.perf_counter() - t0, "epochs": epochs,
                       "loss_first": hist[0], "loss_last": hist[-1]}
    m, g = net.predict(z[-hold:])
    out["heldout_prior"] = {"misfit_r2": _r2(m, mis[-hold:]),
                            "gradient_rel_err": _rel(g, grads[-hold:])}
    say("trained: %s" % out["heldout_prior"])

    # Burn-in screened by the prior alone; its states feed the local set.
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed + 5)
    z0 = 0.5 * torch.randn((n_chains, 3, 20, 10), device=dev, generator=gen)
    bi = sg.da_hmc(post, net, z0, burn_in, eps, n_leap, seed=seed + 11, screen=0.0, force=0.0)
    zs = bi["samples"][burn_in // 2:].reshape(-1, 3, 20, 10)
    idx = torch.randperm(zs.shape[0], device=dev, generator=gen)[:n_local]
    t0 = time.perf_counter()
    zl, ml, gl = sg.triples_at(post, zs[idx])
    nl = max(1, n_local // 4)
    base = min(n_train - hold, 4 * n_local)
    zz = torch.cat([z[:base]] + [zl[:-nl]] * 4)
    mm = torch.cat([mis[:base]] + [ml[:-nl]] * 4)
    gg = torch.cat([grads[:base]] + [gl[:-nl]] * 4)
    sg.train(net, zz, mm, gg, epochs=max(10, epochs // 3), batch=256, lr=5e-4, seed=seed + 1,
             keep_norm=True)
    torch.cuda.synchronize()
    out["refinement"] = {"triples": n_local, "seconds": time.perf_counter() - t0}
    m, g = net.predict(zl[-nl:])
    out["heldout_local"] = {"misfit_r2": _r2(m, ml[-nl:]), "gradient_rel_err": _rel(g, gl[-nl:]),
                            "misfit_rms_in_potential_units":
                                float(((m - ml[-nl:]) ** 2).mean().sqrt()) / post.s2}
    say("refined: %s" % out["heldout_local"])

    zb = bi["z"]
    keep = lambda r: {k: r[k] for k in ("proposals", "stage1_accepted", "accepted", "seconds",
                                        "accepted_per_s") if k in r}
    da = sg.da_hmc(post, net, zb, n_iter, eps, n_leap, seed=seed + 3, screen=0.5, force=0.0)
    out["da_hmc"] = keep(da)
    say("DA-HMC: %s" % out["da_hmc"])
    po = sg.da_hmc(post, net, zb, n_iter, eps, n_leap, seed=seed + 3, screen=0.0, force=0.0)
    out["prior_screened_hmc"] = keep(po)
    say("prior-screened: %s" % out["prior_screened_hmc"])
    pl = sg.plain_hmc(post, zb[:plain_chains], plain_iter, eps, n_leap, seed=seed + 3,
                      threads=plain_chains)
    out["plain_hmc"] = keep(pl)
    say("plain: %s" % out["plain_hmc"])
    out["value"] = out["da_hmc"]["accepted_per_s"]
    out["speedup_vs_plain"] = out["value"] / max(out["plain_hmc"]["accepted_per_s"], 1e-12)
    out["speedup_vs_prior_screened"] = out["value"] / max(
        out["prior_screened_hmc"]["accepted_per_s"], 1e-12)

    # Posterior summaries of the exact samplers (z units): the network-
    # screened chains against plain HMC (the same chains' starting states,
    # fewer samples) and against the prior-screened chains (same number of
    # samples). Each: the RMS over the 600 parameters of the difference of
    # means in posterior standard deviations, and the mean variance ratio.
    def compare(a, b):
        sd = a.std(0).clamp_min(1e-12)
        return {"samples": [int(a.shape[0]), int(b.shape[0])],
                "rms_mean_difference_over_sd":
                    float((((a.mean(0) - b.mean(0)) / sd) ** 2).mean().sqrt()),
                "mean_variance_ratio": float((b.var(0) / a.var(0).clamp_min(1e-24)).mean())}

    a = da["samples"].reshape(n_iter, n_chains, -1).double()
    out["posterior_vs_plain"] = compare(a[:, :plain_chains].reshape(-1, 600),
                                        pl["samples"].reshape(-1, 600).double())
    out["posterior_vs_prior_screened"] = compare(
        a.reshape(-1, 600), po["samples"].reshape(n_iter, n_chains, -1).double().reshape(-1, 600))
    out["n_chains"], out["n_iter"], out["eps"], out["n_leap"] = n_chains, n_iter, eps, n_leap
    return out


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--train", type=int, default=20000)
    p.add_argument("--local", type=int, default=1024)
    p.add_argument("--chains", type=int, default=128)
    p.add_argument("--iters", type=int, default=400)  # 128 chains x 400 = 51200 proposals
    p.add_argument("--plain-chains", type=int, default=16)
    p.add_argument("--plain-iters", type=int, default=32)  # 16 x 32 = 512 plain samples
    a = p.parse_args()
    out = run(n_train=a.train, n_local=a.local, n_chains=a.chains, n_iter=a.iters,
              plain_chains=a.plain_chains, plain_iter=a.plain_iters,
              log=lambda s: print(s, flush=True))
    print(json.dumps(out))


if __name__ == "__main__":
    main()
