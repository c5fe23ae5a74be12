"""Surrogate-screened Monte Carlo over the medium.

The medium is parameterised on a coarse grid (vp, vs, rho on 20 x 10 nodes,
prior N(mean, sigma^2) independently per node; sampling runs in the
normalised coordinates z = (theta - mean) / sigma). The posterior of z given
observed seismograms is

    U(z) = misfit(z) / s2 + |z|^2 / 2,     pi(z) ~ exp(-U(z)),

with misfit the reference's L2 misfit (src/fdModel.cpp:1128-1145) and s2 a
stated data-noise scale.

* CoarseParam -- the coarse-to-grid map and its transpose (CUDA kernels of
  the C library).
* SurrogateNet -- the CNN that predicts misfit(z) and its gradient. Its
  forward, backward and Adam kernels are the project's own CUDA kernels.
* FDPosterior -- the finite-difference solver as the judge. It gives batched
  potentials (one launch per time step for all chains, psv_batch) and exact
  gradients (the exact discrete adjoint).
* generate_training_set, train -- (z, misfit, gradient) triples from the
  solver, and the network fitted to them.
* da_hmc -- delayed-acceptance HMC (Christen and Fox, 2005). Leapfrog
  trajectories are driven by the surrogate's gradient. A first stage
  accepts with the surrogate Hamiltonian. Only proposals that pass go to
  the second stage, which the solver judges with
  min(1, exp(-(U(y) - U(x)) + (U~(y) - U~(x)))). The chain therefore has
  the exact posterior as its stationary law, whatever the surrogate's
  error. Leapfrog with any force field is volume-preserving and reversible,
  so the first stage is a valid Metropolis step for the surrogate's own
  density.
* plain_hmc -- the same sampler with the solver's exact gradient in every
  leapfrog step: the method without the surrogate.
"""
import ctypes
import threading
import time

import numpy as np
import torch

from . import _capi, workloads
from .batch import Batch
from .model import fdModel

_f32p = ctypes.c_void_p


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class CoarseParam:
    """Coarse medium parameters -> (vp, vs, rho) grids of a model geometry."""

    def __init__(self, nx, nz, np_boundary, mean, sigma, device=0):
        self.mean = np.ascontiguousarray(mean, dtype=np.float64)
        self.sigma = np.ascontiguousarray(sigma, dtype=np.float64)
        _, self.ncx, self.ncz = self.mean.shape
        self.nx, self.nz, self.device = nx, nz, device
        self._lib = _capi.load()
        h = ctypes.c_void_p()
        dp = ctypes.POINTER(ctypes.c_double)
        _capi.check(self._lib.psv_coarse_create(
            device, nx, nz, np_boundary, self.ncx, self.ncz, self.mean.ctypes.data_as(dp),
            self.sigma.ctypes.data_as(dp), ctypes.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.psv_coarse_destroy(self._h)
            self._h = None

    def _dev(self):
        return torch.device("cuda", self.device)

    def to_fields(self, z):
        """z [B][3][ncx][ncz] -> fields [B][3][nx][nz] (float64, CUDA)."""
        z = z.detach().to(self._dev(), torch.float32).contiguous().view(-1, 3, self.ncx, self.ncz)
        out = torch.empty((z.shape[0], 3, self.nx, self.nz), dtype=torch.float64, device=self._dev())
        torch.cuda.current_stream(self._dev()).synchronize()
        _capi.check(self._lib.psv_coarse_to_fields(self._h, z.shape[0], _ptr(z), _ptr(out), None))
        return out

    def gradient(self, gfields, scale=1.0):
        """Field gradients [B][3][nx][nz] -> z gradients [B][3][ncx][ncz] x scale."""
        g = gfields.detach().to(self._dev(), torch.float64).contiguous()
        out = torch.empty((g.shape[0], 3, self.ncx, self.ncz), dtype=torch.float32, device=self._dev())
        torch.cuda.current_stream(self._dev()).synchronize()
        _capi.check(self._lib.psv_coarse_gradient(self._h, g.shape[0], _ptr(g), _ptr(out),
                                                  float(scale), None))
        return out


def _num_params():
    n = ctypes.c_size_t()
    _capi.check(_capi.load().psv_cnn_num_params(ctypes.byref(n)))
    return n.value


# Architecture of the network (include/psvwave_surrogate.h): inputs are the 3
# parameter channels plus 2 channels of node coordinates in [-1, 1].
CNN_LAYERS = ((5, 32), (32, 64), (64, 64), (64, 4))


def init_params(seed=0):
    """He-normal weights, zero biases (float32), in the parameter layout:
    per layer, weights [cout][cin][3][3] then bias [cout]. The last layer
    starts 100x smaller: its misfit channel is summed over 200 grid points,
    and full-size initial outputs make the first Adam steps diverge."""
    rng = np.random.default_rng(seed)
    parts = []
    for l, (cin, cout) in enumerate(CNN_LAYERS):
        scale = np.sqrt(2.0 / (cin * 9)) * (0.01 if l + 1 == len(CNN_LAYERS) else 1.0)
        parts.append(rng.standard_normal(cout * cin * 9) * scale)
        parts.append(np.zeros(cout))
    return np.concatenate(parts).astype(np.float32)


class SurrogateNet:
    """The surrogate network on one GPU. States are z [B][3][20][10] (float32,
    CUDA); the network sees them with two coordinate channels appended
    (`features`). Its outputs are in normalised units; `norm` maps them back:
    misfit = m0 + ms * m, gradient = gs * g with gs a per-node scale
    [3][20][10] (the RMS of the training gradients at that node)."""

    def __init__(self, device=0, max_batch=512, seed=0):
        self._lib = _capi.load()
        self.device, self.max_batch = device, max_batch
        self.num_params = _num_params()
        h = ctypes.c_void_p()
        _capi.check(self._lib.psv_cnn_create(device, max_batch, ctypes.byref(h)))
        self._h = h
        dev = torch.device("cuda", device)
        xc = torch.linspace(-1.0, 1.0, 20, device=dev)[:, None].expand(20, 10)
        zc = torch.linspace(-1.0, 1.0, 10, device=dev)[None, :].expand(20, 10)
        self._coords = torch.stack([xc, zc]).float().contiguous()
        self.norm = {"m0": 0.0, "ms": 1.0, "gs": torch.ones((3, 20, 10), device=dev)}
        self.set_params(init_params(seed))

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.psv_cnn_destroy(self._h)
            self._h = None

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != self.num_params:
            raise ValueError("expected %d parameters" % self.num_params)
        _capi.check(self._lib.psv_cnn_set_params(self._h, p.ctypes.data_as(_f32p)))

    def get_params(self):
        p = np.empty(self.num_params, dtype=np.float32)
        _capi.check(self._lib.psv_cnn_get_params(self._h, p.ctypes.data_as(_f32p)))
        return p

    def _x(self, x):
        x = x.detach().to(torch.device("cuda", self.device), torch.float32).contiguous()
        torch.cuda.current_stream(x.device).synchronize()
        return x

    def features(self, z):
        """Network inputs [B][5][20][10] of states z [B][3][20][10]."""
        z = z.detach().to(torch.device("cuda", self.device), torch.float32).reshape(-1, 3, 20, 10)
        return torch.cat([z, self._coords.expand(z.shape[0], 2, 20, 10)], 1).contiguous()

    def predict_features(self, x):
        """Normalised outputs (m [B], g [B][3][20][10]) of network inputs x."""
        x = self._x(x)
        B = x.shape[0]
        m = torch.empty(B, dtype=torch.float32, device=x.device)
        g = torch.empty((B, 3, 20, 10), dtype=torch.float32, device=x.device)
        for s in range(0, B, self.max_batch):
            e = min(B, s + self.max_batch)
            _capi.check(self._lib.psv_cnn_predict(self._h, e - s, _ptr(x[s:e]), _ptr(m[s:e]),
                                                  _ptr(g[s:e])))
        return m, g

    def predict(self, z):
        """(misfit [B] float64, gradient [B][3][20][10] float32) at states z,
        in physical units."""
        m, g = self.predict_features(self.features(z))
        n = self.norm
        return n["m0"] + n["ms"] * m.double(), n["gs"] * g

    def loss_grad(self, x, m, g, w_misfit=1.0, w_grad=1.0):
        """Loss and parameter gradient for network inputs x and normalised
        targets m, g."""
        x, m, g = self._x(x), self._x(m), self._x(g)
        loss = ctypes.c_double()
        d = np.empty(self.num_params, dtype=np.float32)
        _capi.check(self._lib.psv_cnn_loss_grad(self._h, x.shape[0], _ptr(x), _ptr(m), _ptr(g),
                                                float(w_misfit), float(w_grad), ctypes.byref(loss),
                                                d.ctypes.data_as(_f32p)))
        return loss.value, d

    def train_step(self, x, m, g, w_misfit=1.0, w_grad=1.0, lr=1e-3, beta1=0.9, beta2=0.999,
                   eps=1e-8):
        """One Adam step on network inputs x and normalised targets."""
        loss = ctypes.c_double()
        _capi.check(self._lib.psv_cnn_train_step(self._h, x.shape[0], _ptr(x), _ptr(m), _ptr(g),
                                                 float(w_misfit), float(w_grad), float(lr),
                                                 float(beta1), float(beta2), float(eps),
                                                 ctypes.byref(loss)))
        return loss.value

    def save(self, path):
        n = self.norm
        np.savez(path, params=self.get_params(), m0=np.float64(n["m0"]), ms=np.float64(n["ms"]),
                 gs=n["gs"].cpu().numpy())

    def load(self, path):
        d = np.load(path)
        self.set_params(d["params"])
        self.norm = {"m0": float(d["m0"]), "ms": float(d["ms"]),
                     "gs": torch.tensor(d["gs"], device=torch.device("cuda", self.device))}


class FDPosterior:
    """The solver as the judge: U(z) = misfit(z) / s2 + |z|^2 / 2 for the
    c4 geometry, with one FP32 model per chain (n_models) batched into one
    launch per time step for potentials, and exact-adjoint gradients."""

    def __init__(self, params, coarse, observed, s2, n_models, checkpoint_every=100, device=0):
        self.coarse, self.s2, self.ck = coarse, float(s2), int(checkpoint_every)
        self.device = device
        self.models = []
        for _ in range(n_models):
            m = fdModel.from_parameters(params, device=device)
            m.set_observed_data(*observed)
            # Media updates are only queued on the model's stream; the batched
            # forward and the exact gradient wait for it.
            m.set_async(True)
            self.models.append(m)
        self.batch = Batch(device)
        for m in self.models:
            self.batch.add(m, 0)
        # The judge's batched forward is most of a sampler iteration: time
        # every launch scheme and tile shape once and keep the fastest.
        self.batch.autotune(50)
        self.n_potentials = 0
        self.n_gradients = 0

    def _set(self, k, fields_k, sync=True):
        self.models[k].set_parameter_fields_device(fields_k[0], fields_k[1], fields_k[2], sync)

    def misfits(self, z, mask=None):
        """FD misfits of z [B][3][20][10] (B <= n_models), one batched
        forward of the states selected by `mask` (all by default); float64
        numpy [B], NaN where not selected."""
        B = z.shape[0]
        if B > len(self.models):
            raise ValueError("more states than models")
        sel = np.ones(B, dtype=bool) if mask is None else np.asarray(mask, dtype=bool)
        out = np.full(B, np.nan)
        if not sel.any():
            return out
        # One wait for the fields and one call for every selected member;
        # each model only queues its copies and medium update (the batched
        # forward waits for every member's stream, and `fields` lives until
        # it returns).
        fields = self.coarse.to_fields(z)
        self.batch.set_parameter_fields_device(fields, sel)
        flags = np.zeros(len(self.models), dtype=bool)
        flags[:B] = sel
        self.batch.set_active(flags)
        self.batch.forward()
        mis = self.batch.misfits()
        out[sel] = mis[:B][sel]
        self.n_potentials += int(sel.sum())
        return out

    def potentials(self, z, mask=None):
        zz = z.detach().double().reshape(z.shape[0], -1)
        return self.misfits(z, mask) / self.s2 + 0.5 * (zz * zz).sum(1).cpu().numpy()

    def misfit_gradient(self, k, z_k):
        """Exact misfit and its z-gradient at one state, with model k."""
        fields = self.coarse.to_fields(z_k.reshape(1, 3, self.coarse.ncx, self.coarse.ncz))
        self._set(k, fields[0])
        mis, g = self.models[k].exact_gradient(self.ck, on_device=True)
        gz = self.coarse.gradient(torch.stack(g)[None], 1.0)[0]
        self.n_gradients += 1
        return mis, gz

    def potential_gradient(self, k, z_k):
        mis, gz = self.misfit_gradient(k, z_k)
        zz = z_k.detach().reshape(gz.shape).to(gz.device, torch.float32)
        return mis / self.s2 + 0.5 * float((zz.double() ** 2).sum()), gz / self.s2 + zz


def c4_setup(n_models, seed=4, s2=None, device=0):
    """The c4 workload: geometry, coarse map, a true z drawn from the prior,
    observed data from it, and the posterior judge. s2 defaults to the
    misfit of the prior mean / 2000."""
    params = workloads.c4_params()
    mean, sigma = workloads.c4_prior()
    probe = fdModel.from_parameters(params, device=device)
    coarse = CoarseParam(probe.nx, probe.nz, probe.np_boundary, mean, sigma, device)
    rng = np.random.default_rng(seed)
    z_true = torch.tensor(rng.standard_normal((1, 3) + workloads.C4_COARSE), dtype=torch.float32,
                          device="cuda:%d" % device)
    f = coarse.to_fields(z_true)[0]
    probe.set_parameter_fields_device(f[0], f[1], f[2])
    probe.forward_simulate(0, False)
    observed = probe.get_synthetic_data()
    if s2 is None:
        f0 = coarse.to_fields(torch.zeros_like(z_true))[0]
        probe.set_observed_data(*observed)
        probe.set_parameter_fields_device(f0[0], f0[1], f0[2])
        probe.forward_simulate(0, False)
        probe.calculate_l2_misfit()
        s2 = probe.misfit / 2000.0
    post = FDPosterior(params, coarse, observed, s2, n_models, device=device)
    return {"params": params, "coarse": coarse, "z_true": z_true, "observed": observed,
            "s2": s2, "posterior": post}


def generate_training_set(post, n, seed=0, threads=None):
    """n triples (z, misfit, misfit gradient w.r.t. z) with z drawn from the
    prior, computed by the solver's exact adjoint on the posterior's models
    in parallel threads (one model and stream per thread)."""
    rng = np.random.default_rng(seed)
    shape = (3,) + (post.coarse.ncx, post.coarse.ncz)
    z = torch.tensor(rng.standard_normal((n,) + shape), dtype=torch.float32,
                     device="cuda:%d" % post.device)
    return triples_at(post, z, threads)


def triples_at(post, z, threads=None):
    """(z, misfit, misfit gradient w.r.t. z) at given states z [n][3][20][10]
    by the solver's exact adjoint, in parallel threads."""
    threads = min(threads or len(post.models), len(post.models))
    z = z.detach().float().contiguous()
    n = z.shape[0]
    mis = np.empty(n)
    grads = torch.empty_like(z)
    errors = []

    def work(k):
        try:
            for i in range(k, n, threads):
                m, g = post.misfit_gradient(k, z[i])
                mis[i] = m
                grads[i] = g
        except Exception as e:  # reported below
            errors.append(e)

    ts = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    if errors:
        raise errors[0]
    return z, torch.tensor(mis, device=z.device), grads


def train(net, z, mis, grads, epochs=30, batch=256, lr=1e-3, w_misfit=1.0, w_grad=1.0, seed=0,
          log=None, keep_norm=False):
    """Fit the network to (z, misfit, gradient) triples by Adam with a
    cosine-decayed learning rate. Unless keep_norm (fine-tuning), sets
    net.norm from the data (misfit standardised, gradient scaled per node by
    its RMS). Returns the loss history (mean per epoch)."""
    if not keep_norm:
        m0 = float(mis.mean())
        ms = float(mis.std()) or 1.0
        gs = grads.float().pow(2).mean(0).sqrt().clamp_min(1e-30)
        net.norm = {"m0": m0, "ms": ms, "gs": gs}
    m0, ms, gs = net.norm["m0"], net.norm["ms"], net.norm["gs"]
    mt = ((mis - m0) / ms).float().contiguous()
    gt = (grads / gs).float().contiguous()
    z = net.features(z)
    n = z.shape[0]
    gen = torch.Generator(device=z.device)
    gen.manual_seed(seed)
    history = []
    steps = max(1, epochs * max(1, n // batch))
    step = 0
    for ep in range(epochs):
        perm = torch.randperm(n, device=z.device, generator=gen)
        tot, cnt = 0.0, 0
        for s in range(0, n - batch + 1, batch):
            idx = perm[s:s + batch]
            rate = lr * 0.5 * (1.0 + np.cos(np.pi * step / steps))
            tot += net.train_step(z[idx].contiguous(), mt[idx].contiguous(),
                                  gt[idx].contiguous(), w_misfit, w_grad, rate)
            cnt += 1
            step += 1
        history.append(tot / max(cnt, 1))
        if log:
            log("epoch %d loss %.5f" % (ep, history[-1]))
    return history


def _surrogate_ug(net, z, s2, screen=1.0, force=1.0):
    """First-stage potential U~ = screen misfit~ / s2 + |z|^2 / 2 and the
    leapfrog force (force / s2) grad misfit~ + z at states z [B][3][20][10]."""
    m, g = net.predict(z)
    zz = z.reshape(z.shape[0], -1).double()
    u = screen * m / s2 + 0.5 * (zz * zz).sum(1)
    return u, (force / s2) * g + z


def da_hmc(post, net, z0, n_iter, eps, n_leap, seed=0, record=True, screen=1.0, force=1.0,
           chains=None):
    """Delayed-acceptance HMC of len(z0) chains in parallel. Returns a dict
    with the samples [n_iter][B][...], acceptance counts and timings.

    The first stage uses U~ = screen misfit~ / s2 + |z|^2 / 2; leapfrog
    trajectories follow the force (force / s2) grad misfit~ + z. Only
    proposals that pass the first stage are simulated (one batched forward
    per iteration). Any screen and force weights leave the posterior exact:
    leapfrog with any force is volume-preserving and reversible, and the
    second stage divides out the first stage's density. screen = force = 0
    screens with the prior alone.

    chains = (indices, n_total): z0 holds chains `indices` of a run of
    n_total chains. The random numbers of all n_total chains are drawn from
    `seed` and these chains use their share, so each chain follows the same
    trajectory as in the full run (the chains of a run can be split across
    processes)."""
    gen = torch.Generator(device=z0.device)
    gen.manual_seed(seed)
    rng = np.random.default_rng(seed)
    s2 = post.s2
    z = z0.clone().float()
    B = z.shape[0]
    if chains is None:
        sel_idx, n_total = None, B
    else:
        sel_idx, n_total = np.asarray(chains[0], dtype=np.int64), int(chains[1])
        if sel_idx.size != B:
            raise ValueError("chains must list one index per row of z0")
    sel_t = None if sel_idx is None else torch.tensor(sel_idx, device=z.device)

    def draw_p():
        p = torch.randn((n_total,) + tuple(z.shape[1:]), generator=gen, device=z.device)
        return p if sel_t is None else p[sel_t]

    def draw_u():
        u = rng.random(n_total)
        return u if sel_idx is None else u[sel_idx]

    U = post.potentials(z)
    Ut, gt = _surrogate_ug(net, z, s2, screen, force)
    samples = [] if record else None
    stage1 = stage2 = proposals = 0
    t0 = time.perf_counter()
    for _ in range(n_iter):
        p = draw_p()
        k0 = 0.5 * (p.double() ** 2).reshape(B, -1).sum(1)
        zq, pq = z.clone(), p - 0.5 * eps * gt
        for l in range(n_leap):
            zq = zq + eps * pq
            Uq, gq = _surrogate_ug(net, zq, s2, screen, force)
            pq = pq - (eps if l + 1 < n_leap else 0.5 * eps) * gq
        k1 = 0.5 * (pq.double() ** 2).reshape(B, -1).sum(1)
        h0 = (Ut + k0).cpu().numpy()
        h1 = (Uq + k1).cpu().numpy()
        finite = np.isfinite(h1) & np.isfinite(h0)
        with np.errstate(over="ignore", invalid="ignore"):
            a1 = finite & (np.log(draw_u()) < np.where(finite, h0 - h1, -np.inf))
        # The judge: one batched forward of the proposals that passed.
        Uy = post.potentials(zq, a1)
        ut_x, ut_y = Ut.cpu().numpy(), Uq.cpu().numpy()
        u2 = np.log(draw_u())
        with np.errstate(over="ignore", invalid="ignore"):
            a2 = a1 & (u2 < np.where(a1, -(Uy - U) + (ut_y - ut_x), -np.inf))
        acc = a2
        proposals += B
        stage1 += int(a1.sum())
        stage2 += int(acc.sum())
        if acc.any():
            sel = torch.tensor(acc, device=z.device)
            z[sel] = zq[sel]
            Ut = torch.where(sel, Uq, Ut)
            gt[sel] = gq[sel]
            U = np.where(acc, Uy, U)
        if record:
            samples.append(z.clone())
    if z.is_cuda:
        torch.cuda.synchronize(z.device)
    dt = time.perf_counter() - t0
    return {"samples": torch.stack(samples) if record else None, "z": z, "U": U,
            "proposals": proposals, "stage1_accepted": stage1, "accepted": stage2,
            "seconds": dt, "accepted_per_s": stage2 / dt}


def plain_hmc(post, z0, n_iter, eps, n_leap, seed=0, threads=None, record=True):
    """HMC with the solver's exact gradient in every leapfrog step. Chains
    run in parallel threads, one posterior model and stream per chain
    (len(z0) <= number of models)."""
    B = z0.shape[0]
    threads = threads or B
    z = z0.clone().float()
    samples = torch.empty((n_iter,) + tuple(z.shape), dtype=torch.float32, device=z.device) \
        if record else None
    accepted = [0] * B
    errors = []

    def chain(k):
        try:
            gen = torch.Generator(device=z.device)
            gen.manual_seed(seed * 1000003 + k)
            rng = np.random.default_rng(seed * 1000003 + k)
            zk = z[k].clone()
            U, g = post.potential_gradient(k, zk)
            for it in range(n_iter):
                p = torch.randn(zk.shape, generator=gen, device=zk.device)
                h0 = U + 0.5 * float((p.double() ** 2).sum())
                zq, pq = zk.clone(), p - 0.5 * eps * g
                for l in range(n_leap):
                    zq = zq + eps * pq
                    Uq, gq = post.potential_gradient(k, zq)
                    pq = pq - (eps if l + 1 < n_leap else 0.5 * eps) * gq
                h1 = Uq + 0.5 * float((pq.double() ** 2).sum())
                if np.isfinite(h1) and np.log(rng.random()) < h0 - h1:
                    zk, U, g = zq, Uq, gq
                    accepted[k] += 1
                if record:
                    samples[it, k] = zk
            z[k] = zk
        except Exception as e:  # reported below
            errors.append(e)

    t0 = time.perf_counter()
    groups = [list(range(t, B, threads)) for t in range(threads)]

    def run(group):
        for k in group:
            chain(k)

    ts = [threading.Thread(target=run, args=(g,)) for g in groups]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    if z.is_cuda:
        torch.cuda.synchronize(z.device)
    dt = time.perf_counter() - t0
    if errors:
        raise errors[0]
    acc = sum(accepted)
    return {"samples": samples, "z": z, "proposals": B * n_iter, "accepted": acc,
            "seconds": dt, "accepted_per_s": acc / dt}
