"""Seeded synthetic workloads with the shapes of the benchmark
configurations: model parameters (fdModel.from_parameters keywords) and
media (vp, vs, rho on the padded [nx][nz] grid).

* c0 -- 200 x 100 inner cells, 25-cell Cerjan boundary (factor 0.015),
  dx = dz = 1.249, dt = 2.5e-4, nt = 4000; homogeneous 2000/800/1500 with a
  radius-15-cell inclusion of +10 % vp, vs, rho at a seeded position; two
  reverse-fault sources (dips 45 and 60 degrees) in one shot, Ricker 50 Hz,
  delay_cycles_per_shot 24; 19 receivers along z = 10; snapshot interval 10.
* c1 -- 2000 x 800 inner cells, 50-cell boundary, dx = dz = 5, dt = 4e-4,
  nt = 5000; 30 horizontal layers with vp drawn uniformly in [1500, 4500]
  and sorted to increase with depth, vs = vp / 1.73, rho = 310 vp^0.25
  (Gardner), times a smooth Gaussian random field (sigma 5 %, correlation
  length 40 cells); one explosive + dip source (an isotropic tensor plus
  the 45-degree dip tensor, c1_moment), Ricker 15 Hz; 400 receivers along
  z = 5.
* c2 -- many models of uneven sizes (c2_models).
* c3 -- 1000 x 400 inner cells, 50-cell boundary, dx = dz = 5, dt = 4e-4
  (CFL number 0.59 at vp 4500), nt = 6000; 8 shots of one 45-degree source
  each, evenly spaced along z = 10, Ricker 25 Hz; 200 receivers along
  z = 5. True medium: 30 layers as c1 (no random field) plus 3 seeded
  elliptic anomalies of +-15 % vs; start medium: the true one smoothed by a
  Gaussian of 20 cells.
"""
import numpy as np


def c0_params():
    return dict(nt=4000, nx_inner=200, nz_inner=100, nx_inner_boundary=10, nz_inner_boundary=20,
                dx=1.249, dz=1.249, dt=2.5e-4, np_boundary=25, np_factor=0.015,
                scalar_rho=1500.0, scalar_vp=2000.0, scalar_vs=800.0, npx=1, npz=1,
                peak_frequency=50.0, source_timeshift=0.0, delay_cycles_per_shot=24,
                n_sources=2, ix_sources=[66, 133], iz_sources=[50, 50], moment_angles=[45.0, 60.0],
                which_source_to_fire_in_which_shot=[[0, 1]], nr=19,
                ix_receivers=[10 + 10 * k for k in range(19)], iz_receivers=[10] * 19,
                snapshot_interval=10)


def c0_media(seed=0):
    p = c0_params()
    nx, nz = p["nx_inner"] + 2 * p["np_boundary"], p["nz_inner"] + 2 * p["np_boundary"]
    rng = np.random.default_rng(seed)
    cx = p["np_boundary"] + rng.uniform(40, p["nx_inner"] - 40)
    cz = p["np_boundary"] + rng.uniform(30, p["nz_inner"] - 30)
    x = np.arange(nx)[:, None]
    z = np.arange(nz)[None, :]
    inside = ((x - cx) ** 2 + (z - cz) ** 2) < 15.0 ** 2
    start = tuple(np.full((nx, nz), v) for v in (2000.0, 800.0, 1500.0))
    target = tuple(a * (1 + 0.1 * inside) for a in start)
    return target, start


def c1_params(nt=5000):
    n_rec = 400
    return dict(nt=nt, nx_inner=2000, nz_inner=800, nx_inner_boundary=10, nz_inner_boundary=10,
                dx=5.0, dz=5.0, dt=4e-4, np_boundary=50, np_factor=0.015,
                scalar_rho=2000.0, scalar_vp=2500.0, scalar_vs=1445.0, npx=1, npz=1,
                peak_frequency=15.0, source_timeshift=0.0, delay_cycles_per_shot=0,
                n_sources=1, ix_sources=[1000], iz_sources=[10], moment_angles=[45.0],
                which_source_to_fire_in_which_shot=[[0]], nr=n_rec,
                ix_receivers=[2 + 5 * k for k in range(n_rec)], iz_receivers=[5] * n_rec,
                snapshot_interval=10)


def c1_moment(dip_degrees=45.0):
    """The explosive + dip source of c1 as one full moment tensor [1][2][2]:
    an isotropic part diag(1, 1) plus the reference's dip-angle tensor
    [[cos t, -sin t], [-sin t, -cos t]] (src/fdModel.cpp:233-246, with its
    PI = 3.14159265), both scaled by 1e15 as the reference scales its
    tensors. Set it with fdModel.set_moment after construction; the
    reference's dip-angle parameterisation alone has no isotropic part."""
    t = dip_degrees * 3.14159265 / 180.0
    dip = np.array([[np.cos(t), -np.sin(t)], [-np.sin(t), -np.cos(t)]])
    return ((np.eye(2) + dip) * 1e15)[None]


def c1_model(nt=5000, precision="fp32", device=0, seed=1):
    """An fdModel of the c1 workload: c1_params(nt), the explosive + dip
    tensor of c1_moment, and the c1_media(seed) medium."""
    from .model import fdModel

    m = fdModel.from_parameters(c1_params(nt=nt), precision=precision, device=device)
    m.set_moment(c1_moment())
    m.set_parameter_fields(*c1_media(seed))
    return m


def gaussian_random_field(shape, corr_len, sigma, rng):
    """Zero-mean field with a Gaussian covariance of length `corr_len`
    cells and standard deviation `sigma` (FFT-filtered white noise)."""
    noise = rng.standard_normal(shape)
    kx = np.fft.fftfreq(shape[0])[:, None]
    kz = np.fft.rfftfreq(shape[1])[None, :]
    filt = np.exp(-2.0 * (np.pi * corr_len) ** 2 * (kx ** 2 + kz ** 2) / 2.0)
    f = np.fft.irfft2(np.fft.rfft2(noise) * filt, s=shape)
    f -= f.mean()
    return f * (sigma / f.std())


def layered_media(nx, nz, np_boundary, n_layers, seed, vp_range=(1500.0, 4500.0),
                  sigma=0.05, corr_len=40.0):
    rng = np.random.default_rng(seed)
    vps = np.sort(rng.uniform(vp_range[0], vp_range[1], n_layers))
    inner = nz - 2 * np_boundary
    depth = np.clip(np.arange(nz) - np_boundary, 0, inner - 1)
    layer = np.minimum((depth * n_layers) // inner, n_layers - 1)
    vp = np.repeat(vps[layer][None, :], nx, axis=0)
    vp = vp * (1.0 + gaussian_random_field((nx, nz), corr_len, sigma, rng))
    vs = vp / 1.73
    rho = 310.0 * vp ** 0.25
    return vp, vs, rho


def c1_media(seed=1):
    p = c1_params()
    nx, nz = p["nx_inner"] + 2 * p["np_boundary"], p["nz_inner"] + 2 * p["np_boundary"]
    return layered_media(nx, nz, p["np_boundary"], 30, seed)


def c2_models(n_models=256, nt=1000, seed=2):
    """The batching workload: n_models independent models of uneven sizes,
    nx_inner uniform in [200, 800] and nz_inner in [100, 400], each with a
    25-cell boundary and 1-4 shots (one source per shot, evenly spaced at
    z = 10), Ricker 20-50 Hz, 50 receivers along z = 5, seeded layered +
    Gaussian-random media as c1. dx = dz = 5, dt = 4e-4, and nt = 1000
    steps (the configuration leaves nt open). Returns [(params, media)]."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_models):
        nxi = int(rng.integers(200, 801))
        nzi = int(rng.integers(100, 401))
        shots = int(rng.integers(1, 5))
        nb = 25
        xs = [int(nxi * (s + 1) / (shots + 1)) for s in range(shots)]
        nr = 50
        p = dict(nt=nt, nx_inner=nxi, nz_inner=nzi, nx_inner_boundary=10, nz_inner_boundary=10,
                 dx=5.0, dz=5.0, dt=4e-4, np_boundary=nb, np_factor=0.015,
                 scalar_rho=2000.0, scalar_vp=2500.0, scalar_vs=1445.0, npx=1, npz=1,
                 peak_frequency=float(rng.uniform(20.0, 50.0)), source_timeshift=0.0,
                 delay_cycles_per_shot=0, n_sources=shots, ix_sources=xs,
                 iz_sources=[10] * shots,
                 moment_angles=[float(a) for a in rng.uniform(0.0, 180.0, shots)],
                 which_source_to_fire_in_which_shot=[[s] for s in range(shots)], nr=nr,
                 ix_receivers=[int(2 + (nxi - 4) * r / (nr - 1)) for r in range(nr)],
                 iz_receivers=[5] * nr, snapshot_interval=nt)
        media = layered_media(nxi + 2 * nb, nzi + 2 * nb, nb, 30, seed=1000 * seed + k,
                              corr_len=20.0)
        out.append((p, media))
    return out


def c3_params(nt=6000, n_shots=8, nx_inner=1000, nz_inner=400, n_rec=200):
    """The differentiation workload (smaller variants for tests: fewer steps,
    shots, cells or receivers)."""
    xs = [int(nx_inner * (k + 0.5) / n_shots) for k in range(n_shots)]
    rec = [int(2 + (nx_inner - 4) * r / max(1, n_rec - 1)) for r in range(n_rec)]
    return dict(nt=nt, nx_inner=nx_inner, nz_inner=nz_inner, nx_inner_boundary=10,
                nz_inner_boundary=10, dx=5.0, dz=5.0, dt=4e-4, np_boundary=50, np_factor=0.015,
                scalar_rho=2000.0, scalar_vp=2500.0, scalar_vs=1445.0, npx=1, npz=1,
                peak_frequency=25.0, source_timeshift=0.0, delay_cycles_per_shot=0,
                n_sources=n_shots, ix_sources=xs, iz_sources=[10] * n_shots,
                moment_angles=[45.0] * n_shots,
                which_source_to_fire_in_which_shot=[[k] for k in range(n_shots)], nr=n_rec,
                ix_receivers=rec, iz_receivers=[5] * n_rec, snapshot_interval=10)


def gaussian_smooth(a, sigma):
    """Gaussian smoothing with edge replication (FFT on a padded copy)."""
    pad = int(4 * sigma)
    b = np.pad(a, pad, mode="edge")
    kx = np.fft.fftfreq(b.shape[0])[:, None]
    kz = np.fft.rfftfreq(b.shape[1])[None, :]
    filt = np.exp(-2.0 * (np.pi * sigma) ** 2 * (kx ** 2 + kz ** 2))
    out = np.fft.irfft2(np.fft.rfft2(b) * filt, s=b.shape)
    return out[pad:pad + a.shape[0], pad:pad + a.shape[1]]


def c3_media(params=None, seed=3):
    """(true, start) media of the differentiation workload for `params`
    (default c3_params())."""
    p = params or c3_params()
    nb = p["np_boundary"]
    nx, nz = p["nx_inner"] + 2 * nb, p["nz_inner"] + 2 * nb
    rng = np.random.default_rng(seed)
    vps = np.sort(rng.uniform(1500.0, 4500.0, 30))
    inner = nz - 2 * nb
    depth = np.clip(np.arange(nz) - nb, 0, inner - 1)
    vp = np.repeat(vps[np.minimum((depth * 30) // inner, 29)][None, :], nx, axis=0)
    vs = vp / 1.73
    x = np.arange(nx)[:, None]
    z = np.arange(nz)[None, :]
    for sign in (1.0, -1.0, 1.0):
        cx = nb + rng.uniform(0.15, 0.85) * p["nx_inner"]
        cz = nb + rng.uniform(0.3, 0.8) * p["nz_inner"]
        ax = rng.uniform(0.04, 0.1) * p["nx_inner"]
        az = rng.uniform(0.04, 0.1) * p["nz_inner"]
        inside = ((x - cx) / ax) ** 2 + ((z - cz) / az) ** 2 < 1.0
        vs = np.where(inside, vs * (1.0 + sign * 0.15), vs)
    rho = 310.0 * vp ** 0.25
    true = (vp, vs, rho)
    start = tuple(gaussian_smooth(a, 20.0) for a in true)
    return true, start


def c4_params(nt=2000, peak_frequency=15.0):
    """The surrogate Monte Carlo workload: the c0 grid (200 x 100 inner
    cells, 25-cell boundary, dx = dz = 1.249) with dt = 2e-4 (c0's 2.5e-4
    is reduced so that prior draws 4 sigma above the mean stay inside the CFL
    limit), nt = 2000; c0's two sources (45 and 60 degrees) fired together
    without delay, 19 receivers along z = 10. The Ricker wavelet peaks at
    15 Hz: a 10 % velocity change shifts the two-way travel time through the
    model by about 12 ms, under the 33 ms half-period, so prior draws stay
    within half a cycle of the data (at c0's 50 Hz they would not)."""
    p = c0_params()
    p.update(nt=nt, dt=2e-4, delay_cycles_per_shot=0, snapshot_interval=10,
             peak_frequency=peak_frequency)
    return p


C4_COARSE = (20, 10)


def c4_prior():
    """Mean and standard deviation [3][20][10] of the coarse parameters (vp,
    vs, rho): a layered mean, vp from 1600 m/s at the top coarse row to 2200
    m/s at the bottom, vs = 0.45 vp, rho = 310 vp^0.25 (Gardner); sigma =
    10 % of the mean."""
    ncx, ncz = C4_COARSE
    vp = np.repeat((1600.0 + 600.0 * np.arange(ncz) / (ncz - 1))[None, :], ncx, axis=0)
    mean = np.stack([vp, 0.45 * vp, 310.0 * vp ** 0.25])
    return mean, 0.1 * mean
