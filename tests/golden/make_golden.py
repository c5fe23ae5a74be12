"""Generates the golden fixtures under tests/golden/ by running the psvWave
reference's own solver (oracle/_ref/libpsv_ref.so, built from the reference
sources by oracle/build_ref.sh). Run from the repository root:

    python oracle/build.py && python tests/golden/make_golden.py

Fixtures (FP64, bit-exact outputs of the reference):
  small.ini / small_golden.npz -- a 68 x 56 grid, 2 shots, 3 sources, 7
      receivers, 2x2 basis blocks, seeded heterogeneous target and start
      models; forward seismograms, snapshots at one instant, misfit, adjoint
      sources, Lame and velocity kernels, model and gradient vectors.
  nb2.ini -- the configuration of the reference's Notebook 2 FWI example
      (250 x 150 grid, 8000 steps); its known answers are quoted in the tests.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refbind  # noqa: E402

SMALL_INI = """\
; Small test configuration in the reference's INI dialect: values carry
; trailing ';' text and inline comments the way the reference's own files do.
[domain]
nt = 400;                 int
nx_inner = 48;            int
nz_inner = 36;            int
nx_inner_boundary = 4;    int
nz_inner_boundary = 6;    int
dx = 1.249;               float
dz = 1.249;               float
dt = 0.00025;             float

[boundary]
np_boundary = 10;      int
np_factor = 0.05;      float

[medium]; background values
scalar_rho = 1500.0;    float
scalar_vp = 2000.0;     float
scalar_vs = 800.0;      float

[sources]
peak_frequency = 50.0;                  float
n_sources = 3;                          int
n_shots = 2;                            int
source_timeshift = 0.005;
delay_cycles_per_shot = 3; // over f
moment_angles = {90, 45, 180} ;
ix_sources = {10, 30, 38};
iz_sources = {8, 8, 27};
which_source_to_fire_in_which_shot = {{0, 1}, {2}};

[receivers]
nr = 7; !!
ix_receivers = {6, 12, 18, 24, 30, 36, 42}; !!
iz_receivers = {30, 30, 30, 30, 30, 30, 4}; !!

[inversion]
snapshot_interval = 10; int

[basis]
npx = 2
npz = 2

[output]
observed_data_folder = .
stf_folder = .
"""

NB2_INI = """\
[domain]
nt = 8000;                              int
nx_inner = 200;                         int
nz_inner = 100;                         int
nx_inner_boundary = 10;                 int
nz_inner_boundary = 20;                 int
dx = 1.249;                             float
dz = 1.249;                             float
dt = 0.00025;                           float

[boundary]
np_boundary = 25;      int
np_factor = 0.015;     float

[medium]; background values
scalar_rho = 1500.0;    float
scalar_vp = 2000.0;     float
scalar_vs = 800.0;      float

[sources]
peak_frequency = 50.0;                  float
n_sources = 4;                          int
n_shots = 1;                            int
source_timeshift = 0.005;
delay_cycles_per_shot = 24; // over f
moment_angles = {90, 180, 90, 180} ;
ix_sources = {25, 75, 125, 175};
iz_sources = {10, 10, 10, 10};
which_source_to_fire_in_which_shot = {{0, 1, 2, 3}};

[receivers]
nr = 19; !!
ix_receivers = {10, 20, 30, 40, 50, 60, 70, 80, 90, 100, 110, 120, 130, 140, 150, 160, 170, 180, 190}; !!
iz_receivers = {90, 90, 90, 90, 90, 90, 90, 90, 90, 90, 90, 90, 90, 90, 90, 90, 90, 90, 90}; !!

[inversion]
snapshot_interval = 10; int

[basis]
npx = 1
npz = 1

[output]
observed_data_folder = .
stf_folder = .
"""


def small_media(nx, nz, seed=7):
    """Seeded smooth heterogeneous target and start media for the small grid."""
    rng = np.random.default_rng(seed)
    x = np.arange(nx)[:, None]
    z = np.arange(nz)[None, :]
    base_vp = 2000.0 + 4.0 * z + 0 * x
    base_vs = base_vp / 2.3
    base_rho = 1500.0 + 1.5 * z + 0 * x
    cx, cz = rng.uniform(25, 45), rng.uniform(22, 34)
    blob = np.exp(-((x - cx) ** 2 + (z - cz) ** 2) / (2 * 5.0 ** 2))
    tgt = (base_vp * (1 + 0.08 * blob), base_vs * (1 - 0.1 * blob), base_rho * (1 + 0.05 * blob))
    start = (base_vp, base_vs, base_rho)
    return tgt, start


def nb2_media(nx, nz, np_boundary, dx, dz):
    """Notebook 2's targets: three r < 15 m circles on a 2000/800/1500
    background; start = background."""
    IX, IZ = np.meshgrid((np.arange(nx) - np_boundary) * dx, (np.arange(nz) - np_boundary) * dz,
                         indexing="ij")
    vp0 = np.full((nx, nz), 2000.0)
    vs0 = np.full((nx, nz), 800.0)
    rho0 = np.full((nx, nz), 1500.0)
    zm = (IZ.max() + IZ.min()) / 2
    c = ((IX - (IX.max() + IX.min()) / 2) ** 2 + (IZ - zm) ** 2) ** 0.5 < 15
    vs = vs0 * (1 - 0.1 * c)
    vp = vp0 * (1 - 0.1 * c)
    rho = rho0.copy()
    c = ((IX - (IX.max() + IX.min()) / 6) ** 2 + (IZ - zm) ** 2) ** 0.5 < 15
    vs = vs * (1 + 0.1 * c)
    rho = rho * (1 + 0.1 * c)
    c = ((IX - (IX.max() + IX.min()) * 5 / 6) ** 2 + (IZ - zm) ** 2) ** 0.5 < 15
    vp = vp * (1 + 0.1 * c)
    rho = rho * (1 + 0.1 * c)
    return (vp, vs, rho), (vp0, vs0, rho0)


def fwi_gradient(m, target, start):
    """Observed data from `target`, then one gradient at `start` (the
    reference's documented call order, src/psvWave.cpp:518-545)."""
    m.set_parameter_fields(*target)
    for s in range(m.n_shots):
        m.forward_simulate(s, True)
    m.set_observed_data(*m.get_synthetic_data())
    m.set_parameter_fields(*start)
    for s in range(m.n_shots):
        m.forward_simulate(s, True)
    misfit = m.calculate_l2_misfit()
    m.calculate_l2_adjoint_sources()
    m.reset_kernels()
    for s in range(m.n_shots):
        m.adjoint_simulate(s)
    m.map_kernels_to_velocity()
    return misfit


def main():
    if not refbind.available():
        raise SystemExit("oracle/_ref/libpsv_ref.so missing: run oracle/build.py first")
    small = os.path.join(HERE, "small.ini")
    with open(small, "w") as f:
        f.write(SMALL_INI)
    with open(os.path.join(HERE, "nb2.ini"), "w") as f:
        f.write(NB2_INI)
    m = refbind.RefModel(small)
    target, start = small_media(m.nx, m.nz)
    misfit = fwi_gradient(m, target, start)
    out = {
        "info": np.array([m.info[k] for k in refbind.INFO_FIELDS]),
        "target": np.stack(target), "start": np.stack(start),
        "taper": m.array("taper"), "stf": m.array("stf"), "moment": m.array("moment"),
        "rtf_ux": m.array("rtf_ux"), "rtf_uz": m.array("rtf_uz"),
        "obs_ux": m.array("rtf_ux_true"), "obs_uz": m.array("rtf_uz_true"),
        "a_stf_ux": m.array("a_stf_ux"), "a_stf_uz": m.array("a_stf_uz"),
        "misfit": np.array(misfit),
        "lambda_kernel": m.array("lambda_kernel"), "mu_kernel": m.array("mu_kernel"),
        "density_l_kernel": m.array("density_l_kernel"),
        "vp_kernel": m.array("vp_kernel"), "vs_kernel": m.array("vs_kernel"),
        "density_v_kernel": m.array("density_v_kernel"),
        "model_vector": m.get_model_vector(), "gradient_vector": m.get_gradient_vector(),
        # Forward snapshot of shot 1 at snapshot index 25 (step 250), all fields.
        "snap_shot1_25": np.stack([m.array(n)[1, 25] for n in
                                   ("accu_vx", "accu_vz", "accu_txx", "accu_tzz", "accu_txz")]),
        # Adjoint wave fields after the last adjoint call (shot 1, it = 0).
        "adjoint_fields": np.stack([m.array(n) for n in ("vx", "vz", "txx", "tzz", "txz")]),
    }
    np.savez_compressed(os.path.join(HERE, "small_golden.npz"), **out)
    print("small: misfit %.12g, |g|inf %.6g" % (misfit, np.abs(out["gradient_vector"]).max()))


if __name__ == "__main__":
    main()
