"""Batched forward simulation: members of uneven sizes advanced together
give exactly the seismograms that each model's own forward_simulate gives
(same step kernel, same tile shape), with and without CUDA-graph replay."""
import numpy as np
import pytest

import psvwave_gb300 as psv
from psvwave_gb300 import workloads

pytestmark = pytest.mark.gpu


def small_models(n=3, nt=300):
    models = []
    for p, media in workloads.c2_models(n_models=n, nt=nt, seed=5):
        p = dict(p)
        m = psv.fdModel.from_parameters(p)
        m.set_parameter_fields(*media)
        models.append(m)
    return models


@pytest.mark.parametrize("shape", ["16x28", "20x28", "32x60", "16x60"])
@pytest.mark.parametrize("persistent", [True, False])
def test_batch_matches_individual_runs(shape, persistent):
    models = small_models()
    ref = []
    for m in models:
        m.kernel_variant = "fused_tma"  # the batch's step kernel
        m.tile_shape = shape
        out = []
        for s in range(m.n_shots):
            m.forward_simulate(s, False)
            out.append([a[s].copy() for a in m.get_synthetic_data()])
        ref.append(out)
        m.set_synthetic_data(*[np.zeros_like(a) for a in m.get_synthetic_data()])
    b = psv.Batch()
    for m in models:
        b.add_all_shots(m)
    b.tile_shape = shape
    b.persistent = persistent
    info = b.info()
    assert info["members"] == sum(m.n_shots for m in models)
    for _ in range(3):  # eager, graph capture, graph replay
        b.forward()
        for m, out in zip(models, ref):
            ux, uz = m.get_synthetic_data()
            for s in range(m.n_shots):
                assert np.array_equal(ux[s], out[s][0])
                assert np.array_equal(uz[s], out[s][1])


def test_batch_rejects_mixed_nt_and_fp64():
    a = small_models(1, nt=300)[0]
    p, media = workloads.c2_models(n_models=1, nt=200, seed=6)[0]
    other = psv.fdModel.from_parameters(p)
    b = psv.Batch()
    b.add(a, 0)
    with pytest.raises(ValueError):
        b.add(other, 0)
    p64 = dict(p)
    m64 = psv.fdModel.from_parameters(p64, precision="fp64")
    with pytest.raises(ValueError):
        b.add(m64, 0)


def test_batch_autotune_picks_a_shape():
    models = small_models(2, nt=200)
    b = psv.Batch()
    for m in models:
        b.add_all_shots(m)
    assert b.autotune(20) in ("32x60", "16x28", "20x28", "16x60")


@pytest.mark.parametrize("persistent", [True, False])
def test_batch_subset_matches_full_run(persistent):
    # Members switched off keep their previous seismograms; the others match
    # a full run bit for bit, with the captured loop reused across subsets.
    models = small_models()
    b = psv.Batch()
    for m in models:
        b.add(m, 0)
    b.persistent = persistent
    b.forward()
    full = [m.get_synthetic_data() for m in models]
    for m in models:
        m.set_synthetic_data(*[np.zeros_like(a) for a in m.get_synthetic_data()])
    mask = [k % 2 == 0 for k in range(len(models))]
    for _ in range(3):
        b.set_active(mask)
        b.forward()
    for k, m in enumerate(models):
        ux, uz = m.get_synthetic_data()
        if mask[k]:
            assert np.array_equal(ux[0], full[k][0][0]) and np.array_equal(uz[0], full[k][1][0])
        else:
            assert not ux[0].any() and not uz[0].any()


def test_batch_misfits_equal_each_models_misfit():
    # One reduction per active member, bit for bit what each model's own
    # calculate_l2_misfit gives; NaN for members switched off.
    models = small_models()
    for m in models:
        m.set_observed_data(*[0.5 * a for a in m.get_synthetic_data()])
    b = psv.Batch()
    for m in models:
        b.add(m, 0)
    mask = [True, False, True]
    b.set_active(mask)
    b.forward()
    mis = b.misfits()
    assert mis.shape == (len(models),)
    for k, m in enumerate(models):
        if mask[k]:
            assert mis[k] == m.misfit  # the model's misfit is updated
            m.calculate_l2_misfit()
            assert mis[k] == m.misfit and mis[k] > 0
        else:
            assert np.isnan(mis[k])


def cluster_models(nt=300):
    # c0-size members and a smaller one: every member fits a cluster.
    models = []
    for k, (nxi, nzi) in enumerate([(200, 100), (200, 100), (120, 64)]):
        p = dict(workloads.c0_params(), nt=nt, nx_inner=nxi, nz_inner=nzi)
        p["ix_sources"] = [nxi // 3, 2 * nxi // 3]
        p["iz_sources"] = [nzi // 2, nzi // 2]
        p["ix_receivers"] = [5 + 5 * j for j in range(19)]
        m = psv.fdModel.from_parameters(p)
        nx, nz = m.nx, m.nz
        rng = np.random.default_rng(10 + k)
        vp = 2000.0 * (1 + 0.05 * rng.standard_normal((nx, nz)))
        m.set_parameter_fields(vp, 0.4 * vp, np.full((nx, nz), 1500.0))
        models.append(m)
    return models


def test_batch_cluster_scheme_matches_model_cluster_runs():
    # Every member in its own cluster, all in one launch: each model's own
    # cluster-resident run (variant fused_cluster) bit for bit, for the
    # members switched on; the others keep their seismograms.
    models = cluster_models()
    ref = []
    for m in models:
        m.kernel_variant = "fused_cluster"
        m.forward_simulate(0, False)
        ref.append([a.copy() for a in m.get_synthetic_data()])
        m.set_synthetic_data(*[np.zeros_like(a) for a in m.get_synthetic_data()])
    b = psv.Batch()
    for m in models:
        b.add(m, 0)
    assert b.cluster_fits
    b.cluster = True
    assert b.cluster
    for _ in range(3):  # eager, graph capture, graph replay
        b.forward()
        for m, out in zip(models, ref):
            ux, uz = m.get_synthetic_data()
            assert np.array_equal(ux, out[0]) and np.array_equal(uz, out[1])
    for m in models:
        m.set_synthetic_data(*[np.zeros_like(a) for a in m.get_synthetic_data()])
    mask = [True, False, True]
    b.set_active(mask)
    b.forward()
    for k, m in enumerate(models):
        ux, uz = m.get_synthetic_data()
        if mask[k]:
            assert np.array_equal(ux, ref[k][0]) and np.array_equal(uz, ref[k][1])
        else:
            assert not ux.any() and not uz.any()
    b.persistent = False  # switches the cluster scheme off
    assert not b.cluster


def test_batch_cluster_scheme_refused_for_large_members():
    models = small_models(2)  # c2-size members, too large for a cluster
    b = psv.Batch()
    for m in models:
        b.add(m, 0)
    if not b.cluster_fits:
        with pytest.raises(ValueError):
            b.cluster = True


def test_batch_sets_member_media_from_one_device_tensor():
    # One call sets the flagged members' media from rows of a device tensor:
    # the same seismograms as each model's own set_parameter_fields.
    import torch

    models = cluster_models(nt=200)[:2] + cluster_models(nt=200)[:1]
    shapes = {(m.nx, m.nz) for m in models}
    assert len(shapes) == 1  # rows of one tensor
    nx, nz = models[0].nx, models[0].nz
    rng = np.random.default_rng(3)
    media = []
    for _ in models:
        vp = 2000.0 * (1 + 0.05 * rng.standard_normal((nx, nz)))
        media.append((vp, 0.45 * vp, np.full((nx, nz), 1600.0)))
    ref = []
    for m, md in zip(models, media):
        m.kernel_variant = "fused_tma"
        m.tile_shape = "20x28"
        m.set_parameter_fields(*md)
        m.forward_simulate(0, False)
        ref.append([a.copy() for a in m.get_synthetic_data()])
        m.set_parameter_fields(*[np.full((nx, nz), v) for v in (2000.0, 800.0, 1500.0)])
    b = psv.Batch()
    for m in models:
        b.add(m, 0)
    b.tile_shape = "20x28"
    fields = torch.tensor(np.stack([np.stack(md) for md in media]), dtype=torch.float64,
                          device="cuda")
    b.set_parameter_fields_device(fields, [True, False, True])
    b.forward()
    for k, m in enumerate(models):
        if k == 1:
            assert np.allclose(m.get_parameter_fields()[0], 2000.0)
            continue
        ux, uz = m.get_synthetic_data()
        assert np.array_equal(ux, ref[k][0]) and np.array_equal(uz, ref[k][1])
        assert np.array_equal(m.get_parameter_fields()[0], media[k][0])
