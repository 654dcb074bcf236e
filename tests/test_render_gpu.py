"""GPU: the wavefront path tracer against the CPU oracle of the reference's estimator (same PCG
sequence, so images agree sample by sample up to FP contraction), the light table against the
restated Vose build, and convergence/unbiasedness against an FP64-accumulated high-spp image."""
import numpy as np
import pytest
import torch

import gbpt
import pyoracle
from gbpt import scenes

pytestmark = pytest.mark.gpu


def _emitter_scene(n_emit=64, seed=3):
    """Heightfield with small emissive triangles of log-uniform radiance above it."""
    rng = np.random.Generator(np.random.PCG64(seed))
    hf = scenes.heightfield(cells=24, amplitude=0.2, seed=seed)
    em = scenes.random_triangles(n_emit, seed=seed + 1, lo=(-0.8, 0.35, -0.8), hi=(0.8, 0.9, 0.8), sigma=0.05)
    mesh = scenes.merge(hf, em)
    n_hf = hf.n_triangles
    mat_of = np.concatenate([np.zeros(n_hf, np.int32), 1 + np.arange(n_emit, dtype=np.int32)])
    albedo = np.concatenate([[[0.6, 0.5, 0.4]], np.full((n_emit, 3), 0.5)]).astype(np.float32)
    rad = np.exp(rng.uniform(0, np.log(1000), n_emit))
    emission = np.concatenate([[[0, 0, 0]], rad[:, None] * rng.uniform(0.2, 1.0, (n_emit, 3))]).astype(np.float32)
    return mesh, mat_of, albedo, emission


def _render(scene, settings, launches=1):
    r = gbpt.Renderer(scene, settings)
    r.render(launches)
    torch.cuda.synchronize()
    a32, a64 = r.image_sums()
    return r, a32, a64


def _oracle(scene_args, scene, settings, spp):
    mesh, mat_of, albedo, emission = scene_args
    lt = scene.light_table()
    return pyoracle.pt_render(mesh.triangle_soup(), mat_of, albedo, emission, lt["emissive"], lt["probas"],
                              lt["alias"], lt["power_sum"], settings, spp)


def _compare(gpu, orc):
    denom = np.maximum(np.abs(orc), 1e-3)
    rel = np.abs(gpu - orc) / denom
    frac_close = float((rel.max(axis=-1) < 1e-3).mean())
    mean_rel = abs(gpu.mean() - orc.mean()) / orc.mean()
    return frac_close, mean_rel


def test_cornell_matches_oracle_sample_by_sample(cuda):
    cb = scenes.cornell_box()
    st = gbpt.cornell_settings(48, 48, samples_per_launch=8)
    scene = gbpt.Scene.from_cornell(cb)
    _, _, gpu = _render(scene, st)
    orc = _oracle((cb.mesh, cb.material_of_triangle, cb.albedo, cb.emission), scene, st, 8)
    frac_close, mean_rel = _compare(gpu, orc)
    assert frac_close > 0.97, frac_close
    assert mean_rel < 2e-3, mean_rel


def test_power_sampling_many_emitters_matches_oracle(cuda):
    args = _emitter_scene()
    mesh, mat_of, albedo, emission = args
    scene = gbpt.Scene(mesh.positions, mesh.indices, mat_of, albedo, emission)
    iv, ip = gbpt.look_at_camera((0.0, 1.6, -2.2), (0.0, 0.0, 0.0), vfov_deg=45.0)
    st = gbpt.RenderSettings(width=40, height=40, samples_per_launch=4, nb_bounces=3, light_sampling=gbpt.render.LIGHT_POWER,
                             russian_roulette_min_depth=2, inverse_view=iv, inverse_projection=ip)
    _, _, gpu = _render(scene, st)
    orc = _oracle(args, scene, st, 4)
    frac_close, mean_rel = _compare(gpu, orc)
    assert frac_close > 0.95, frac_close
    assert mean_rel < 5e-3, mean_rel


def test_light_table_matches_vose_restatement(cuda):
    mesh, mat_of, albedo, emission = _emitter_scene(n_emit=500, seed=5)
    scene = gbpt.Scene(mesh.positions, mesh.indices, mat_of, albedo, emission)
    lt = scene.light_table()
    # emissive list in triangle order, power list in the reference's float order (bit-exact)
    want_emissive = np.nonzero(np.any(emission[mat_of] != 0, axis=1))[0]
    assert np.array_equal(lt["emissive"], want_emissive)
    p32 = pyoracle.emissive_power(mesh.triangle_soup(), mat_of, emission, lt["emissive"])
    exact64 = p32.astype(np.float64).sum()
    assert abs(lt["power_sum64"] - exact64) <= 1e-12 * exact64
    assert lt["power_sum"] == np.float32(lt["power_sum64"])
    # same table as Utils::compute_alias_table restated, given the same power list and FP64 sum
    prob, alias = pyoracle.vose_alias(p32, lt["power_sum64"])
    assert np.array_equal(prob, lt["probas"])
    assert np.array_equal(alias, lt["alias"])
    dist = pyoracle.alias_distribution(lt["probas"], lt["alias"])
    assert np.allclose(dist, p32 / p32.astype(np.float64).sum(), rtol=1e-5, atol=1e-9)


def test_deterministic_and_fp64_matches_fp32(cuda):
    cb = scenes.cornell_box()
    st = gbpt.cornell_settings(32, 32, samples_per_launch=4)
    scene = gbpt.Scene.from_cornell(cb)
    _, a32, a64 = _render(scene, st, launches=2)
    _, b32, b64 = _render(scene, st, launches=2)
    assert np.array_equal(a64, b64) and np.array_equal(a32, b32)
    assert np.allclose(a32, a64, rtol=1e-5, atol=1e-4)


def test_relmse_decreases_and_unbiased_over_seeds(cuda):
    """relMSE against a 16384-spp FP64 image falls ~1/spp; the mean of 64 seeds agrees with the
    FP64 image within 3 sigma (Russian roulette clamp off, as the unbiasedness test requires)."""
    cb = scenes.cornell_box()
    scene = gbpt.Scene.from_cornell(cb)
    ref_st = gbpt.cornell_settings(32, 32, samples_per_launch=1024, seed=1000)
    _, _, ref = _render(scene, ref_st, launches=16)
    ref = ref / 16384.0

    def relmse(img):
        return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))

    errs = []
    for spp in (16, 64, 256):
        st = gbpt.cornell_settings(32, 32, samples_per_launch=spp, seed=7)
        _, _, img = _render(scene, st)
        errs.append(relmse(img / spp))
    assert errs[0] > errs[1] > errs[2]
    assert errs[0] / errs[2] > 8.0  # ideal 16x for a 16x spp increase

    means = []
    for seed in range(64):
        st = gbpt.cornell_settings(32, 32, samples_per_launch=16, seed=seed + 1)
        _, _, img = _render(scene, st)
        means.append((img / 16).mean())
    means = np.array(means)
    sigma = means.std(ddof=1) / np.sqrt(len(means))
    assert abs(means.mean() - ref.mean()) < 3 * sigma + 1e-6, (means.mean(), ref.mean(), sigma)


def test_pass_entry_points_equal_render(cuda):
    cb = scenes.cornell_box()
    st = gbpt.cornell_settings(24, 24, samples_per_launch=2)
    scene = gbpt.Scene.from_cornell(cb)
    _, _, full = _render(scene, st)
    r = gbpt.Renderer(scene, st)
    r.pass_camera_rays()
    for b in range(st.nb_bounces + 1):
        r.pass_bounce(b)
    r.pass_accumulate()
    _, parts = r.image_sums()
    assert np.array_equal(full, parts)
    s = r.stats()
    assert s["samples"] == 24 * 24 * 2 and s["extension_rays"] >= 24 * 24 * 2


def test_sample_range_shards_add_up_to_the_full_image(cuda):
    """Two renderers covering launches [0, 3) and [3, 5) (set_sample_index) sum to the 5-launch
    image: the sharding the multi-GPU path uses, one renderer per rank."""
    from gbpt import sharding
    cb = scenes.cornell_box()
    scene = gbpt.Scene.from_cornell(cb)
    st = gbpt.cornell_settings(32, 32, samples_per_launch=2, seed=4)
    _, _, full = _render(scene, st, launches=5)
    total = np.zeros_like(full)
    for rank in range(2):
        first, count = sharding.sample_range(rank, 2, 5)
        r = gbpt.Renderer(scene, st)
        r.set_sample_index(first * st.samples_per_launch)
        r.render(count)
        torch.cuda.synchronize()
        total += r.image_sums()[1]
    np.testing.assert_allclose(total, full, rtol=1e-12, atol=1e-12)
