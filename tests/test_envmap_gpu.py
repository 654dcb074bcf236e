"""GPU: the world around the scene — uniform ambient light and an environment map importance
sampled by alias table or CDF search, or found only by misses (the reference's ESS_ALIAS_TABLE /
ESS_BINARY_SEARCH / ESS_NO_SAMPLING, src/Device/includes/LightSampling/Envmap.h) — in the
wavefront path tracer. Device tables (RGB9E5 texels, FP64 CDF, alias table) against the oracle's
build; images against the oracle drawing the same random numbers (sample by sample) for Lambertian
and principled scenes, with one-light MIS and RIS direct lighting; the sampled estimators against
the miss-only one on a smooth sky; world changes, black and zero-intensity envmaps, batching."""
import os

import numpy as np
import pytest
import torch

import gbpt
import pyoracle
from gbpt import GbptError, scenes
from gbpt.render import (AMBIENT_ENVMAP, AMBIENT_NONE, AMBIENT_UNIFORM, BSDF_PRINCIPLED, DIRECT_RIS,
                         ENVMAP_ALIAS_TABLE, ENVMAP_BINARY_SEARCH, ENVMAP_NO_SAMPLING, RenderSettings, World)

pytestmark = pytest.mark.gpu

GOLDEN = os.path.dirname(os.path.abspath(__file__)) + "/golden/"
ROT = np.array([[0.8, 0.0, 0.6], [0.0, 1.0, 0.0], [-0.6, 0.0, 0.8]], np.float32)


def _render(scene, st, launches=1):
    r = gbpt.Renderer(scene, st)
    r.render(launches)
    torch.cuda.synchronize()
    return r.image_sums()[1]


def _close(gpu, orc):
    rel = np.abs(gpu - orc) / np.maximum(np.abs(orc), 1e-3)
    return float((rel.max(axis=-1) < 1e-3).mean())


def _settings(spp, seed=3, w=40, h=40, **kw):
    """The Cornell box seen from further out (60 degree FOV): the image frame shows the sky around
    the box, and the sky lights the box through its open side."""
    iv, ip = gbpt.look_at_camera((2.75, 2.75, -8.0), (2.75, 2.75, 0.0), vfov_deg=60.0, aspect=w / h)
    return gbpt.cornell_settings(w, h, samples_per_launch=spp, seed=seed, inverse_view=iv, inverse_projection=ip, **kw)


def _cornell(world):
    cb = scenes.cornell_box()
    scene = gbpt.Scene.from_cornell(cb)
    scene.set_world(world)
    return cb, scene


def _oracle_env(scene):
    w = scene.world
    return pyoracle.OracleEnv.from_world(w, scene.envmap_tables() if w.ambient == AMBIENT_ENVMAP else None)


def _oracle_image(cb, scene, st, spp):
    lt = scene.light_table()
    return pyoracle.pt_render(cb.mesh.triangle_soup(), cb.material_of_triangle, cb.albedo, cb.emission,
                              lt["emissive"], lt["probas"], lt["alias"], lt["power_sum"], st, spp,
                              env=_oracle_env(scene))


# ---- tables --------------------------------------------------------------------------------------
@pytest.mark.parametrize("hw", [(32, 64), (19, 37), (1, 1), (512, 1024)])
def test_envmap_tables_match_oracle_build(cuda, hw):
    h, w = hw
    img = scenes.sky_envmap(w, h, seed=7) if h > 1 else np.array([[[0.5, 1.0, 2.0]]], np.float32)
    _, scene = _cornell(World(ambient=AMBIENT_ENVMAP, envmap=img))
    got = scene.envmap_tables()
    want = pyoracle.env_tables(img, total_sum64=got["total_sum64"])
    np.testing.assert_array_equal(got["texels"], want["texels"])
    # FP64 running sums differ from the oracle's sequential ones in association only: <= 1 ulp
    np.testing.assert_array_max_ulp(got["cdf"], want["cdf"], maxulp=1)
    assert abs(got["total_sum64"] - want["total_sum64"]) <= 1e-12 * want["total_sum64"]
    np.testing.assert_array_equal(got["probas"], want["probas"])
    np.testing.assert_array_equal(got["alias"], want["alias"])
    assert got["total_sum"] == np.float32(got["total_sum64"])


# ---- images against the oracle, sample by sample ---------------------------------------------------
WORLDS = {
    "alias": dict(),
    "cdf": dict(sampling=ENVMAP_BINARY_SEARCH),
    "no_sampling": dict(sampling=ENVMAP_NO_SAMPLING),
    "no_bsdf_mis": dict(bsdf_mis=False),
    "bilinear_rotated": dict(bilinear=True, rotation=ROT),
    "intensity_scaled_background": dict(intensity=2.5, scale_background=True),
    "intensity_unscaled_background": dict(intensity=0.4),
}


@pytest.mark.parametrize("name", sorted(WORLDS))
def test_envmap_cornell_matches_oracle_sample_by_sample(cuda, name):
    cb, scene = _cornell(World(ambient=AMBIENT_ENVMAP, envmap=scenes.sky_envmap(64, 32, seed=2), **WORLDS[name]))
    st = _settings(6)
    gpu = _render(scene, st)
    orc = _oracle_image(cb, scene, st, 6)
    assert _close(gpu, orc) > 0.97
    assert abs(gpu.mean() - orc.mean()) / orc.mean() < 2e-3
    assert np.isfinite(gpu).all()


@pytest.mark.parametrize("m,n", [(4, 1), (2, 0)])
def test_envmap_with_ris_direct_lighting_matches_oracle(cuda, m, n):
    cb, scene = _cornell(World(ambient=AMBIENT_ENVMAP, envmap=scenes.sky_envmap(64, 32, seed=2)))
    st = _settings(6, direct_lighting=DIRECT_RIS, ris_light_candidates=m, ris_bsdf_candidates=n)
    gpu = _render(scene, st)
    orc = _oracle_image(cb, scene, st, 6)
    assert _close(gpu, orc) > 0.97
    assert abs(gpu.mean() - orc.mean()) / orc.mean() < 2e-3


def test_uniform_ambient_matches_oracle(cuda):
    cb, scene = _cornell(World(ambient=AMBIENT_UNIFORM, uniform_color=(0.3, 0.5, 0.8)))
    st = _settings(6)
    gpu = _render(scene, st)
    orc = _oracle_image(cb, scene, st, 6)
    assert _close(gpu, orc) > 0.97
    # the frame around the box sees the uniform colour itself
    assert np.allclose(gpu[0, 0] / 6, (0.3, 0.5, 0.8), rtol=1e-6)


@pytest.mark.parametrize("kind", ["mis", "ris"])
def test_envmap_principled_matches_reference_bsdf_golden(cuda, kind):
    g = np.load(GOLDEN + "pt_principled_cornell.npz")
    e = np.load(GOLDEN + "pt_principled_env_cornell.npz")
    w, h, spp, nb, rr, seed = (int(v) for v in g["settings"])
    scene = gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=g["materials"])
    scene.set_world(World(ambient=AMBIENT_ENVMAP, envmap=e["sky"], intensity=float(e["intensity"])))
    tb = scene.envmap_tables()
    for k in ("texels", "probas", "alias"):
        np.testing.assert_array_equal(tb[k], e[k])  # the golden image used these tables
    st = RenderSettings(width=w, height=h, samples_per_launch=spp, nb_bounces=nb, russian_roulette_min_depth=rr,
                        bsdf=BSDF_PRINCIPLED, seed=seed, inverse_view=g["inverse_view"],
                        inverse_projection=g["inverse_projection"])
    if kind == "ris":
        st.direct_lighting, st.ris_light_candidates, st.ris_bsdf_candidates = DIRECT_RIS, 4, 1
    gpu = _render(scene, st)
    want = e["image_" + kind]
    rel = np.abs(gpu - want) / np.maximum(np.abs(want), 1e-3)
    close = rel.max(axis=-1) < 1e-3
    # as for the principled scenes without a world: a path crossing a branch threshold (lobe
    # choice, refraction vs reflection, Russian roulette) on one side only diverges entirely
    assert close.mean() > 0.93, close.mean()
    assert abs(gpu[close].mean() - want[close].mean()) / want[close].mean() < 1e-4


# ---- estimator properties ----------------------------------------------------------------------------
def _launch_means(scene, st, launches):
    r = gbpt.Renderer(scene, st)
    prev = np.zeros((st.height, st.width, 3))
    means = []
    for _ in range(launches):
        r.render(1)
        torch.cuda.synchronize()
        cur = r.image_sums()[1]
        means.append((cur - prev).mean() / st.samples_per_launch)
        prev = cur
    return np.array(means)


@pytest.mark.parametrize("sampling", [ENVMAP_ALIAS_TABLE, ENVMAP_BINARY_SEARCH])
def test_sampled_envmap_agrees_with_miss_only_estimator_on_a_smooth_sky(cuda, sampling):
    """Without a sun the reference's texel-corner sampling is consistent: the importance-sampled
    image and the miss-only image (BSDF sampling alone) have the same mean within 3 sigma."""
    sky = scenes.sky_envmap(128, 64, seed=4, sun_radiance=(0.0, 0.0, 0.0))
    _, sampled = _cornell(World(ambient=AMBIENT_ENVMAP, envmap=sky, sampling=sampling))
    _, misses = _cornell(World(ambient=AMBIENT_ENVMAP, envmap=sky, sampling=ENVMAP_NO_SAMPLING))
    a = _launch_means(sampled, _settings(64, seed=11, w=32, h=32), 24)
    b = _launch_means(misses, _settings(64, seed=12, w=32, h=32), 24)
    sigma = np.hypot(a.std(ddof=1) / np.sqrt(len(a)), b.std(ddof=1) / np.sqrt(len(b)))
    assert abs(a.mean() - b.mean()) < 3 * sigma + 2e-3 * b.mean(), (a.mean(), b.mean(), sigma)
    # importance sampling is the less noisy of the two
    assert a.std() < b.std()


def test_zero_intensity_and_black_envmaps_add_nothing(cuda):
    cb = scenes.cornell_box()
    plain = gbpt.Scene.from_cornell(cb)
    st = _settings(4)
    base = _render(plain, st)
    _, zero = _cornell(World(ambient=AMBIENT_ENVMAP, envmap=scenes.sky_envmap(64, 32), intensity=0.0))
    np.testing.assert_array_equal(_render(zero, st), base)
    _, black = _cornell(World(ambient=AMBIENT_ENVMAP, envmap=np.zeros((16, 32, 3), np.float32)))
    assert black.envmap_tables()["total_sum64"] == 0.0
    np.testing.assert_array_equal(_render(black, st), base)


def test_world_changes_reach_existing_renderers(cuda):
    cb = scenes.cornell_box()
    scene = gbpt.Scene.from_cornell(cb)
    st = _settings(4)
    r = gbpt.Renderer(scene, st)
    r.render(1)
    scene.set_world(World(ambient=AMBIENT_ENVMAP, envmap=scenes.sky_envmap(64, 32, seed=2)))
    r.reset()
    r.render(1)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(r.image_sums()[1], _render(scene, st))
    scene.set_world(World())  # back to no world
    r.reset()
    r.render(1)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(r.image_sums()[1], _render(gbpt.Scene.from_cornell(cb), st))


def test_world_validation(cuda):
    _, scene = _cornell(World())
    bad_texel = scenes.sky_envmap(8, 4)
    bad_texel[1, 2, 0] = np.nan
    for w in (World(ambient=AMBIENT_ENVMAP, envmap=bad_texel),
              World(ambient=AMBIENT_ENVMAP, envmap=-scenes.sky_envmap(8, 4)),
              World(ambient=AMBIENT_ENVMAP, envmap=scenes.sky_envmap(8, 4), intensity=-1.0),
              World(ambient=AMBIENT_ENVMAP, envmap=scenes.sky_envmap(8, 4), sampling=7),
              World(ambient=AMBIENT_UNIFORM, uniform_color=(0.1, -0.1, 0.1)),
              World(ambient=5)):
        with pytest.raises(GbptError):
            scene.set_world(w)
    w = World(ambient=AMBIENT_ENVMAP, envmap=scenes.sky_envmap(8, 4))
    w.inverse_rotation = ROT  # not the inverse of the identity
    with pytest.raises(GbptError):
        scene.set_world(w)
    assert scene.world.ambient == AMBIENT_NONE  # failed calls leave the world as it was
    with pytest.raises(GbptError):
        scene.envmap_tables()  # no envmap in the scene's world


def test_batch_with_envmap_scene_equals_single_renders(cuda):
    cb = scenes.cornell_box()
    sky_scene = gbpt.Scene.from_cornell(cb)
    sky_scene.set_world(World(ambient=AMBIENT_ENVMAP, envmap=scenes.sky_envmap(64, 32, seed=2)))
    plain = gbpt.Scene.from_cornell(cb)
    jobs = [(sky_scene, _settings(6, seed=2, w=24, h=20)), (plain, _settings(5, seed=3, w=16, h=16))]
    b = gbpt.Batch(jobs, samples_per_iteration=2)
    b.render()
    torch.cuda.synchronize()
    for k, (scene, st) in enumerate(jobs):
        one = RenderSettings(**{**st.__dict__, "samples_per_launch": 1})
        r = gbpt.Renderer(scene, one)
        r.render(st.samples_per_launch)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(b.image_sums(k)[1], r.image_sums()[1])
    # the world of a scene a batch renders cannot change under it
    with pytest.raises(GbptError):
        sky_scene.set_world(World())
    b.destroy()
    sky_scene.set_world(World())
