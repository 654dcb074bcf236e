"""GPU: RIS direct lighting (the reference's default LSS_RIS_BSDF_AND_LIGHT, src/Device/includes/RIS/
RIS.h) in the wavefront against the oracle's restatement drawing the same random numbers (sample by
sample), for Lambertian and principled scenes, and its unbiasedness against plain MIS."""
import os

import numpy as np
import pytest
import torch

import gbpt
import pyoracle
from gbpt import scenes
from gbpt.render import BSDF_PRINCIPLED, DIRECT_RIS, LIGHT_POWER, LIGHT_UNIFORM, RenderSettings

pytestmark = pytest.mark.gpu

GOLDEN = os.path.dirname(os.path.abspath(__file__)) + "/golden/"


def _render(scene, st, launches=1):
    r = gbpt.Renderer(scene, st)
    r.render(launches)
    torch.cuda.synchronize()
    return r.image_sums()[1]


def _close(gpu, orc):
    rel = np.abs(gpu - orc) / np.maximum(np.abs(orc), 1e-3)
    close = rel.max(axis=-1) < 1e-3
    return float(close.mean()), close


def _emitter_scene(n_emit=64, seed=3):
    rng = np.random.Generator(np.random.PCG64(seed))
    hf = scenes.heightfield(cells=24, amplitude=0.2, seed=seed)
    em = scenes.random_triangles(n_emit, seed=seed + 1, lo=(-0.8, 0.35, -0.8), hi=(0.8, 0.9, 0.8), sigma=0.05)
    mesh = scenes.merge(hf, em)
    mat_of = np.concatenate([np.zeros(hf.n_triangles, np.int32), 1 + np.arange(n_emit, dtype=np.int32)])
    albedo = np.concatenate([[[0.6, 0.5, 0.4]], np.full((n_emit, 3), 0.5)]).astype(np.float32)
    rad = np.exp(rng.uniform(0, np.log(1000), n_emit))
    emission = np.concatenate([[[0, 0, 0]], rad[:, None] * rng.uniform(0.2, 1.0, (n_emit, 3))]).astype(np.float32)
    return mesh, mat_of, albedo, emission


def _emitter_settings(spp, seed, **kw):
    iv, ip = gbpt.look_at_camera((0.0, 1.5, -2.2), (0.0, 0.2, 0.0), vfov_deg=50.0)
    return RenderSettings(width=40, height=40, samples_per_launch=spp, nb_bounces=3, light_sampling=LIGHT_POWER,
                          seed=seed, inverse_view=iv, inverse_projection=ip, **kw)


@pytest.mark.parametrize("m,n", [(4, 1), (16, 1), (3, 0), (0, 1)])
def test_ris_cornell_matches_oracle_sample_by_sample(cuda, m, n):
    cb = scenes.cornell_box()
    scene = gbpt.Scene.from_cornell(cb)
    st = gbpt.cornell_settings(40, 40, samples_per_launch=6, direct_lighting=DIRECT_RIS, ris_light_candidates=m,
                               ris_bsdf_candidates=n)
    gpu = _render(scene, st)
    lt = scene.light_table()
    orc = pyoracle.pt_render(cb.mesh.triangle_soup(), cb.material_of_triangle, cb.albedo, cb.emission, lt["emissive"],
                             lt["probas"], lt["alias"], lt["power_sum"], st, 6)
    frac, _ = _close(gpu, orc)
    assert frac > 0.97, frac
    assert abs(gpu.mean() - orc.mean()) / orc.mean() < 2e-3


def test_ris_many_emitters_matches_oracle(cuda):
    mesh, mat_of, albedo, emission = _emitter_scene()
    scene = gbpt.Scene(mesh.positions, mesh.indices, mat_of, albedo, emission)
    st = _emitter_settings(4, 2, direct_lighting=DIRECT_RIS, ris_light_candidates=8)
    gpu = _render(scene, st)
    lt = scene.light_table()
    orc = pyoracle.pt_render(mesh.triangle_soup(), mat_of, albedo, emission, lt["emissive"], lt["probas"], lt["alias"],
                             lt["power_sum"], st, 4)
    frac, _ = _close(gpu, orc)
    assert frac > 0.97, frac


def test_ris_principled_cornell_matches_reference_bsdf_oracle(cuda):
    g = np.load(GOLDEN + "pt_principled_cornell.npz")
    ris = np.load(GOLDEN + "pt_principled_ris_cornell.npz")
    w, h, spp, nb, rr, seed = (int(v) for v in g["settings"])
    m, n = (int(v) for v in ris["ris"])
    st = RenderSettings(width=w, height=h, samples_per_launch=spp, nb_bounces=nb, russian_roulette_min_depth=rr,
                        light_sampling=LIGHT_UNIFORM, bsdf=BSDF_PRINCIPLED, seed=seed, inverse_view=g["inverse_view"],
                        inverse_projection=g["inverse_projection"], direct_lighting=DIRECT_RIS, ris_light_candidates=m,
                        ris_bsdf_candidates=n)
    scene = gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=g["materials"])
    gpu = _render(scene, st)
    frac, close = _close(gpu, ris["image"])
    # as for MIS, a path crossing a branch threshold on one side only diverges entirely
    assert frac > 0.93, frac
    assert abs(gpu[close].mean() - ris["image"][close].mean()) / ris["image"][close].mean() < 1e-4


def test_ris_is_unbiased_and_beats_mis_with_many_emitters(cuda):
    """Mean over 48 seeds of 4-spp RIS images agrees with a 16k-spp MIS FP64 image within 3 sigma,
    and at equal spp RIS has the lower relMSE on 64 emitters of radiance 1..1000."""
    mesh, mat_of, albedo, emission = _emitter_scene()
    scene = gbpt.Scene(mesh.positions, mesh.indices, mat_of, albedo, emission)
    ref = _render(scene, _emitter_settings(1024, 1000), launches=16) / 16384
    means = np.array([(_render(scene, _emitter_settings(4, 100 + k, direct_lighting=DIRECT_RIS, ris_light_candidates=8))
                       / 4).mean() for k in range(48)])
    sigma = means.std(ddof=1) / np.sqrt(len(means))
    assert abs(means.mean() - ref.mean()) < 3 * sigma + 1e-6, (means.mean(), ref.mean(), sigma)

    def relmse(img):
        return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))

    e_mis = np.mean([relmse(_render(scene, _emitter_settings(16, 200 + k)) / 16) for k in range(4)])
    e_ris = np.mean([relmse(_render(scene, _emitter_settings(16, 300 + k, direct_lighting=DIRECT_RIS,
                                                             ris_light_candidates=8)) / 16) for k in range(4)])
    assert e_ris < e_mis, (e_ris, e_mis)


def test_ris_settings_are_validated(cuda):
    from gbpt import GbptError
    cb = scenes.cornell_box()
    scene = gbpt.Scene.from_cornell(cb)
    for kw in (dict(ris_light_candidates=0, ris_bsdf_candidates=0), dict(ris_bsdf_candidates=2),
               dict(ris_light_candidates=65)):
        with pytest.raises(GbptError):
            gbpt.Renderer(scene, gbpt.cornell_settings(8, 8, direct_lighting=DIRECT_RIS, **kw))
