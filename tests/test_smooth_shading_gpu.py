"""GPU: smooth shading with vertex normals (get_shading_normal, src/Device/includes/Intersect.h:114-134,
followed by the backface fix). Lambertian: the GPU image against the live path-tracing oracle given
the same corner normals, sample by sample; principled: against the golden image of the oracle
shading with the reference's own BSDF; zero normals shade exactly like no normals; ReSTIR DI on
the smooth scene stays unbiased against NEE."""
import os

import numpy as np
import pytest
import torch

import gbpt
import pyoracle
from gbpt import render, scenes
from gbpt.render import BSDF_PRINCIPLED, LIGHT_POWER, RenderSettings

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pt_principled_smooth_cornell.npz")


def _image(scene, st, launches=1):
    r = gbpt.Renderer(scene, st)
    r.render(launches)
    torch.cuda.synchronize()
    return r.image_sums()[1]


def _compare(gpu, orc):
    rel = np.abs(gpu - orc) / np.maximum(np.abs(orc), 1e-3)
    frac_close = float((rel.max(axis=-1) < 1e-3).mean())
    mean_rel = abs(gpu.mean() - orc.mean()) / orc.mean()
    return frac_close, mean_rel


def test_smooth_lambertian_matches_oracle(cuda):
    sc = scenes.smooth_cornell()
    scene = gbpt.Scene(sc.mesh.positions, sc.mesh.indices, sc.material_of_triangle, sc.albedo, sc.emission,
                       vertex_normals=sc.vertex_normals)
    st = gbpt.cornell_settings(48, 48, samples_per_launch=8)
    gpu = _image(scene, st)
    lt = scene.light_table()
    orc = pyoracle.pt_render(sc.mesh.triangle_soup(), sc.material_of_triangle, sc.albedo, sc.emission, lt["emissive"],
                             lt["probas"], lt["alias"], lt["power_sum"], st, 8, normals=sc.corner_normals())
    frac_close, mean_rel = _compare(gpu, orc)
    assert frac_close > 0.97, frac_close
    assert mean_rel < 2e-3, mean_rel
    # the normals matter: the flat-shaded oracle image differs on the spheres
    flat = pyoracle.pt_render(sc.mesh.triangle_soup(), sc.material_of_triangle, sc.albedo, sc.emission, lt["emissive"],
                              lt["probas"], lt["alias"], lt["power_sum"], st, 8)
    assert _compare(gpu, flat)[0] < frac_close - 0.05


def test_zero_normals_shade_flat(cuda):
    sc = scenes.smooth_cornell()
    st = gbpt.cornell_settings(40, 40, samples_per_launch=4)
    args = (sc.mesh.positions, sc.mesh.indices, sc.material_of_triangle, sc.albedo, sc.emission)
    none = _image(gbpt.Scene(*args), st)
    zero = _image(gbpt.Scene(*args, vertex_normals=np.zeros_like(sc.vertex_normals)), st)
    np.testing.assert_array_equal(none.view(np.uint64), zero.view(np.uint64))
    with pytest.raises(gbpt.GbptError, match="normal"):
        bad = sc.vertex_normals.copy()
        bad[5, 1] = np.nan
        gbpt.Scene(*args, vertex_normals=bad)


def test_smooth_principled_matches_reference_bsdf_oracle(cuda):
    g = np.load(GOLDEN)
    w, h, spp, nb, rr, seed = (int(v) for v in g["settings"])
    st = RenderSettings(width=w, height=h, samples_per_launch=spp, nb_bounces=nb, russian_roulette_min_depth=rr,
                        light_sampling=render.LIGHT_UNIFORM, bsdf=BSDF_PRINCIPLED, seed=seed,
                        inverse_view=g["inverse_view"], inverse_projection=g["inverse_projection"])
    scene = gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=g["materials"],
                       vertex_normals=g["vertex_normals"])
    gpu = _image(scene, st)
    orc = g["image"]
    rel = np.abs(gpu - orc) / np.maximum(np.abs(orc), 1e-3)
    close = rel.max(axis=-1) < 1e-3
    # as the flat principled golden: paths that cross a branch threshold on one side only diverge
    # (the glass sphere refracts most camera paths), the rest agree to 1e-3
    assert close.mean() > 0.9, close.mean()
    mean_rel_close = abs(gpu[close].mean() - orc[close].mean()) / orc[close].mean()
    assert mean_rel_close < 1e-4, mean_rel_close


def test_restir_on_smooth_scene_unbiased_against_nee(cuda):
    g = np.load(GOLDEN)
    scene = gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=g["materials"],
                       vertex_normals=g["vertex_normals"])
    base = dict(width=32, height=32, nb_bounces=0, light_sampling=LIGHT_POWER, bsdf=BSDF_PRINCIPLED,
                inverse_view=g["inverse_view"], inverse_projection=g["inverse_projection"])
    ref = gbpt.Renderer(scene, RenderSettings(samples_per_launch=1024, seed=99, **base))
    ref.render(8)
    torch.cuda.synchronize()
    want = ref.image_sums()[1] / (1024 * 8)
    r = gbpt.Renderer(scene, RenderSettings(samples_per_launch=1, seed=7, **base))
    r.set_restir_di(render.restir_di_settings(light_candidates=8, bsdf_candidates=1, do_visibility_reuse=1,
                                              m_cap=20, use_confidence_weights=1, bias_correction_visibility=1,
                                              do_fused_spatiotemporal=1))
    frames, prev = [], np.zeros_like(want)
    for _ in range(256):
        r.render(1)
        cur = r.image_sums()[1]
        frames.append((cur - prev).mean())
        prev = cur
    frames = np.array(frames)
    batches = frames.reshape(16, 16).mean(axis=1)
    sigma = batches.std(ddof=1) / np.sqrt(len(batches))
    assert abs(frames.mean() - want.mean()) < 4 * sigma + 2e-3 * want.mean(), (frames.mean(), want.mean(), sigma)
