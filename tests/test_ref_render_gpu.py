"""GPU: the wavefront path tracer in GBPT_RNG_REFERENCE mode against frames rendered by the
REFERENCE's own CPU kernels (CameraRays + MegaKernel compiled from the reference's sources,
tests/golden/ref_render_cornell.npz, made by tests/golden/make_ref_render_golden.py).

In that mode every path draws the reference's random numbers in the reference's order (Xorshift32
seeded by wang_hash((pixel + 1)(sample + 1) random_number) with one random_number per pass as the
reference's GPU renderer draws them, BSDF samples continuing the path's generator), the camera hit
is shaded from the reference's packed G-buffer, and the scene stores the reference's 8-bit packed
materials, so the GPU reproduces each of the reference's frames pixel by pixel. The tolerance is 1e-3 relative per
pixel: the GPU contracts multiply-adds (and uses its own sqrt/sin/cos), so a path that crosses a
branch threshold (a lobe choice, Russian roulette, a grazing hit) on one side only diverges; the
test requires 97% of the pixels of every frame to agree."""
import os

import numpy as np
import pytest
import torch

import gbpt
from gbpt.render import (BSDF_LAMBERTIAN, BSDF_PRINCIPLED, DIRECT_RIS, LIGHT_POWER, LIGHT_UNIFORM,
                         MATERIALS_PACKED, RNG_REFERENCE, RenderSettings)

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_render_cornell.npz")


def _settings(g, bsdf, light):
    n = int(g["size"])
    return RenderSettings(width=n, height=n, samples_per_launch=1, nb_bounces=4, russian_roulette_min_depth=3,
                          russian_roulette_throughput_clamp=0.0, light_sampling=light, bsdf=bsdf,
                          inverse_view=g["inverse_view"], inverse_projection=g["inverse_projection"],
                          rng_mode=RNG_REFERENCE, random_number=0)


def _frames(scene, st, n):
    """n launches of one sample per pixel; returns each launch's sample (H, W, 3)."""
    r = gbpt.Renderer(scene, st)
    out, prev = [], 0.0
    for _ in range(n):
        r.render(1)
        torch.cuda.synchronize()
        s = r.image_sums()[1]
        out.append(s - prev)
        prev = s
    return np.stack(out)


def _agreement(gpu, ref):
    rel = np.abs(gpu - ref) / np.maximum(np.abs(ref), 1e-3)
    return (rel.max(axis=-1) < 1e-3).mean(axis=(1, 2))


def test_lambert_cornell_matches_reference_megakernel(cuda):
    """The path-tracing benchmark's Cornell box (Lambertian, uniform light sampling, 4 bounces,
    Russian roulette from bounce 3) frame by frame against the reference's MegaKernel."""
    g = np.load(GOLDEN)
    mats = g["lambert_materials"]
    scene = gbpt.Scene(g["positions"], g["indices"], g["lambert_material_of"], mats[:, 0:3], mats[:, 4:7],
                       material_packing=MATERIALS_PACKED)
    gpu = _frames(scene, _settings(g, BSDF_LAMBERTIAN, LIGHT_UNIFORM), int(g["frames"]))
    ref = g["lambert"]
    frac = _agreement(gpu, ref)
    assert frac.min() >= 0.97, frac
    assert abs(gpu.mean() - ref.mean()) <= 2e-3 * ref.mean(), (gpu.mean(), ref.mean())


@pytest.mark.parametrize("name", ["principled", "principled_glass", "principled_ris", "principled_thin_film",
                                  "principled_dispersion"])
def test_principled_cornell_matches_reference_megakernel(cuda, name):
    """Coated, glossy dielectric, anisotropic metal, metallic-blend and mirror materials (and a
    rough glass box entered and left through the nested-dielectric volume stack), power light
    sampling, against the reference's MegaKernel with its own principled BSDF; principled_ris
    with RIS direct lighting over 4 light and 1 BSDF candidates (LSS_RIS_BSDF_AND_LIGHT);
    principled_thin_film with thin films on five materials; principled_dispersion with a dispersive
    glass box (a wavelength drawn per path at its first hit on the box, in the reference's order)."""
    g = np.load(GOLDEN)
    scene = gbpt.Scene(g["positions"], g["indices"], g[f"{name}_material_of"], principled=g[f"{name}_materials"],
                       material_packing=MATERIALS_PACKED)
    lt = scene.light_table()
    assert abs(lt["power_sum"] - float(g[f"{name}_power_sum"])) <= 1e-6 * lt["power_sum"]
    st = _settings(g, BSDF_PRINCIPLED, LIGHT_POWER)
    if name.endswith("_ris"):
        st = RenderSettings(**{**st.__dict__, "direct_lighting": DIRECT_RIS, "ris_light_candidates": 4,
                               "ris_bsdf_candidates": 1})
    gpu = _frames(scene, st, int(g["frames"]))
    ref = g[name]
    frac = _agreement(gpu, ref)
    assert frac.min() >= 0.97, frac
    assert abs(gpu.mean() - ref.mean()) <= 5e-3 * ref.mean(), (gpu.mean(), ref.mean())


def test_reference_rng_frames_differ_from_pcg_and_repeat_after_reset(cuda):
    """The mode changes the random numbers, not the estimator: a PCG render of the same scene has
    the same mean within noise but other pixels; a reset renderer repeats its frames exactly."""
    g = np.load(GOLDEN)
    mats = g["lambert_materials"]
    scene = gbpt.Scene(g["positions"], g["indices"], g["lambert_material_of"], mats[:, 0:3], mats[:, 4:7],
                       material_packing=MATERIALS_PACKED)
    st = _settings(g, BSDF_LAMBERTIAN, LIGHT_UNIFORM)
    a = _frames(scene, st, 2)
    r = gbpt.Renderer(scene, st)
    r.render(1)
    r.reset()
    r.render(1)
    torch.cuda.synchronize()
    assert np.array_equal(r.image_sums()[1], a[0])
    pcg = _frames(scene, RenderSettings(**{**st.__dict__, "rng_mode": 0}), 2)
    assert not np.array_equal(pcg, a)
