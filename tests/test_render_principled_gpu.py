"""GPU: the wavefront path tracer with the principled BSDF against the golden image of the
path-tracing oracle shading with the reference's own principled BSDF (same PCG stream, same
Xorshift32 seeds per BSDF sample, so paths agree sample by sample up to FMA contraction), and its
convergence/unbiasedness against an FP64-accumulated high-spp image."""
import os

import numpy as np
import pytest
import torch

import gbpt
from gbpt.render import BSDF_PRINCIPLED, LIGHT_UNIFORM, RenderSettings

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pt_principled_cornell.npz")
GOLDEN_ON = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pt_principled_oren_nayar_cornell.npz")
GOLDEN_TF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pt_principled_thin_film_cornell.npz")


def _load():
    g = np.load(GOLDEN)
    w, h, spp, nb, rr, seed = (int(v) for v in g["settings"])
    st = RenderSettings(width=w, height=h, samples_per_launch=spp, nb_bounces=nb, russian_roulette_min_depth=rr,
                        light_sampling=LIGHT_UNIFORM, bsdf=BSDF_PRINCIPLED, seed=seed,
                        inverse_view=g["inverse_view"], inverse_projection=g["inverse_projection"])
    scene = gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=g["materials"])
    return g, st, scene


def _render(scene, st, launches=1):
    r = gbpt.Renderer(scene, st)
    r.render(launches)
    torch.cuda.synchronize()
    return r.image_sums()[1]


def test_principled_cornell_matches_reference_bsdf_oracle(cuda):
    g, st, scene = _load()
    gpu = _render(scene, st)
    orc = g["image"]
    rel = np.abs(gpu - orc) / np.maximum(np.abs(orc), 1e-3)
    close = rel.max(axis=-1) < 1e-3
    frac_close = float(close.mean())
    # a pixel whose path crosses a branch threshold (lobe choice, refraction vs reflection, Russian
    # roulette) on one side only diverges completely: those are few (and may be fireflies through
    # the glass box and the mirror), the rest match to 1e-3
    assert frac_close > 0.93, frac_close
    mean_rel_close = abs(gpu[close].mean() - orc[close].mean()) / orc[close].mean()
    assert mean_rel_close < 1e-4, mean_rel_close


@pytest.mark.parametrize("golden", [GOLDEN_ON, GOLDEN_TF], ids=["oren_nayar", "thin_film"])
def test_lobe_variant_cornell_matches_reference(cuda, golden):
    """Every material on the Oren-Nayar diffuse lobe (per-material sigma), or thin films on the
    walls, the metal, the glass box and the mirror, against the oracle image shaded by the
    reference's BSDF (compiled with its Oren-Nayar lobe for the first)."""
    g, st, _ = _load()
    on = np.load(golden)
    scene = gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=on["materials"])
    gpu = _render(scene, st)
    orc = on["image"]
    rel = np.abs(gpu - orc) / np.maximum(np.abs(orc), 1e-3)
    close = rel.max(axis=-1) < 1e-3
    assert close.mean() > 0.93, close.mean()
    assert abs(gpu[close].mean() - orc[close].mean()) / orc[close].mean() < 1e-4


def test_principled_relmse_decreases_and_unbiased_over_seeds(cuda):
    g, st, scene = _load()
    ref_st = RenderSettings(**{**st.__dict__, "samples_per_launch": 512, "seed": 1000})
    ref = _render(scene, ref_st, launches=32) / (512 * 32)

    def relmse(img):
        return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))

    errs = []
    for spp in (16, 64, 256):
        s = RenderSettings(**{**st.__dict__, "samples_per_launch": spp, "seed": 7})
        errs.append(relmse(_render(scene, s) / spp))
    assert errs[0] > errs[1] > errs[2], errs
    means = []
    for seed in range(64):
        s = RenderSettings(**{**st.__dict__, "samples_per_launch": 32, "seed": seed + 1})
        means.append((_render(scene, s) / 32).mean())
    means = np.array(means)
    sigma = means.std(ddof=1) / np.sqrt(len(means))
    assert abs(means.mean() - ref.mean()) < 3 * sigma + 1e-6, (means.mean(), ref.mean(), sigma)


def test_principled_needs_principled_scene(cuda):
    g, st, _ = _load()
    plain = gbpt.Scene(g["positions"], g["indices"], g["material_of"], g["materials"][:, 0:3], g["materials"][:, 4:7])
    with pytest.raises(gbpt.GbptError):
        gbpt.Renderer(plain, st)
    bad = g["materials"].copy()
    bad[0, 36] = 0.5  # sheen
    with pytest.raises(gbpt.GbptError):
        gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=bad)
    bad = g["materials"].copy()
    bad[0, 45] = np.array([7], np.int32).view(np.float32)[0]  # no such diffuse lobe
    with pytest.raises(gbpt.GbptError, match="diffuse_lobe"):
        gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=bad)
