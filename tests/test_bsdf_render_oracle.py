"""CPU: the Oren-Nayar diffuse lobe and thin films at render level. The path-tracing oracle shading
with the library's principled BSDF built for the host (oracle/libhost_bsdf.so, from
csrc/principled.h) reproduces, sample by sample, the golden Cornell images the same oracle rendered
with the reference's BSDF: compiled with its Oren-Nayar lobe, and with thin films on the walls, the
metal, the glass box and the mirror (tests/golden/make_pt_principled_golden.py)."""
import os

import numpy as np

import pyoracle
from gbpt import materials as M, scenes
from gbpt.render import BSDF_PRINCIPLED, LIGHT_UNIFORM, RenderSettings

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "pt_principled_cornell.npz")
GOLDEN_ON = os.path.join(HERE, "golden", "pt_principled_oren_nayar_cornell.npz")
GOLDEN_TF = os.path.join(HERE, "golden", "pt_principled_thin_film_cornell.npz")


def _host_render(g, raw):
    eff = M.pack_many([M.coat_roughened(M.unpack(r)) for r in raw])
    w, h, spp, nb, rr, seed = (int(v) for v in g["settings"])
    st = RenderSettings(width=w, height=h, samples_per_launch=spp, nb_bounces=nb, russian_roulette_min_depth=rr,
                        light_sampling=LIGHT_UNIFORM, bsdf=BSDF_PRINCIPLED, seed=seed,
                        inverse_view=g["inverse_view"], inverse_projection=g["inverse_projection"])
    soup = scenes.Mesh(g["positions"], g["indices"]).triangle_soup()
    mat_of = g["material_of"]
    emission = raw[:, 4:7]
    emissive = np.nonzero(np.any(emission[mat_of] != 0, axis=1))[0].astype(np.int32)
    return pyoracle.pt_render_principled(soup, mat_of, eff, emission, emissive, None, None, 0.0, st, spp, bsdf="host")


def test_host_bsdf_thin_film_cornell_matches_reference():
    pyoracle.build(ref=False)
    g, tf = np.load(GOLDEN), np.load(GOLDEN_TF)
    assert (tf["materials"][:, 47] > 0).sum() == 5
    img = _host_render(g, tf["materials"])
    ref = tf["image"]
    rel = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
    frac = float((rel.max(axis=-1) < 1e-4).mean())
    assert frac > 0.97, frac
    assert abs(ref.mean() - g["image"].mean()) > 0.02 * g["image"].mean()


def test_host_bsdf_oren_nayar_cornell_matches_reference_lobe():
    pyoracle.build(ref=False)
    g, on = np.load(GOLDEN), np.load(GOLDEN_ON)
    raw = on["materials"]
    assert (raw[:, 45].view(np.int32) == M.DIFFUSE_OREN_NAYAR).all()
    eff = M.pack_many([M.coat_roughened(M.unpack(r)) for r in raw])
    w, h, spp, nb, rr, seed = (int(v) for v in g["settings"])
    st = RenderSettings(width=w, height=h, samples_per_launch=spp, nb_bounces=nb, russian_roulette_min_depth=rr,
                        light_sampling=LIGHT_UNIFORM, bsdf=BSDF_PRINCIPLED, seed=seed,
                        inverse_view=g["inverse_view"], inverse_projection=g["inverse_projection"])
    soup = scenes.Mesh(g["positions"], g["indices"]).triangle_soup()
    mat_of = g["material_of"]
    emission = raw[:, 4:7]
    emissive = np.nonzero(np.any(emission[mat_of] != 0, axis=1))[0].astype(np.int32)
    img = pyoracle.pt_render_principled(soup, mat_of, eff, emission, emissive, None, None, 0.0, st, spp, bsdf="host")
    ref = on["image"]
    rel = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
    frac = float((rel.max(axis=-1) < 1e-4).mean())
    assert frac > 0.97, frac
    # and the lobe shows: the Lambertian scene's image is not this one
    assert abs(ref.mean() - g["image"].mean()) > 0.02 * g["image"].mean()
