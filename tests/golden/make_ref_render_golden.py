"""Generates tests/golden/ref_render_cornell.npz: frames rendered by the REFERENCE's own CPU
render kernels — CameraRays + MegaKernel compiled from the reference's sources
(oracle/ref_render.cpp, built by `make -C oracle ref`) — which pin the GPU path tracer's
GBPT_RNG_REFERENCE mode sample by sample.

Six scenes, each rendered for FRAMES frames of one sample per pixel with the reference's
per-pass random numbers as its GPU renderer draws them: the renderer's Xorshift32, seeded with 42
(GPURenderer.cpp:750-751), gives one number to the G-buffer pass and one to the MegaKernel pass of
every sample (FillGBufferRenderPass.cpp:91, MegaKernelRenderPass.cpp:53):
  * lambert: the Cornell box (36 triangles, albedos 0.73 / red / green, light (17, 12, 4)),
    Lambertian BSDF override, uniform light sampling, 4 bounces, Russian roulette from bounce 3 —
    the configuration the path-tracing benchmark names (at 64 x 64 instead of 256 x 256);
  * principled: the Cornell box with coated, glossy, anisotropic metal and mirror materials
    (no transmissive object), power light sampling;
  * principled_glass: the same with a rough glass short box (nested-dielectric volume tracking);
  * principled_ris: the principled scene with direct lighting by RIS over 4 light and 1 BSDF
    candidates (LSS_RIS_BSDF_AND_LIGHT, the reference's default strategy, RIS.h:83-255);
  * principled_thin_film: the principled scene with thin films on the walls, the boxes and the
    mirror (the packed record's 8-bit film weight and hue, and its boolean base-IOR override);
  * principled_dispersion: the glass scene with a dispersive glass box.
Each frame image is the frame's sample (float32 H x W x 3); the scene arrays and settings are stored
with it, so the GPU test needs nothing else.
Usage (where the reference tree is present):  python tests/golden/make_ref_render_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "hiprt-path-tracer_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from gbpt import materials as M, scenes  # noqa: E402
from gbpt.render import LIGHT_POWER, LIGHT_UNIFORM, look_at_camera  # noqa: E402
import pyoracle  # noqa: E402

OUT = os.path.join(HERE, "ref_render_cornell.npz")
FRAMES = 4
SIZE = 64

OPAQUE = [
    dict(base_color=(0.73, 0.73, 0.73), roughness=0.5, coat=0.5, coat_roughness=0.1),       # 0 white walls
    dict(base_color=(0.63, 0.065, 0.05), roughness=0.4),                                     # 1 red wall
    dict(base_color=(0.14, 0.45, 0.09), roughness=0.35, metallic=1.0, anisotropy=0.6),        # 2 green wall
    dict(base_color=(0.0, 0.0, 0.0), emission=(17.0, 12.0, 4.0)),                            # 3 light
    dict(base_color=(0.8, 0.75, 0.7), roughness=0.25, metallic=0.5),                         # 4 short box
    dict(base_color=(0.9, 0.9, 0.9), roughness=0.0, metallic=1.0),                           # 5 tall box (mirror)
]
# thin films (ThinFilm.h) on the coated walls, the red dielectric wall, the metal wall, the half-metal
# box (with the base IOR override) and the mirror
FILMS = [
    dict(OPAQUE[0], thin_film=1.0, thin_film_ior=1.45, thin_film_thickness=420.0),
    dict(OPAQUE[1], thin_film=0.6, thin_film_ior=1.8, thin_film_thickness=650.0, thin_film_hue_shift=0.25),
    dict(OPAQUE[2], thin_film=1.0, thin_film_ior=1.33, thin_film_thickness=300.0),
    OPAQUE[3],
    dict(OPAQUE[4], thin_film=0.8, thin_film_ior=1.6, thin_film_thickness=900.0, thin_film_do_ior_override=1,
         thin_film_base_ior_override=1.7, thin_film_kappa_3=0.5),
    dict(OPAQUE[5], thin_film=1.0, thin_film_ior=1.25, thin_film_thickness=520.0),
]
GLASS = OPAQUE[:4] + [
    dict(base_color=(0.95, 0.95, 0.95), roughness=0.15, specular_transmission=1.0, ior=1.5),  # 4 glass box
    OPAQUE[5],
]
# the glass box dispersive (Dispersion.h): a wavelength per path drawn at its first hit on the box,
# the box's IORs taken at it, the path's colour filtered by it once
DISPERSIVE = GLASS[:4] + [dict(GLASS[4], dispersion_scale=1.0, dispersion_abbe_number=18.0), GLASS[5]]


def frame_random_numbers(n, seed=42):
    """(camera pass, MegaKernel pass) random numbers of each of the reference's first n frames."""
    x, out = seed, []
    for _ in range(n):
        cam = x = pyoracle.xorshift32(x)
        mk = x = pyoracle.xorshift32(x)
        out.append((cam, mk))
    return out


class Settings:
    def __init__(self, light):
        self.width = self.height = SIZE
        self.nb_bounces = 4
        self.do_russian_roulette = True
        self.russian_roulette_min_depth = 3
        self.russian_roulette_throughput_clamp = 0.0
        self.do_jittering = True
        self.light_sampling = light
        self.ris_light_candidates, self.ris_bsdf_candidates = 4, 1
        self.inverse_view, self.inverse_projection = look_at_camera((2.75, 2.75, -8.0), (2.75, 2.75, 0.0),
                                                                    vfov_deg=40.0, aspect=1.0)


def render(bsdf, light, mesh, mat_of, mats, st):
    r = pyoracle.RefRender(bsdf, light, mesh.positions, mesh.indices, mat_of, mats)
    frames = np.stack([r.render(st, k, rn) for k, rn in enumerate(frame_random_numbers(FRAMES))])
    return frames, r.light_table()


def main():
    pyoracle.build(ref=True)
    cb = scenes.cornell_box()
    out = dict(frames=np.int32(FRAMES), size=np.int32(SIZE), positions=cb.mesh.positions, indices=cb.mesh.indices,
               random_numbers=np.array(frame_random_numbers(FRAMES), np.uint32))
    st = Settings(LIGHT_UNIFORM)
    out["inverse_view"], out["inverse_projection"] = st.inverse_view, st.inverse_projection
    lam = np.stack([M.pack(base_color=tuple(cb.albedo[i]), emission=tuple(cb.emission[i])) for i in range(4)])
    img, _ = render("lambert", "uniform", cb.mesh, cb.material_of_triangle, lam, st)
    out.update(lambert_materials=lam, lambert_material_of=cb.material_of_triangle, lambert=img)
    print(f"lambert: mean {img.mean():.5f}")
    mat_of = cb.material_of_triangle.copy()
    mat_of[10:22] = 4
    mat_of[22:34] = 5
    for name, mats, light in (("principled", OPAQUE, "power"), ("principled_glass", GLASS, "power"),
                              ("principled_ris", OPAQUE, "power_ris"), ("principled_thin_film", FILMS, "power"),
                              ("principled_dispersion", DISPERSIVE, "power")):
        raw = M.pack_many(mats)
        img, lt = render("principled", light, cb.mesh, mat_of, raw, Settings(LIGHT_POWER))
        out.update({f"{name}_materials": raw, f"{name}_material_of": mat_of, name: img,
                    f"{name}_power_sum": np.float32(lt["power_sum"])})
        print(f"{name}: mean {img.mean():.5f}")
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes)")


if __name__ == "__main__":
    main()
