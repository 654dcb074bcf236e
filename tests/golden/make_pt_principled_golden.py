"""Generates tests/golden/pt_principled_cornell.npz: a Cornell box with principled materials
rendered by the path-tracing oracle (oracle/pt_oracle.cpp) shading with the REFERENCE's own
principled BSDF (oracle/_ref/libref.so; energy compensation and regularization compiled out).

The GPU path tracer draws the same random numbers (PCG per path, one PCG draw seeding the
Xorshift32 generator of each BSDF sample), so its image agrees with this one sample by sample up
to floating-point contraction. Materials: coated diffuse walls, a rough dielectric red wall, an
anisotropic metal green wall, a rough glass short box (closed: paths enter and leave it), a mirror
tall box (a delta BSDF: no light sampling), the area light. The scene and settings are stored with
the image so the GPU test needs nothing else. A third file renders the smooth-shading scene (two
coarse spheres shaded with their vertex normals); a fourth, pt_principled_oren_nayar_cornell.npz,
the Cornell scene with the Oren-Nayar diffuse lobe, shaded by the reference's BSDF built with that
lobe (oracle/_ref/libref_bsdf_oren_nayar.so); a fifth, pt_principled_thin_film_cornell.npz, the
Cornell scene with thin films on the walls, the metal, the glass box and the mirror (reference BSDF).
Usage (where the reference tree is present):  python tests/golden/make_pt_principled_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "hiprt-path-tracer_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from gbpt import materials as M, scenes  # noqa: E402
from gbpt.render import LIGHT_UNIFORM, BSDF_PRINCIPLED, RenderSettings, look_at_camera  # noqa: E402
import pyoracle  # noqa: E402

OUT = os.path.join(HERE, "pt_principled_cornell.npz")
OUT_RIS = os.path.join(HERE, "pt_principled_ris_cornell.npz")
OUT_SMOOTH = os.path.join(HERE, "pt_principled_smooth_cornell.npz")
OUT_ON = os.path.join(HERE, "pt_principled_oren_nayar_cornell.npz")
OUT_TF = os.path.join(HERE, "pt_principled_thin_film_cornell.npz")


MATERIALS = [
    dict(base_color=(0.73, 0.73, 0.73), roughness=0.5, coat=0.5, coat_roughness=0.1),          # 0 white walls
    dict(base_color=(0.63, 0.065, 0.05), roughness=0.4),                                        # 1 red wall
    dict(base_color=(0.14, 0.45, 0.09), roughness=0.35, metallic=1.0, anisotropy=0.6),           # 2 green wall
    dict(base_color=(0.0, 0.0, 0.0), emission=(17.0, 12.0, 4.0)),                               # 3 light
    dict(base_color=(0.95, 0.95, 0.95), roughness=0.15, specular_transmission=1.0, ior=1.5),    # 4 short box
    dict(base_color=(0.9, 0.9, 0.9), roughness=0.0, metallic=1.0),                              # 5 tall box
]

# the smooth-shading scene (gbpt.scenes.smooth_cornell): walls and light as above, a rough glass
# sphere and a glossy metal sphere, both shaded with their vertex normals
SMOOTH_MATERIALS = MATERIALS[:4] + [
    dict(base_color=(0.9, 0.6, 0.3), roughness=0.25, metallic=1.0),                             # 4 metal sphere
    dict(base_color=(0.95, 0.95, 0.95), roughness=0.1, specular_transmission=1.0, ior=1.5),     # 5 glass sphere
]


def scene():
    cb = scenes.cornell_box()
    mat_of = cb.material_of_triangle.copy()
    mat_of[10:22] = 4
    mat_of[22:34] = 5
    raw = M.pack_many(MATERIALS)
    eff = M.pack_many([M.coat_roughened(m) for m in MATERIALS])
    return cb.mesh, mat_of, raw, eff


def settings(width=32, height=32, spp=8):
    iv, ip = look_at_camera((2.75, 2.75, -8.0), (2.75, 2.75, 0.0), vfov_deg=40.0, aspect=width / height)
    return RenderSettings(width=width, height=height, samples_per_launch=spp, nb_bounces=4,
                          russian_roulette_min_depth=3, light_sampling=LIGHT_UNIFORM, bsdf=BSDF_PRINCIPLED, seed=3,
                          inverse_view=iv, inverse_projection=ip)


def main():
    pyoracle.build(ref=True)
    mesh, mat_of, raw, eff = scene()
    st = settings()
    emission = raw[:, 4:7]
    emissive = np.nonzero(np.any(emission[mat_of] != 0, axis=1))[0].astype(np.int32)
    img = pyoracle.pt_render_principled(mesh.triangle_soup(), mat_of, eff, emission, emissive, None, None, 0.0, st,
                                        st.samples_per_launch)
    np.savez_compressed(OUT, positions=mesh.positions, indices=mesh.indices, material_of=mat_of, materials=raw,
                        effective_materials=eff, inverse_view=st.inverse_view, inverse_projection=st.inverse_projection,
                        settings=np.array([st.width, st.height, st.samples_per_launch, st.nb_bounces,
                                           st.russian_roulette_min_depth, st.seed], np.int32), image=img)
    print(f"wrote {OUT}: mean {img.mean() / st.samples_per_launch:.4f}, nonzero {np.mean(img.sum(-1) > 0):.3f}")
    # the same scene with RIS direct lighting (4 light + 1 BSDF candidates), the reference's
    # default strategy
    st.direct_lighting, st.ris_light_candidates, st.ris_bsdf_candidates = 1, 4, 1
    ris = pyoracle.pt_render_principled(mesh.triangle_soup(), mat_of, eff, emission, emissive, None, None, 0.0, st,
                                        st.samples_per_launch)
    np.savez_compressed(OUT_RIS, image=ris, ris=np.array([4, 1], np.int32))
    print(f"wrote {OUT_RIS}: mean {ris.mean() / st.samples_per_launch:.4f}")
    # smooth shading: vertex normals on the spheres
    sc = scenes.smooth_cornell()
    mat_of = sc.material_of_triangle.copy()
    n_walls = 12
    n_s1 = int(np.sum(mat_of[n_walls:] == 0))
    mat_of[n_walls:n_walls + n_s1] = 5
    raw = M.pack_many(SMOOTH_MATERIALS)
    eff = M.pack_many([M.coat_roughened(m) for m in SMOOTH_MATERIALS])
    st = settings(spp=16)
    emission = raw[:, 4:7]
    emissive = np.nonzero(np.any(emission[mat_of] != 0, axis=1))[0].astype(np.int32)
    img = pyoracle.pt_render_principled(sc.mesh.triangle_soup(), mat_of, eff, emission, emissive, None, None, 0.0, st,
                                        st.samples_per_launch, normals=sc.corner_normals())
    np.savez_compressed(OUT_SMOOTH, positions=sc.mesh.positions, indices=sc.mesh.indices, material_of=mat_of,
                        materials=raw, vertex_normals=sc.vertex_normals, inverse_view=st.inverse_view,
                        inverse_projection=st.inverse_projection,
                        settings=np.array([st.width, st.height, st.samples_per_launch, st.nb_bounces,
                                           st.russian_roulette_min_depth, st.seed], np.int32), image=img)
    print(f"wrote {OUT_SMOOTH}: mean {img.mean() / st.samples_per_launch:.4f}")
    # the Cornell scene with the Oren-Nayar diffuse lobe on every material (rough facets on the
    # walls), shaded by the reference's BSDF built with PrincipledBSDFDiffuseLobe = Oren-Nayar
    mesh, mat_of, _, _ = scene()
    on = [dict(m, diffuse_lobe=M.DIFFUSE_OREN_NAYAR, oren_nayar_sigma=s)
          for m, s in zip(MATERIALS, (0.6, 1.0, 0.3, 0.0, 0.2, 0.4))]
    raw = M.pack_many(on)
    eff = M.pack_many([M.coat_roughened(m) for m in on])
    st = settings()
    emission = raw[:, 4:7]
    emissive = np.nonzero(np.any(emission[mat_of] != 0, axis=1))[0].astype(np.int32)
    img = pyoracle.pt_render_principled(mesh.triangle_soup(), mat_of, eff, emission, emissive, None, None, 0.0, st,
                                        st.samples_per_launch, bsdf="reference_oren_nayar")
    np.savez_compressed(OUT_ON, materials=raw, image=img)
    print(f"wrote {OUT_ON}: mean {img.mean() / st.samples_per_launch:.4f}")
    # the Cornell scene with thin films: iridescent coated walls, a filmed metal green wall, a
    # filmed rough glass box (base IOR override with extinction), a filmed mirror box
    films = (dict(thin_film=1.0, thin_film_ior=1.45, thin_film_thickness=420.0),
             dict(thin_film=0.7, thin_film_ior=1.8, thin_film_thickness=650.0, thin_film_hue_shift=0.25),
             dict(thin_film=1.0, thin_film_ior=1.33, thin_film_thickness=300.0),
             dict(),
             dict(thin_film=0.8, thin_film_ior=1.6, thin_film_thickness=900.0, thin_film_do_ior_override=1,
                  thin_film_base_ior_override=1.7, thin_film_kappa_3=0.5),
             dict(thin_film=1.0, thin_film_ior=1.25, thin_film_thickness=520.0))
    tf = [dict(m, **f) for m, f in zip(MATERIALS, films)]
    raw = M.pack_many(tf)
    eff = M.pack_many([M.coat_roughened(m) for m in tf])
    img = pyoracle.pt_render_principled(mesh.triangle_soup(), mat_of, eff, emission, emissive, None, None, 0.0, st,
                                        st.samples_per_launch)
    np.savez_compressed(OUT_TF, materials=raw, image=img)
    print(f"wrote {OUT_TF}: mean {img.mean() / st.samples_per_launch:.4f}")


if __name__ == "__main__":
    main()
