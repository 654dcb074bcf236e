"""Generates tests/golden/bsdf_principled.npz from the REFERENCE's own principled BSDF.

Runs oracle/_ref/libref.so (ref_bsdf.cpp: the reference's src/Device/includes/BSDFs/Principled.h
compiled behind clean-room shims by `make -C oracle ref`, energy compensation and microfacet
regularization compiled out) on seeded materials and directions, and stores inputs and outputs:
  eval:   material, view, normals, light direction -> rgb, pdf   [principled_bsdf_eval :1620]
  pdf:    same inputs -> pdf                                      [principled_bsdf_pdf :1717]
  sample: material, view, normals, Xorshift32 seed -> direction, rgb, pdf, sampled lobe,
          generator state after sampling                         [principled_bsdf_sample :1803]
With --thin-film, writes tests/golden/bsdf_thin_film.npz from the same library: every material of the
set carries a thin film (weight, film IOR, thickness, hue shift and, on a third of them, the base IOR
and extinction override, all seeded; ThinFilm.h). Sampling queries where the glass lobe picks
refraction at a totally reflecting interface (possible once the film's Fresnel term is blended in)
are left out: the reference's refraction returns a NaN direction there and its CPU sanity check
then takes the harness down. They are found beforehand with the library's BSDF built for the host
(tests/native), which returns f = 0, pdf = 0 for them.
With --dispersion, writes tests/golden/bsdf_dispersion.npz from the same library: every material
dispersive (scale and Abbe number seeded; Dispersion.h), each query with a wavelength in
[360, 830] nm as the path would carry it (stored as eval_w / sample_w).
With --oren-nayar, writes tests/golden/bsdf_oren_nayar.npz from oracle/_ref/libref_bsdf_oren_nayar.so
instead: the same BSDF compiled with the reference's Oren-Nayar diffuse lobe
(PrincipledBSDFDiffuseLobe = PRINCIPLED_DIFFUSE_LOBE_OREN_NAYAR, src/Device/includes/BSDFs/OrenNayar.h),
every material carrying diffuse_lobe = Oren-Nayar and a seeded facet-slope deviation sigma.
Usage (where the reference tree is present):  python tests/golden/make_bsdf_golden.py [--oren-nayar | --thin-film | --dispersion]
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "hiprt-path-tracer_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from gbpt import materials as M  # noqa: E402
import pyoracle  # noqa: E402

OUT = os.path.join(HERE, "bsdf_principled.npz")
OUT_ON = os.path.join(HERE, "bsdf_oren_nayar.npz")
OUT_TF = os.path.join(HERE, "bsdf_thin_film.npz")
OUT_DISP = os.path.join(HERE, "bsdf_dispersion.npz")
REF_ON_SO = os.path.join(REPO, "oracle", "_ref", "libref_bsdf_oren_nayar.so")


def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def material_set(rng, oren_nayar=False, thin_film=False, dispersion=False):
    """Edge cases of every lobe first, then the random principled distribution. With oren_nayar,
    every material selects the Oren-Nayar diffuse lobe with sigma in [0, 1.2] rad (0 and the
    default 20 degrees among them)."""
    base = [
        dict(base_color=(0.8, 0.3, 0.2), roughness=0.5, specular=0.0),                     # diffuse only
        dict(base_color=(0.8, 0.3, 0.2), roughness=0.5),                                   # specular over diffuse
        dict(base_color=(0.9, 0.6, 0.3), roughness=0.25, metallic=1.0),                     # rough metal
        dict(base_color=(0.9, 0.6, 0.3), roughness=0.0, metallic=1.0),                      # delta metal
        dict(base_color=(0.9, 0.6, 0.3), roughness=0.4, metallic=1.0, anisotropy=0.7, anisotropy_rotation=0.3),
        dict(base_color=(0.7, 0.7, 0.9), roughness=0.3, metallic=1.0, metallic_F82=(0.6, 0.8, 0.9),
             metallic_F90=(1.0, 0.9, 0.8), metallic_F90_falloff_exponent=3.0, second_roughness_weight=0.4,
             second_roughness=0.7),
        dict(base_color=(0.9, 0.9, 0.9), roughness=0.2, specular_transmission=1.0, ior=1.5),  # rough glass
        dict(base_color=(0.9, 0.9, 0.9), roughness=0.0, specular_transmission=1.0, ior=1.5),  # smooth glass
        dict(base_color=(0.9, 0.8, 0.9), roughness=0.3, specular_transmission=1.0, ior=1.45, thin_walled=1),
        dict(base_color=(0.5, 0.6, 0.2), roughness=0.4, coat=1.0, coat_roughness=0.1, coat_ior=1.6),
        dict(base_color=(0.5, 0.6, 0.2), roughness=0.4, coat=0.6, coat_roughness=0.0,
             coat_medium_absorption=(0.8, 0.5, 0.3), coat_medium_thickness=2.0),
        dict(base_color=(0.3, 0.6, 0.8), roughness=0.5, diffuse_transmission=0.7),
        dict(base_color=(0.3, 0.6, 0.8), roughness=0.5, specular_darkening=1.0, specular_tint=0.5,
             specular_color=(1.0, 0.5, 0.2)),
        dict(base_color=(0.6, 0.6, 0.6), roughness=0.35, metallic=0.5, specular_transmission=0.5, coat=0.3,
             coat_roughness=0.2, diffuse_transmission=0.2),
    ]
    mats = base + M.random_principled(rng, 50)
    if oren_nayar:
        sig = rng.uniform(0.0, 1.2, len(mats))
        sig[0], sig[1] = 0.0, M.DEFAULTS["oren_nayar_sigma"]
        mats = [dict(m, diffuse_lobe=M.DIFFUSE_OREN_NAYAR, oren_nayar_sigma=float(s)) for m, s in zip(mats, sig)]
    if thin_film:
        n = len(mats)
        weight = rng.uniform(0.2, 1.0, n)
        weight[:4] = 1.0  # a full film on the first lobes' edge cases
        override = rng.random(n) < 1.0 / 3.0
        mats = [dict(m, thin_film=float(weight[i]), thin_film_ior=float(rng.uniform(1.1, 2.2)),
                     thin_film_thickness=float(rng.uniform(80.0, 1500.0)),
                     thin_film_hue_shift=float(rng.choice([0.0, rng.uniform(0.0, 1.0)])),
                     thin_film_do_ior_override=int(override[i]),
                     thin_film_base_ior_override=float(rng.uniform(1.0, 3.0)),
                     thin_film_kappa_3=float(rng.uniform(0.0, 3.0)))
                for i, m in enumerate(mats)]
    if dispersion:
        mats = [dict(m, dispersion_scale=float(rng.uniform(0.3, 1.0)), dispersion_abbe_number=float(rng.uniform(15.0, 60.0)))
                for m in mats]
    return M.pack_many([M.coat_roughened(m) for m in mats])


def queries(rng, mats, n, sample):
    """16 floats per query (oracle/ref_bsdf.cpp): view, shading normal, geometric normal,
    light direction, eta incident, eta outgoing, inside flag, incident light info."""
    n_mat = len(mats)
    mi = rng.integers(0, n_mat, n).astype(np.int32)
    ns = _unit(rng, n)
    # geometric normal: the shading normal, or a perturbed copy for a quarter of the queries
    ng = ns.copy()
    k = rng.random(n) < 0.25
    ng[k] = ns[k] + 0.2 * _unit(rng, int(k.sum()))
    ng /= np.linalg.norm(ng, axis=1, keepdims=True)
    v = _unit(rng, n)
    v = np.where((np.sum(v * ns, 1) < 0)[:, None], -v, v)  # view in the shading hemisphere
    # a few grazing and a few normal-incidence views
    g = rng.random(n) < 0.05
    v[g] = ns[g] * 0.02 + np.cross(ns[g], _unit(rng, int(g.sum())))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    l = _unit(rng, n)
    # light direction near the mirror direction for a third of the queries (specular peaks)
    r = rng.random(n) < 0.33
    mirror = 2 * np.sum(v * ns, 1, keepdims=True) * ns - v
    l[r] = mirror[r] + 0.15 * _unit(rng, int(r.sum()))
    l /= np.linalg.norm(l, axis=1, keepdims=True)
    ior = mats[mi, 37]
    transm = mats[mi, 38]
    thin = mats[mi, 44].view(np.int32)
    inside = (rng.random(n) < 0.3) & (transm > 0) & (thin == 0)
    eta_i = np.where(inside, ior, 1.0).astype(np.float32)
    eta_o = np.where(inside, 1.0, ior).astype(np.float32)
    q = np.zeros((n, 16), np.float32)
    q[:, 0:3], q[:, 3:6], q[:, 6:9], q[:, 9:12] = v, ns, ng, l
    q[:, 12], q[:, 13], q[:, 14], q[:, 15] = eta_i, eta_o, inside.astype(np.float32), 0.0
    return mi, q


def refraction_under_tir(mats, smi, sq, seeds, sw=None):
    """Sampling queries whose glass refraction meets total internal reflection (host build)."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from native import build_emu
    import bsdf_golden
    lib = ctypes.CDLL(build_emu.build())
    vp = ctypes.c_void_p
    lib.emu_bsdf_sample.argtypes = [vp, vp, vp, vp, ctypes.c_int64, ctypes.c_int, vp, vp, vp]
    q = bsdf_golden.queries(sq, sw)
    mi = np.ascontiguousarray(smi, np.int32)
    sd = np.ascontiguousarray(seeds, np.uint32)
    out = np.zeros((len(q), 8), np.float32)
    lobe = np.zeros(len(q), np.int32)
    st = np.zeros(len(q), np.uint32)
    lib.emu_bsdf_sample(mats.ctypes.data, mi.ctypes.data, q.ctypes.data, sd.ctypes.data, len(q), 0, out.ctypes.data,
                        lobe.ctypes.data, st.ctypes.data)
    return (lobe == 64) & (out[:, 6] == 0) & np.all(out[:, 0:3] == sq[:, 3:6], axis=1)


def main():
    oren_nayar = "--oren-nayar" in sys.argv[1:]
    thin_film = "--thin-film" in sys.argv[1:]
    dispersion = "--dispersion" in sys.argv[1:]
    pyoracle.build(ref=True)
    lib = ctypes.CDLL(REF_ON_SO if oren_nayar else pyoracle.REF_SO)
    fp = ctypes.POINTER(ctypes.c_float)
    ip = ctypes.POINTER(ctypes.c_int32)
    up = ctypes.POINTER(ctypes.c_uint32)
    lib.ref_principled_eval.argtypes = [fp, ip, fp, fp, ctypes.c_int64, fp]
    lib.ref_principled_pdf.argtypes = [fp, ip, fp, fp, ctypes.c_int64, fp]
    lib.ref_principled_sample.argtypes = [fp, ip, fp, fp, up, ctypes.c_int64, fp, ip, up]

    rng = np.random.Generator(np.random.PCG64(20241 if oren_nayar else 20242 if thin_film else 20243 if dispersion
                                              else 20240))
    mats = np.ascontiguousarray(material_set(rng, oren_nayar, thin_film, dispersion))
    n_eval, n_sample = 8192, 8192
    emi, eq = queries(rng, mats, n_eval, sample=False)
    ew = rng.uniform(360.0, 830.0, n_eval).astype(np.float32) if dispersion else None
    eout = np.zeros((n_eval, 4), np.float32)
    pout = np.zeros(n_eval, np.float32)
    lib.ref_principled_eval(mats.ctypes.data_as(fp), emi.ctypes.data_as(ip), eq.ctypes.data_as(fp),
                            None if ew is None else ew.ctypes.data_as(fp), n_eval, eout.ctypes.data_as(fp))
    lib.ref_principled_pdf(mats.ctypes.data_as(fp), emi.ctypes.data_as(ip), eq.ctypes.data_as(fp),
                           None if ew is None else ew.ctypes.data_as(fp), n_eval, pout.ctypes.data_as(fp))
    smi, sq = queries(rng, mats, n_sample, sample=True)
    seeds = rng.integers(1, 2**32 - 1, n_sample, dtype=np.uint64).astype(np.uint32)
    sw = rng.uniform(360.0, 830.0, n_sample).astype(np.float32) if dispersion else None
    if thin_film or dispersion:
        keep = ~refraction_under_tir(mats, smi, sq, seeds, sw)
        smi, sq, seeds = np.ascontiguousarray(smi[keep]), np.ascontiguousarray(sq[keep]), np.ascontiguousarray(seeds[keep])
        if sw is not None:
            sw = np.ascontiguousarray(sw[keep])
        n_sample = len(smi)
    sout = np.zeros((n_sample, 8), np.float32)
    sinfo = np.zeros(n_sample, np.int32)
    srng = np.zeros(n_sample, np.uint32)
    lib.ref_principled_sample(mats.ctypes.data_as(fp), smi.ctypes.data_as(ip), sq.ctypes.data_as(fp),
                              None if sw is None else sw.ctypes.data_as(fp), seeds.ctypes.data_as(up), n_sample,
                              sout.ctypes.data_as(fp), sinfo.ctypes.data_as(ip), srng.ctypes.data_as(up))
    out_path = OUT_ON if oren_nayar else OUT_TF if thin_film else OUT_DISP if dispersion else OUT
    extra = dict(eval_w=ew, sample_w=sw) if dispersion else {}
    np.savez_compressed(out_path, materials=mats, eval_mat=emi, eval_q=eq, eval_out=eout, pdf_out=pout,
                        sample_mat=smi, sample_q=sq, seeds=seeds, sample_out=sout, sample_info=sinfo, sample_rng=srng,
                        **extra)
    print(f"wrote {out_path}: {len(mats)} materials, {n_eval} eval/pdf + {n_sample} sample queries; "
          f"nonzero eval {np.mean(eout[:, 3] > 0):.2f}, sampled lobes {np.unique(sinfo, return_counts=True)}")


if __name__ == "__main__":
    main()
