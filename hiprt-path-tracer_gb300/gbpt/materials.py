"""Principled material records (gbpt_principled_material, include/gbpt_bsdf.h) as numpy arrays.

One material = 64 32-bit words (256 B). Field meanings and defaults follow the reference's
DeviceUnpackedEffectiveMaterial (src/HostDeviceCommon/Material/MaterialUnpacked.h). The word
offsets here must match the C struct; tests/test_bsdf.py checks them against the library.
"""
from __future__ import annotations

import numpy as np

WORDS = 64

# (name, word offset, component count)
FIELDS = [
    ("base_color", 0, 3), ("roughness", 3, 1),
    ("emission", 4, 3), ("metallic", 7, 1),
    ("metallic_F82", 8, 3), ("metallic_F90_falloff_exponent", 11, 1),
    ("metallic_F90", 12, 3), ("anisotropy", 15, 1),
    ("anisotropy_rotation", 16, 1), ("second_roughness_weight", 17, 1), ("second_roughness", 18, 1), ("specular", 19, 1),
    ("specular_color", 20, 3), ("specular_tint", 23, 1),
    ("specular_darkening", 24, 1), ("coat", 25, 1), ("coat_roughness", 26, 1), ("coat_roughening", 27, 1),
    ("coat_medium_absorption", 28, 3), ("coat_medium_thickness", 31, 1),
    ("coat_darkening", 32, 1), ("coat_anisotropy", 33, 1), ("coat_anisotropy_rotation", 34, 1), ("coat_ior", 35, 1),
    ("sheen", 36, 1), ("ior", 37, 1), ("specular_transmission", 38, 1), ("diffuse_transmission", 39, 1),
    ("absorption_color", 40, 3), ("absorption_at_distance", 43, 1),
    ("thin_walled", 44, 1), ("diffuse_lobe", 45, 1), ("oren_nayar_sigma", 46, 1),
    ("thin_film", 47, 1), ("thin_film_ior", 48, 1), ("thin_film_thickness", 49, 1), ("thin_film_kappa_3", 50, 1),
    ("thin_film_hue_shift", 51, 1), ("thin_film_base_ior_override", 52, 1), ("thin_film_do_ior_override", 53, 1),
    ("dispersion_scale", 54, 1), ("dispersion_abbe_number", 55, 1),
]
INT_FIELDS = ("thin_walled", "diffuse_lobe", "thin_film_do_ior_override")
DIFFUSE_LAMBERTIAN, DIFFUSE_OREN_NAYAR = 0, 1  # GBPT_DIFFUSE_*
OFFSETS = {n: (o, c) for n, o, c in FIELDS}

DEFAULTS = {
    "base_color": (1.0, 1.0, 1.0), "roughness": 0.3, "emission": (0.0, 0.0, 0.0), "metallic": 0.0,
    "metallic_F82": (1.0, 1.0, 1.0), "metallic_F90_falloff_exponent": 5.0, "metallic_F90": (1.0, 1.0, 1.0),
    "anisotropy": 0.0, "anisotropy_rotation": 0.0, "second_roughness_weight": 0.0, "second_roughness": 0.5,
    "specular": 1.0, "specular_color": (1.0, 1.0, 1.0), "specular_tint": 1.0, "specular_darkening": 0.0,
    "coat": 0.0, "coat_roughness": 0.0, "coat_roughening": 1.0, "coat_medium_absorption": (1.0, 1.0, 1.0),
    "coat_medium_thickness": 5.0, "coat_darkening": 1.0, "coat_anisotropy": 0.0, "coat_anisotropy_rotation": 0.0,
    "coat_ior": 1.5, "sheen": 0.0, "ior": 1.4, "specular_transmission": 0.0, "diffuse_transmission": 0.0,
    "absorption_color": (1.0, 1.0, 1.0), "absorption_at_distance": 1.0, "thin_walled": 0,
    "diffuse_lobe": DIFFUSE_LAMBERTIAN, "oren_nayar_sigma": 0.34906585039886591538,  # 20 degrees
    "thin_film": 0.0, "thin_film_ior": 1.3, "thin_film_thickness": 500.0, "thin_film_kappa_3": 0.0,
    "thin_film_hue_shift": 0.0, "thin_film_base_ior_override": 1.0, "thin_film_do_ior_override": 0,
    "dispersion_scale": 0.0, "dispersion_abbe_number": 20.0,
}


def pack(**kw) -> np.ndarray:
    """One material record (float32[64]); unspecified fields take the reference's defaults."""
    rec = np.zeros(WORDS, np.float32)
    vals = dict(DEFAULTS)
    for k, v in kw.items():
        if k not in OFFSETS:
            raise KeyError(f"unknown material field {k!r}")
        vals[k] = v
    for name, (off, cnt) in OFFSETS.items():
        v = vals[name]
        if name in INT_FIELDS:
            rec[off:off + 1] = np.array([int(v)], np.int32).view(np.float32)
        else:
            rec[off:off + cnt] = np.broadcast_to(np.asarray(v, np.float32), (cnt,))
    return rec


def unpack(rec: np.ndarray) -> dict:
    """The fields of one material record as a dict (the inverse of pack)."""
    out = {}
    for name, (off, cnt) in OFFSETS.items():
        if name in INT_FIELDS:
            out[name] = int(rec[off:off + 1].view(np.int32)[0])
        elif cnt == 1:
            out[name] = float(rec[off])
        else:
            out[name] = tuple(float(v) for v in rec[off:off + cnt])
    return out


def pack_many(dicts) -> np.ndarray:
    return np.stack([pack(**d) for d in dicts]) if dicts else np.zeros((0, WORDS), np.float32)


def get(rec: np.ndarray, name: str):
    off, cnt = OFFSETS[name]
    if name in INT_FIELDS:
        return int(rec[off:off + 1].view(np.int32)[0])
    return rec[off] if cnt == 1 else rec[off:off + cnt]


def random_principled(rng: np.random.Generator, n: int) -> list:
    """Materials with the parameter distribution of the large instanced scene: base U[0,1]^3,
    roughness U[0.05,1], metallic Bernoulli(0.3), coat U[0,1] with coat roughness U[0,0.3],
    IOR U[1.3,1.8], anisotropy U[0,0.8], specular transmission Bernoulli(0.1)."""
    out = []
    for _ in range(n):
        out.append(dict(
            base_color=tuple(rng.uniform(0, 1, 3)), roughness=float(rng.uniform(0.05, 1.0)),
            metallic=float(rng.random() < 0.3), coat=float(rng.uniform(0, 1)), coat_roughness=float(rng.uniform(0, 0.3)),
            ior=float(rng.uniform(1.3, 1.8)), anisotropy=float(rng.uniform(0, 0.8)),
            anisotropy_rotation=float(rng.uniform(0, 1)),
            specular_transmission=float(rng.random() < 0.1)))
    return out


def coat_roughened(m: dict) -> dict:
    """The reference's coat roughening of the base and second metal roughness
    (src/Device/includes/Material.h:122-146), applied once on the host: the BSDF then sees the
    effective roughnesses, as the reference's BSDF does after its material fetch."""
    m = dict(DEFAULTS, **m)
    coat, rough = float(m["coat"]), float(m["coat_roughening"])
    if coat > 0.0 and rough > 0.0:
        f = np.float32
        one = f(1.0)

        def lerp(a, b, t):
            return (one - t) * a + t * b

        cr = f(m["coat_roughness"])
        cr4 = (cr * cr) * (cr * cr)
        for key, cond in (("roughness", True), ("second_roughness", f(m["second_roughness_weight"]) > 0)):
            if not cond:
                continue
            base = f(m[key])
            b4 = (base * base) * (base * base)
            target = np.sqrt(np.sqrt(min(one, b4 + f(2.0) * cr4)))
            roughened = lerp(base, target, f(coat))
            m[key] = float(lerp(base, roughened, f(rough)))
    return m
