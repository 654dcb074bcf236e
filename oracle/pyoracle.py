"""TEST INFRASTRUCTURE ONLY — ctypes bindings for the CPU oracle libraries.

* ``liboracle.so``: this project's C++ restatement of the reference's CPU intersection path
  (trace_oracle.cpp). Built anywhere by ``make -C oracle``.
* ``_ref/libref.so``: the reference's own CPU code compiled behind clean-room shims
  (ref_trace.cpp). Built only where the reference tree is present (``make -C oracle ref``).
* ``_ref/libref_env.so`` / ``libref_env_bilinear.so``: the reference's own envmap packing, lookups
  and sampling (ref_envmap.cpp), nearest-texel and bilinear builds.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")
HOST_BSDF_SO = os.path.join(HERE, "libhost_bsdf.so")


def bsdf_callbacks(bsdf: str = "reference"):
    """(eval, sample) function pointers of the principled BSDF the oracles shade with: the
    reference's own (oracle/_ref/libref.so, every parity test) or, with bsdf="host", the library's
    BSDF compiled for the host (oracle/libhost_bsdf.so; CPU baselines where the reference tree is
    absent) or, with bsdf="reference_oren_nayar", the reference's BSDF compiled with its Oren-Nayar
    diffuse lobe (oracle/_ref/libref_bsdf_oren_nayar.so)."""
    if bsdf == "reference_oren_nayar":
        lib = ctypes.CDLL(os.path.join(HERE, "_ref", "libref_bsdf_oren_nayar.so"))
        return (ctypes.cast(lib.ref_principled_eval_one, ctypes.c_void_p).value,
                ctypes.cast(lib.ref_principled_sample_one, ctypes.c_void_p).value)
    if bsdf == "host":
        lib = ctypes.CDLL(HOST_BSDF_SO)
        return (ctypes.cast(lib.host_principled_eval_one, ctypes.c_void_p).value,
                ctypes.cast(lib.host_principled_sample_one, ctypes.c_void_p).value)
    ref = ctypes.CDLL(REF_SO)
    return (ctypes.cast(ref.ref_principled_eval_one, ctypes.c_void_p).value,
            ctypes.cast(ref.ref_principled_sample_one, ctypes.c_void_p).value)
REF_ENV_SO = os.path.join(HERE, "_ref", "libref_env.so")
REF_ENV_BILINEAR_SO = os.path.join(HERE, "_ref", "libref_env_bilinear.so")

_c_f = ctypes.POINTER(ctypes.c_float)
_c_i = ctypes.POINTER(ctypes.c_int32)
_c_u8 = ctypes.POINTER(ctypes.c_uint8)
_i64 = ctypes.c_int64


def reference_root() -> str | None:
    """The reference tree, from the GBPT_REFERENCE_ROOT environment variable (None when unset or
    not a reference tree). The only place the test infrastructure learns where it lies."""
    root = os.environ.get("GBPT_REFERENCE_ROOT")
    if root and os.path.isdir(os.path.join(root, "src", "Renderer")):
        return root
    return None


def build(ref: bool | None = None) -> None:
    """Compile the restatement (always) and the reference build (when the reference tree is given
    by GBPT_REFERENCE_ROOT; otherwise reference libraries built earlier in oracle/_ref stay)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    ref_root = reference_root()
    if ref is None:
        ref = ref_root is not None
    if ref:
        if ref_root is None:
            raise RuntimeError("the reference build needs GBPT_REFERENCE_ROOT to name the reference tree")
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={ref_root}"])


def _ptr(a: np.ndarray, t):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(t)


def _rays(rays):
    o = np.ascontiguousarray(rays.origin_tmin, np.float32)
    d = np.ascontiguousarray(rays.dir_tmax, np.float32)
    lp = np.ascontiguousarray(rays.last_prim, np.int32)
    return o, d, lp


class Oracle:
    """The restatement oracle (octree + k-DOP + Moller-Trumbore, reference semantics)."""

    def __init__(self):
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        lib = ctypes.CDLL(ORACLE_SO)
        lib.orc_octree_build.restype = ctypes.c_void_p
        lib.orc_octree_build.argtypes = [_c_f, _i64, ctypes.c_int, ctypes.c_int]
        lib.orc_octree_free.argtypes = [ctypes.c_void_p]
        lib.orc_octree_node_count.restype = _i64
        lib.orc_octree_node_count.argtypes = [ctypes.c_void_p]
        lib.orc_octree_closest.argtypes = [ctypes.c_void_p, _c_f, _c_f, _c_i, _i64, _c_f, ctypes.c_int]
        lib.orc_octree_occluded.argtypes = [ctypes.c_void_p, _c_f, _c_f, _c_i, _i64, _c_u8, ctypes.c_int]
        lib.orc_brute_closest.argtypes = [_c_f, _i64, _c_f, _c_f, _c_i, _i64, _c_f, ctypes.c_int]
        lib.orc_mt_intersect.restype = ctypes.c_int
        lib.orc_mt_intersect.argtypes = [_c_f, _c_f, _c_f, _c_f]
        self.lib = lib

    def octree(self, soup: np.ndarray, max_depth: int = 32, leaf_max: int = 8) -> "OracleOctree":
        return OracleOctree(self, soup, max_depth, leaf_max)

    def brute_closest(self, soup: np.ndarray, rays, nthreads: int = 0) -> np.ndarray:
        soup = np.ascontiguousarray(soup, np.float32)
        o, d, lp = _rays(rays)
        hits = np.zeros((len(o), 4), np.float32)
        self.lib.orc_brute_closest(_ptr(soup, _c_f), soup.shape[0], _ptr(o, _c_f), _ptr(d, _c_f), _ptr(lp, _c_i),
                                   len(o), _ptr(hits, _c_f), nthreads)
        return hits

    def mt(self, tri9: np.ndarray, origin3, dir3):
        tri9 = np.ascontiguousarray(tri9, np.float32).reshape(9)
        o = np.ascontiguousarray(origin3, np.float32).reshape(3)
        d = np.ascontiguousarray(dir3, np.float32).reshape(3)
        out = np.zeros(3, np.float32)
        ok = self.lib.orc_mt_intersect(_ptr(tri9, _c_f), _ptr(o, _c_f), _ptr(d, _c_f), _ptr(out, _c_f))
        return bool(ok), out


def set_scene_accel(octree: "OracleOctree | None") -> None:
    """Makes the path-tracing and ReSTIR oracles trace through this octree (built over the same
    triangles their next calls pass) instead of testing every triangle; None switches back. For
    CPU baselines on large scenes; parity tests keep the exhaustive test."""
    lib = Oracle().lib
    lib.orc_set_scene_accel.argtypes = [ctypes.c_void_p]
    lib.orc_set_scene_accel(octree.h if octree is not None else None)


class OracleOctree:
    def __init__(self, orc: Oracle, soup: np.ndarray, max_depth: int, leaf_max: int):
        self.orc = orc
        self.soup = np.ascontiguousarray(soup, np.float32)
        self.h = orc.lib.orc_octree_build(_ptr(self.soup, _c_f), self.soup.shape[0], max_depth, leaf_max)

    def __del__(self):
        if getattr(self, "h", None):
            self.orc.lib.orc_octree_free(self.h)
            self.h = None

    @property
    def node_count(self) -> int:
        return int(self.orc.lib.orc_octree_node_count(self.h))

    def closest(self, rays, nthreads: int = 0) -> np.ndarray:
        o, d, lp = _rays(rays)
        hits = np.zeros((len(o), 4), np.float32)
        self.orc.lib.orc_octree_closest(self.h, _ptr(o, _c_f), _ptr(d, _c_f), _ptr(lp, _c_i), len(o),
                                        _ptr(hits, _c_f), nthreads)
        return hits

    def occluded(self, rays, nthreads: int = 0) -> np.ndarray:
        o, d, lp = _rays(rays)
        occ = np.zeros(len(o), np.uint8)
        self.orc.lib.orc_octree_occluded(self.h, _ptr(o, _c_f), _ptr(d, _c_f), _ptr(lp, _c_i), len(o),
                                         _ptr(occ, _c_u8), nthreads)
        return occ


def ref_available() -> bool:
    return os.path.exists(REF_SO)


class RefBVH:
    """The reference's own CPU BVH (src/Renderer/BVH.*), compiled behind shims."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = ctypes.CDLL(REF_SO)
            lib.ref_bvh_build.restype = ctypes.c_void_p
            lib.ref_bvh_build.argtypes = [_c_f, _i64]
            lib.ref_bvh_free.argtypes = [ctypes.c_void_p]
            lib.ref_bvh_closest.argtypes = [ctypes.c_void_p, _c_f, _c_f, _c_i, _i64, _c_f]
            lib.ref_shadow_occluded.argtypes = [ctypes.c_void_p, _c_f, _c_f, _c_i, _c_f, _i64, _c_u8]
            cls._lib = lib
        return cls._lib

    def __init__(self, soup: np.ndarray):
        self.soup = np.ascontiguousarray(soup, np.float32)
        self.h = self.lib().ref_bvh_build(_ptr(self.soup, _c_f), self.soup.shape[0])

    def __del__(self):
        if getattr(self, "h", None):
            self.lib().ref_bvh_free(self.h)
            self.h = None

    def closest(self, rays) -> np.ndarray:
        o, d, lp = _rays(rays)
        hits = np.zeros((len(o), 4), np.float32)
        self.lib().ref_bvh_closest(self.h, _ptr(o, _c_f), _ptr(d, _c_f), _ptr(lp, _c_i), len(o), _ptr(hits, _c_f))
        return hits

    def shadow_occluded(self, rays, light_dist: np.ndarray) -> np.ndarray:
        o, d, lp = _rays(rays)
        ld = np.ascontiguousarray(light_dist, np.float32)
        occ = np.zeros(len(o), np.uint8)
        self.lib().ref_shadow_occluded(self.h, _ptr(o, _c_f), _ptr(d, _c_f), _ptr(lp, _c_i), _ptr(ld, _c_f), len(o),
                                       _ptr(occ, _c_u8))
        return occ


class OrcEnvC(ctypes.Structure):
    """OrcEnv of pt_oracle.cpp: the world around the scene."""
    _fields_ = [("ambient", ctypes.c_int32), ("uniform", ctypes.c_float * 3), ("texels", ctypes.c_void_p),
                ("cdf", ctypes.c_void_p), ("probas", ctypes.c_void_p), ("alias", ctypes.c_void_p),
                ("width", ctypes.c_int32), ("height", ctypes.c_int32), ("intensity", ctypes.c_float),
                ("total_sum", ctypes.c_float), ("to_world", ctypes.c_float * 9), ("to_env", ctypes.c_float * 9),
                ("sampling", ctypes.c_int32), ("bsdf_mis", ctypes.c_int32), ("bilinear", ctypes.c_int32),
                ("scale_background", ctypes.c_int32)]


class OracleEnv:
    """The world for the oracle. Envmap tables (texels, cdf, probas, alias: H x W) come from the
    library under test or from env_tables() below; rotation is the envmap-to-world matrix."""

    def __init__(self, ambient=2, uniform=(0.0, 0.0, 0.0), texels=None, cdf=None, probas=None, alias=None,
                 intensity=1.0, total_sum=0.0, rotation=None, inverse_rotation=None, sampling=2, bsdf_mis=True,
                 bilinear=False, scale_background=False):
        c = OrcEnvC()
        c.ambient = int(ambient)
        c.uniform[:] = [float(v) for v in uniform]
        self._keep = []
        if texels is not None:
            arrs = [np.ascontiguousarray(texels, np.uint32), np.ascontiguousarray(cdf, np.float32),
                    np.ascontiguousarray(probas, np.float32), np.ascontiguousarray(alias, np.int32)]
            self._keep = arrs
            c.texels, c.cdf, c.probas, c.alias = (a.ctypes.data for a in arrs)
            c.height, c.width = arrs[0].shape[:2]
        rot = np.eye(3, dtype=np.float32) if rotation is None else np.asarray(rotation, np.float32).reshape(3, 3)
        inv = (np.linalg.inv(rot.astype(np.float64)).astype(np.float32) if inverse_rotation is None
               else np.asarray(inverse_rotation, np.float32).reshape(3, 3))
        c.to_world[:] = [float(v) for v in rot.reshape(-1)]
        c.to_env[:] = [float(v) for v in inv.reshape(-1)]
        c.intensity = float(intensity)
        c.total_sum = float(total_sum)
        c.sampling = int(sampling) if total_sum > 0 else 0
        c.bsdf_mis = int(bool(bsdf_mis))
        c.bilinear = int(bool(bilinear))
        c.scale_background = int(bool(scale_background))
        self.c = c

    @classmethod
    def from_world(cls, world, tables=None):
        """From a gbpt World (duck-typed) and, for an envmap, the tables the library built."""
        if tables is None:
            return cls(ambient=world.ambient, uniform=world.uniform_color)
        return cls(ambient=world.ambient, uniform=world.uniform_color, texels=tables["texels"], cdf=tables["cdf"],
                   probas=tables["probas"], alias=tables["alias"], intensity=world.intensity,
                   total_sum=tables["total_sum"], rotation=world.rotation, inverse_rotation=world.inverse_rotation,
                   sampling=world.sampling, bsdf_mis=world.bsdf_mis, bilinear=world.bilinear,
                   scale_background=world.scale_background)

    def ref(self) -> "RefEnvC":
        r = RefEnvC()
        c = self.c
        r.texels, r.cdf, r.probas, r.alias = c.texels, c.cdf, c.probas, c.alias
        r.width, r.height, r.intensity, r.total_sum = c.width, c.height, c.intensity, c.total_sum
        r.to_world[:] = list(c.to_world)
        r.to_env[:] = list(c.to_env)
        return r


class RefEnvC(ctypes.Structure):
    """RefEnv of ref_envmap.cpp."""
    _fields_ = [("texels", ctypes.c_void_p), ("cdf", ctypes.c_void_p), ("probas", ctypes.c_void_p),
                ("alias", ctypes.c_void_p), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("intensity", ctypes.c_float), ("total_sum", ctypes.c_float), ("to_world", ctypes.c_float * 9),
                ("to_env", ctypes.c_float * 9)]


def _env_ptr(env):
    return ctypes.byref(env.c) if env is not None else None


def _pt_lib():
    orc = Oracle()
    lib = orc.lib
    if not getattr(lib, "_pt_sigs", False):
        lib.orc_pt_render.argtypes = [_c_f, ctypes.c_int, _c_i, _c_f, _c_f, _c_i, ctypes.c_int, _c_f, _c_i,
                                      ctypes.c_float, _c_i, ctypes.c_float, _c_f, _c_f,
                                      ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_void_p, _c_f]
        _u32 = ctypes.POINTER(ctypes.c_uint32)
        lib.orc_env_pack.argtypes = [_c_f, _i64, _u32, _c_f]
        lib.orc_env_unpack.argtypes = [_u32, _i64, _c_f]
        lib.orc_env_cdf.argtypes = [_c_f, _i64, _c_f, ctypes.POINTER(ctypes.c_double)]
        lib.orc_env_lookup.argtypes = [ctypes.c_void_p, _c_f, ctypes.c_int, _c_f]
        lib.orc_env_eval.argtypes = [ctypes.c_void_p, _c_f, ctypes.c_int, _c_f, _c_f]
        lib.orc_env_sample.argtypes = [ctypes.c_void_p, _c_i, _c_f, _c_f, ctypes.c_int, _c_f, _c_f, _c_f, _c_i]
        lib.orc_vose_alias.argtypes = [_c_f, ctypes.c_int, ctypes.c_double, _c_f, _c_i]
        lib.orc_emissive_power.argtypes = [_c_f, _c_i, _c_f, _c_i, ctypes.c_int, _c_f]
        lib._pt_sigs = True
    return lib


def _corner_normals(normals):
    """(T, 3, 3) corner normals of the triangle soup as a float pointer, or NULL."""
    if normals is None:
        return None, None
    n = np.ascontiguousarray(normals, np.float32).reshape(-1, 9)
    return n, _ptr(n, _c_f)


def pt_render(soup, material_of, albedo, emission, emissive, alias_prob, alias_idx, power_sum, settings, spp,
              iteration_base=0, nthreads=0, env: OracleEnv | None = None, normals=None):
    """Path-tracing oracle (Lambertian scenes). Returns the FP64 per-pixel sums (H, W, 3) of
    'spp' samples per pixel, drawn with the same PCG sequence as the GPU kernels. env: the world;
    normals: (T, 3, 3) smooth-shading corner normals (None: flat)."""
    lib = _pt_lib()
    keep, nptr = _corner_normals(normals)
    soup = np.ascontiguousarray(soup, np.float32)
    mo = np.ascontiguousarray(material_of, np.int32)
    al = np.ascontiguousarray(albedo, np.float32)
    em = np.ascontiguousarray(emission, np.float32)
    ei = np.ascontiguousarray(emissive, np.int32)
    ap = np.ascontiguousarray(alias_prob if alias_prob is not None else np.ones(len(ei)), np.float32)
    ai = np.ascontiguousarray(alias_idx if alias_idx is not None else np.arange(len(ei)), np.int32)
    s = settings
    si = np.array([s.width, s.height, s.nb_bounces, 1 if s.do_russian_roulette else 0, s.russian_roulette_min_depth,
                   s.light_sampling, s.seed, 1 if s.do_jittering else 0, spp, iteration_base,
                   getattr(s, "direct_lighting", 0), getattr(s, "ris_light_candidates", 4),
                   getattr(s, "ris_bsdf_candidates", 1), getattr(s, "rng_mode", 0),
                   int(getattr(s, "random_number", 0)) & 0xFFFFFFFF, getattr(s, "gbuffer_materials", 0),
                   int(getattr(s, "random_number_shade", 0)) & 0xFFFFFFFF],
                  np.uint32).view(np.int32)
    iv = np.ascontiguousarray(s.inverse_view, np.float32).reshape(16)
    ip = np.ascontiguousarray(s.inverse_projection, np.float32).reshape(16)
    out = np.zeros((s.height, s.width, 3), np.float64)
    lib.orc_pt_render(_ptr(soup, _c_f), soup.shape[0], _ptr(mo, _c_i), _ptr(al, _c_f), _ptr(em, _c_f), _ptr(ei, _c_i),
                      len(ei), _ptr(ap, _c_f), _ptr(ai, _c_i), float(power_sum), _ptr(si, _c_i),
                      float(s.russian_roulette_throughput_clamp), _ptr(iv, _c_f), _ptr(ip, _c_f),
                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nthreads, _env_ptr(env), nptr)
    del keep
    return out


def pt_render_principled(soup, material_of, pmats_effective, emission, emissive, alias_prob, alias_idx, power_sum,
                         settings, spp, iteration_base=0, nthreads=0, env: OracleEnv | None = None, normals=None,
                         bsdf: str = "reference"):
    """Path-tracing oracle for principled scenes: the estimator of pt_render with the BSDF
    evaluated and sampled by the REFERENCE's own principled BSDF (oracle/_ref/libref.so, built
    only where the reference tree exists). pmats_effective: (M, 64) records after coat
    roughening; normals: (T, 3, 3) smooth-shading corner normals (None: flat). Returns FP64
    per-pixel sums (H, W, 3)."""
    lib = _pt_lib()
    keep, nptr = _corner_normals(normals)
    if not getattr(lib, "_ptp_sig", False):
        lib.orc_pt_render_principled.argtypes = [_c_f, ctypes.c_int, _c_i, _c_f, _c_f, _c_f, ctypes.c_void_p,
                                                 ctypes.c_void_p, _c_i, ctypes.c_int, _c_f, _c_i, ctypes.c_float, _c_i,
                                                 ctypes.c_float, _c_f, _c_f, ctypes.POINTER(ctypes.c_double),
                                                 ctypes.c_int, ctypes.c_void_p, _c_f]
        lib._ptp_sig = True
    eval_fn, sample_fn = bsdf_callbacks(bsdf)
    soup = np.ascontiguousarray(soup, np.float32)
    mo = np.ascontiguousarray(material_of, np.int32)
    pm = np.ascontiguousarray(pmats_effective, np.float32)
    al = np.ascontiguousarray(pm[:, 0:3], np.float32)
    em = np.ascontiguousarray(emission, np.float32)
    ei = np.ascontiguousarray(emissive, np.int32)
    ap = np.ascontiguousarray(alias_prob if alias_prob is not None else np.ones(len(ei)), np.float32)
    ai = np.ascontiguousarray(alias_idx if alias_idx is not None else np.arange(len(ei)), np.int32)
    s = settings
    si = np.array([s.width, s.height, s.nb_bounces, 1 if s.do_russian_roulette else 0, s.russian_roulette_min_depth,
                   s.light_sampling, s.seed, 1 if s.do_jittering else 0, spp, iteration_base,
                   getattr(s, "direct_lighting", 0), getattr(s, "ris_light_candidates", 4),
                   getattr(s, "ris_bsdf_candidates", 1), getattr(s, "rng_mode", 0),
                   int(getattr(s, "random_number", 0)) & 0xFFFFFFFF, getattr(s, "gbuffer_materials", 0),
                   int(getattr(s, "random_number_shade", 0)) & 0xFFFFFFFF],
                  np.uint32).view(np.int32)
    iv = np.ascontiguousarray(s.inverse_view, np.float32).reshape(16)
    ip = np.ascontiguousarray(s.inverse_projection, np.float32).reshape(16)
    out = np.zeros((s.height, s.width, 3), np.float64)
    lib.orc_pt_render_principled(_ptr(soup, _c_f), soup.shape[0], _ptr(mo, _c_i), _ptr(al, _c_f), _ptr(em, _c_f),
                                 _ptr(pm, _c_f), eval_fn, sample_fn, _ptr(ei, _c_i), len(ei), _ptr(ap, _c_f),
                                 _ptr(ai, _c_i), float(power_sum), _ptr(si, _c_i),
                                 float(s.russian_roulette_throughput_clamp), _ptr(iv, _c_f), _ptr(ip, _c_f),
                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nthreads, _env_ptr(env), nptr)
    del keep
    return out


# ---- envmap: tables, lookups and sampling of the oracle, and the reference's own (pin) ----
def env_pack(rgb):
    """(H, W, 3) float texels -> RGB9E5 words (H, W) and float luminances (H, W)."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    h, w = rgb.shape[:2]
    tex = np.zeros((h, w), np.uint32)
    lum = np.zeros((h, w), np.float32)
    _pt_lib().orc_env_pack(_ptr(rgb, _c_f), h * w, tex.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), _ptr(lum, _c_f))
    return tex, lum


def env_unpack(texels):
    tex = np.ascontiguousarray(texels, np.uint32)
    out = np.zeros(tex.shape + (3,), np.float32)
    _pt_lib().orc_env_unpack(tex.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), tex.size, _ptr(out, _c_f))
    return out


def env_tables(rgb, total_sum64=None):
    """The oracle's envmap tables: texels, CDF (double running sum stored as float), alias table of
    the luminances normalised by total_sum64 (default: the oracle's own double sum)."""
    tex, lum = env_pack(rgb)
    cdf = np.zeros_like(lum)
    tot = ctypes.c_double()
    _pt_lib().orc_env_cdf(_ptr(lum, _c_f), lum.size, _ptr(cdf, _c_f), ctypes.byref(tot))
    s64 = tot.value if total_sum64 is None else float(total_sum64)
    prob, alias = vose_alias(lum.reshape(-1), s64)
    return {"texels": tex, "luminance": lum, "cdf": cdf, "probas": prob.reshape(lum.shape),
            "alias": alias.reshape(lum.shape), "total_sum": float(np.float32(s64)), "total_sum64": s64}


def env_lookup(env: OracleEnv, dirs):
    d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    out = np.zeros_like(d)
    _pt_lib().orc_env_lookup(ctypes.byref(env.c), _ptr(d, _c_f), len(d), _ptr(out, _c_f))
    return out


def env_eval(env: OracleEnv, dirs):
    d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    out = np.zeros_like(d)
    pdf = np.zeros(len(d), np.float32)
    _pt_lib().orc_env_eval(ctypes.byref(env.c), _ptr(d, _c_f), len(d), _ptr(out, _c_f), _ptr(pdf, _c_f))
    return out, pdf


def env_sample(env: OracleEnv, index=None, u=None, values=None):
    """Texel by alias draws (index, u) or CDF values -> (direction, radiance, pdf, (x, y))."""
    n = len(values) if values is not None else len(index)
    ix = None if index is None else np.ascontiguousarray(index, np.int32)
    uu = None if u is None else np.ascontiguousarray(u, np.float32)
    vv = None if values is None else np.ascontiguousarray(values, np.float32)
    d = np.zeros((n, 3), np.float32)
    c = np.zeros((n, 3), np.float32)
    p = np.zeros(n, np.float32)
    xy = np.zeros((n, 2), np.int32)
    _pt_lib().orc_env_sample(ctypes.byref(env.c), _ptr(ix, _c_i), _ptr(uu, _c_f), _ptr(vv, _c_f), n, _ptr(d, _c_f),
                             _ptr(c, _c_f), _ptr(p, _c_f), _ptr(xy, _c_i))
    return d, c, p, xy


def ref_env_available() -> bool:
    return os.path.exists(REF_ENV_SO) and os.path.exists(REF_ENV_BILINEAR_SO)


def _ref_env_lib(bilinear: bool):
    lib = ctypes.CDLL(REF_ENV_BILINEAR_SO if bilinear else REF_ENV_SO)
    if not getattr(lib, "_sigs", False):
        _u32 = ctypes.POINTER(ctypes.c_uint32)
        lib.ref_env_rgbe_pack.argtypes = [_c_f, ctypes.c_int, _u32]
        lib.ref_env_rgbe_unpack.argtypes = [_u32, ctypes.c_int, _c_f]
        lib.ref_env_lookup.argtypes = [ctypes.c_void_p, _c_f, ctypes.c_int, _c_f]
        lib.ref_env_eval.argtypes = [ctypes.c_void_p, _c_f, ctypes.c_int, _c_f, _c_f]
        lib.ref_env_sample.argtypes = [ctypes.c_void_p, _u32, ctypes.c_int, _c_f, _c_f, _c_f, _c_i, _c_f]
        lib.ref_env_cdf_search.argtypes = [ctypes.c_void_p, _c_f, ctypes.c_int, _c_i]
        lib._sigs = True
    return lib


def ref_env_pack(rgb):
    rgb = np.ascontiguousarray(rgb, np.float32).reshape(-1, 3)
    out = np.zeros(len(rgb), np.uint32)
    _ref_env_lib(False).ref_env_rgbe_pack(_ptr(rgb, _c_f), len(rgb), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    return out


def ref_env_unpack(texels):
    t = np.ascontiguousarray(texels, np.uint32).reshape(-1)
    out = np.zeros((len(t), 3), np.float32)
    _ref_env_lib(False).ref_env_rgbe_unpack(t.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), len(t), _ptr(out, _c_f))
    return out


def ref_env_lookup(env: OracleEnv, dirs):
    d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    out = np.zeros_like(d)
    r = env.ref()
    _ref_env_lib(bool(env.c.bilinear)).ref_env_lookup(ctypes.byref(r), _ptr(d, _c_f), len(d), _ptr(out, _c_f))
    return out


def ref_env_eval(env: OracleEnv, dirs):
    d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    out = np.zeros_like(d)
    pdf = np.zeros(len(d), np.float32)
    r = env.ref()
    _ref_env_lib(bool(env.c.bilinear)).ref_env_eval(ctypes.byref(r), _ptr(d, _c_f), len(d), _ptr(out, _c_f),
                                                    _ptr(pdf, _c_f))
    return out, pdf


def ref_env_sample(env: OracleEnv, seeds):
    """The reference's envmap_sample (alias table) from Xorshift32 seeds -> direction, radiance,
    pdf, and the two draws it made (table index, alias-test number)."""
    sd = np.ascontiguousarray(seeds, np.uint32)
    n = len(sd)
    d = np.zeros((n, 3), np.float32)
    c = np.zeros((n, 3), np.float32)
    p = np.zeros(n, np.float32)
    idx = np.zeros(n, np.int32)
    u = np.zeros(n, np.float32)
    r = env.ref()
    _ref_env_lib(bool(env.c.bilinear)).ref_env_sample(ctypes.byref(r), sd.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                                      n, _ptr(d, _c_f), _ptr(c, _c_f), _ptr(p, _c_f), _ptr(idx, _c_i),
                                                      _ptr(u, _c_f))
    return d, c, p, idx, u


def ref_env_cdf_search(env: OracleEnv, values):
    v = np.ascontiguousarray(values, np.float32)
    xy = np.zeros((len(v), 2), np.int32)
    r = env.ref()
    _ref_env_lib(False).ref_env_cdf_search(ctypes.byref(r), _ptr(v, _c_f), len(v), _ptr(xy, _c_i))
    return xy


def restir_spatial_seed(frame: int, pass_index: int, seed: int) -> int:
    """Per-frame spatial-neighbour seed shared by all pixels (the library's spatial_seed,
    csrc/render_api.cpp): splitmix64 finaliser of (frame, pass, seed)."""
    m = (1 << 64) - 1
    z = ((frame << 32) ^ (pass_index << 16) ^ seed ^ 0x5851F42D4C957F2D) & m
    z = (z + 0x9E3779B97F4A7C15) & m
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
    s = ((z ^ (z >> 31)) >> 16) & 0xFFFFFFFF
    return s if s != 0 else 0x9E3779B9


def _restir_lib():
    lib = _pt_lib()
    if not getattr(lib, "_restir_sigs", False):
        lib.orc_restir_gbuffer.argtypes = [_c_f, ctypes.c_int, _c_i, _c_f, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, _c_f, _c_f, _c_f, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_uint32]
        lib.orc_restir_pass.argtypes = [ctypes.c_int, _c_f, ctypes.c_int, _c_i, _c_f, _c_i, ctypes.c_int, _c_f, _c_i,
                                        ctypes.c_float, _c_f, ctypes.c_void_p, ctypes.c_void_p, _c_i, _c_f, _c_f,
                                        _c_f, _c_f, _c_f, _c_f, _c_f, ctypes.c_int, ctypes.c_uint32, ctypes.c_int,
                                        _c_f, _c_i]
        lib.orc_restir_presample.argtypes = [_c_f, ctypes.c_int, _c_i, _c_f, _c_i, ctypes.c_int, _c_f, _c_i,
                                             ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_uint32,
                                             ctypes.c_uint32, _c_f]
        lib._restir_sigs = True
    return lib


def restir_gbuffer(soup, material_of, pmats, width, height, seed, frame, jitter, inverse_view, inverse_projection,
                   nthreads=0, random_number=None) -> np.ndarray:
    """G-buffer of the camera hits, (W*H, 12) float32 (int fields as bit patterns). random_number:
    the reference's camera pass instead of the PCG jitter (frame = its sample number), with the
    reference's packed normals."""
    lib = _restir_lib()
    soup = np.ascontiguousarray(soup, np.float32)
    mo = np.ascontiguousarray(material_of, np.int32)
    pm = np.ascontiguousarray(pmats, np.float32)
    iv = np.ascontiguousarray(inverse_view, np.float32).reshape(16)
    ip = np.ascontiguousarray(inverse_projection, np.float32).reshape(16)
    gb = np.zeros((width * height, 12), np.float32)
    lib.orc_restir_gbuffer(_ptr(soup, _c_f), soup.shape[0], _ptr(mo, _c_i), _ptr(pm, _c_f), width, height, seed, frame,
                           1 if jitter else 0, _ptr(iv, _c_f), _ptr(ip, _c_f), _ptr(gb, _c_f), nthreads,
                           0 if random_number is None else 1, 0 if random_number is None else int(random_number) & 0xFFFFFFFF)
    return gb


def restir_presample(scene, strategy, subsets, size, frame, seed) -> np.ndarray:
    """The oracle's light presampling records of a frame, (subsets * size, 8) float32."""
    lib = _restir_lib()
    soup = np.ascontiguousarray(scene["soup"], np.float32)
    mo = np.ascontiguousarray(scene["material_of"], np.int32)
    em = np.ascontiguousarray(scene["emission"], np.float32)
    ei = np.ascontiguousarray(scene["emissive"], np.int32)
    ap = np.ascontiguousarray(scene["alias_prob"], np.float32)
    ai = np.ascontiguousarray(scene["alias_idx"], np.int32)
    out = np.zeros((subsets * size, 8), np.float32)
    lib.orc_restir_presample(_ptr(soup, _c_f), soup.shape[0], _ptr(mo, _c_i), _ptr(em, _c_f), _ptr(ei, _c_i), len(ei),
                             _ptr(ap, _c_f), _ptr(ai, _c_i), float(scene["power_sum"]), int(strategy), subsets * size,
                             frame, seed, _ptr(out, _c_f))
    return out


def restir_presample_seed(frame: int, seed: int) -> int:
    """The frame's presampled-subset seed (the library's spatial seed hash at pass index 31)."""
    return restir_spatial_seed(frame, 31, seed)


def restir_pass(pass_kind, scene, pmats, settings_i, settings_f, prev_vp, gb, gb_prev=None, inp=None, prev=None,
                spatial_index=0, spatial_seed=0, nthreads=0, presampled=None, presample_i=None,
                bsdf: str = "reference") -> np.ndarray:
    """One ReSTIR DI pass of the oracle (0 initial, 1 temporal, 2 spatial, 3 fused spatiotemporal)
    shading with the reference's own BSDF; scene = dict(soup, material_of, emission, emissive,
    alias_prob, alias_idx, power_sum). presampled / presample_i (subsets, size, tile, seed): light
    presampling for the initial pass. Returns (W*H, 8) reservoir records."""
    lib = _restir_lib()
    eval_fn, sample_fn = bsdf_callbacks(bsdf)
    soup = np.ascontiguousarray(scene["soup"], np.float32)
    mo = np.ascontiguousarray(scene["material_of"], np.int32)
    em = np.ascontiguousarray(scene["emission"], np.float32)
    ei = np.ascontiguousarray(scene["emissive"], np.int32)
    ap = np.ascontiguousarray(scene["alias_prob"], np.float32)
    ai = np.ascontiguousarray(scene["alias_idx"], np.int32)
    pm = np.ascontiguousarray(pmats, np.float32)
    si = np.zeros(25, np.int32)
    si_in = np.array([int(v) & 0xFFFFFFFF for v in settings_i], np.uint32).view(np.int32)
    si[:len(si_in)] = si_in
    sf = np.ascontiguousarray(settings_f, np.float32)
    vp = np.ascontiguousarray(prev_vp if prev_vp is not None else np.eye(4), np.float32).reshape(16)
    n = int(si[0]) * int(si[1])
    z = np.zeros((n, 8), np.float32)
    gbp = np.ascontiguousarray(gb_prev if gb_prev is not None else gb, np.float32)
    inp_ = np.ascontiguousarray(inp if inp is not None else z, np.float32)
    prev_ = np.ascontiguousarray(prev if prev is not None else z, np.float32)
    out = np.zeros((n, 8), np.float32)
    gb = np.ascontiguousarray(gb, np.float32)
    ps_ = None if presampled is None else np.ascontiguousarray(presampled, np.float32)
    pi_ = None if presample_i is None else np.array([int(v) & 0xFFFFFFFF for v in presample_i], np.uint32).view(np.int32)
    lib.orc_restir_pass(pass_kind, _ptr(soup, _c_f), soup.shape[0], _ptr(mo, _c_i), _ptr(em, _c_f), _ptr(ei, _c_i),
                        len(ei), _ptr(ap, _c_f), _ptr(ai, _c_i), float(scene["power_sum"]), _ptr(pm, _c_f), eval_fn,
                        sample_fn, _ptr(si, _c_i), _ptr(sf, _c_f), _ptr(vp, _c_f), _ptr(gb, _c_f), _ptr(gbp, _c_f),
                        _ptr(inp_, _c_f), _ptr(prev_, _c_f), _ptr(out, _c_f), spatial_index, spatial_seed, nthreads,
                        _ptr(ps_, _c_f), _ptr(pi_, _c_i))
    return out


def emissive_power(soup, material_of, emission, emissive) -> np.ndarray:
    """Float power list of the emissive triangles, as the reference computes it
    (src/Renderer/GPURenderer.cpp:256-275)."""
    lib = _pt_lib()
    soup = np.ascontiguousarray(soup, np.float32)
    mo = np.ascontiguousarray(material_of, np.int32)
    em = np.ascontiguousarray(emission, np.float32)
    ei = np.ascontiguousarray(emissive, np.int32)
    out = np.zeros(len(ei), np.float32)
    lib.orc_emissive_power(_ptr(soup, _c_f), _ptr(mo, _c_i), _ptr(em, _c_f), _ptr(ei, _c_i), len(ei), _ptr(out, _c_f))
    return out


def vose_alias(power: np.ndarray, total_sum: float):
    """Utils::compute_alias_table restated (src/Utils/Utils.cpp:63-131)."""
    lib = _pt_lib()
    p = np.ascontiguousarray(power, np.float32)
    prob = np.zeros(len(p), np.float32)
    alias = np.zeros(len(p), np.int32)
    lib.orc_vose_alias(_ptr(p, _c_f), len(p), float(total_sum), _ptr(prob, _c_f), _ptr(alias, _c_i))
    return prob, alias


def oct24(normals: np.ndarray) -> np.ndarray:
    """The restated octahedral-24 normal round trip of the reference's G-buffer."""
    lib = _pt_lib()
    n = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
    out = np.zeros_like(n)
    lib.orc_oct24(_ptr(n, _c_f), n.shape[0], _ptr(out, _c_f))
    return out


def alias_distribution(prob: np.ndarray, alias: np.ndarray) -> np.ndarray:
    """Probability of each index under the alias sampler (pick uniform i, keep it with prob[i])."""
    n = len(prob)
    d = prob.astype(np.float64).copy()
    np.add.at(d, alias, 1.0 - prob.astype(np.float64))
    return d / n


# ---- the reference's own render kernels (oracle/ref_render.cpp): CameraRays + MegaKernel ----
REF_RENDER_SO = {
    ("lambert", "uniform"): os.path.join(HERE, "_ref", "libref_render_lambert_uniform.so"),
    ("lambert", "power"): os.path.join(HERE, "_ref", "libref_render_lambert_power.so"),
    ("principled", "power"): os.path.join(HERE, "_ref", "libref_render_principled_power.so"),
    ("principled", "power_ris"): os.path.join(HERE, "_ref", "libref_render_principled_power_ris.so"),
    ("principled", "power_restir"): os.path.join(HERE, "_ref", "libref_render_principled_power_restir.so"),
}
_u32p = ctypes.POINTER(ctypes.c_uint32)


def ref_render_available(bsdf: str = "lambert", light: str = "uniform") -> bool:
    return os.path.exists(REF_RENDER_SO[(bsdf, light)])


def _ref_render_lib(bsdf: str, light: str):
    path = REF_RENDER_SO[(bsdf, light)]
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built: it needs the reference tree (GBPT_REFERENCE_ROOT)")
    lib = ctypes.CDLL(path)
    if not getattr(lib, "_sig", False):
        lib.refr_scene_create.restype = ctypes.c_void_p
        lib.refr_scene_create.argtypes = [_c_f, _i64, _c_i, _i64, _c_i, _c_f, ctypes.c_int32, _c_f]
        lib.refr_scene_free.argtypes = [ctypes.c_void_p]
        lib.refr_scene_light_table.argtypes = [ctypes.c_void_p, _c_i, _c_i, _c_f, _c_i, _c_f]
        lib.refr_alias_table.argtypes = [_c_f, ctypes.c_int32, ctypes.c_float, _c_f, _c_i]
        lib.refr_render.argtypes = [ctypes.c_void_p, _c_i, _c_f, _c_f, _c_f, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_uint32, _c_f,
                                    _c_i, _c_f]
        lib.refr_pack_unpack_material.argtypes = [_c_f, _c_f]
        lib.refr_oct24.argtypes = [_c_f, _i64, _c_f, _u32p]
        lib._sig = True
    return lib


class RefRender:
    """A scene in the reference's own CPU renderer (CameraRays + MegaKernel compiled from the
    reference's sources, one build per BSDF override 'lambert' / 'principled' and light sampling
    'uniform' / 'power' / 'power_ris' (RIS direct lighting over light and BSDF candidates)). materials: (M, 64) gbpt_principled_material records (for 'lambert' only
    base colour and emission matter)."""

    def __init__(self, bsdf, light, positions, indices, material_of, materials, vertex_normals=None):
        self._lib = _ref_render_lib(bsdf, light)
        self._pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        self._idx = np.ascontiguousarray(indices, np.int32).reshape(-1, 3)
        self._mo = np.ascontiguousarray(material_of, np.int32)
        self._mats = np.ascontiguousarray(materials, np.float32).reshape(-1, 64)
        self._nrm = None if vertex_normals is None else np.ascontiguousarray(vertex_normals, np.float32).reshape(-1, 3)
        self._h = self._lib.refr_scene_create(_ptr(self._pos, _c_f), self._pos.shape[0], _ptr(self._idx, _c_i),
                                              self._idx.shape[0], _ptr(self._mo, _c_i), _ptr(self._mats, _c_f),
                                              self._mats.shape[0], _ptr(self._nrm, _c_f))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.refr_scene_free(h)
            self._h = None

    def light_table(self):
        n = ctypes.c_int32(0)
        self._lib.refr_scene_light_table(self._h, ctypes.byref(n), None, None, None, None)
        e = np.zeros(n.value, np.int32)
        p = np.zeros(n.value, np.float32)
        a = np.zeros(n.value, np.int32)
        s = ctypes.c_float(0.0)
        self._lib.refr_scene_light_table(self._h, None, _ptr(e, _c_i), _ptr(p, _c_f), _ptr(a, _c_i), ctypes.byref(s))
        return dict(emissive=e, probas=p, alias=a, power_sum=s.value)

    def render(self, settings, sample_number: int, random_numbers, gbuffer: bool = False):
        """One frame (one sample per pixel) -> (H, W, 3) float32; random_numbers = the camera
        pass's and the MegaKernel pass's HIPRTRenderData::random_number. With gbuffer, also the
        camera pass's first-hit primitives (H, W) and positions (H, W, 3)."""
        rn_cam, rn_mk = (int(v) & 0xFFFFFFFF for v in random_numbers)
        s = settings
        si = np.array([s.width, s.height, s.nb_bounces, 1 if s.do_russian_roulette else 0,
                       s.russian_roulette_min_depth, 1 if s.do_jittering else 0,
                       getattr(s, "ris_light_candidates", 4), getattr(s, "ris_bsdf_candidates", 1)], np.int32)
        sf = np.array([s.russian_roulette_throughput_clamp], np.float32)
        iv = np.ascontiguousarray(s.inverse_view, np.float32).reshape(16)
        ip = np.ascontiguousarray(s.inverse_projection, np.float32).reshape(16)
        out = np.zeros((s.height, s.width, 3), np.float32)
        prim = np.zeros((s.height, s.width), np.int32) if gbuffer else None
        pos = np.zeros((s.height, s.width, 3), np.float32) if gbuffer else None
        self._lib.refr_render(self._h, _ptr(si, _c_i), _ptr(sf, _c_f), _ptr(iv, _c_f), _ptr(ip, _c_f),
                              int(sample_number) & 0xFFFFFFFF, rn_cam, rn_mk, _ptr(out, _c_f),
                              _ptr(prim, _c_i), _ptr(pos, _c_f))
        return (out, prim, pos) if gbuffer else out


class RefRestir(RefRender):
    """ReSTIR DI frames of the reference's own kernels (build 'power_restir': CameraRays,
    ReSTIR_DI_InitialCandidates / TemporalReuse / SpatialReuse and the MegaKernel's ReSTIR DI
    final shading, in the GPU renderer's pass order). Keeps the reference's per-frame state (both
    G-buffers, the reservoir buffers and which one was last frame's output) across frames."""

    def __init__(self, width, height, positions, indices, material_of, materials, vertex_normals=None):
        super().__init__("principled", "power_restir", positions, indices, material_of, materials, vertex_normals)
        lib = self._lib
        if not getattr(lib, "_restir_sig", False):
            lib.refr_restir_create.restype = ctypes.c_void_p
            lib.refr_restir_create.argtypes = [ctypes.c_int32, ctypes.c_int32]
            lib.refr_restir_free.argtypes = [ctypes.c_void_p]
            lib.refr_restir_frame.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _c_i, _c_f, _c_f, _c_f, _c_f, _c_f,
                                              ctypes.c_uint32, _u32p, _c_f, _c_f, _c_f, _c_f, _c_i, _c_f]
            lib._restir_sig = True
        self.width, self.height = int(width), int(height)
        self._st = lib.refr_restir_create(self.width, self.height)

    def __del__(self):
        st = getattr(self, "_st", None)
        if st:
            self._lib.refr_restir_free(st)
            self._st = None
        super().__del__()

    def frame(self, settings, restir, sample_number, random_numbers, prev_inverse_view, prev_view_projection):
        """One frame -> dict(image (H, W, 3), initial / temporal / final reservoirs (H*W, 8) float32
        records, prim (H, W), pos (H, W, 3)). restir: dict with light_candidates, bsdf_candidates,
        do_temporal, temporal_search_count, temporal_search_radius, do_spatial, spatial_passes,
        spatial_neighbors, spatial_radius, m_cap, use_confidence_weights, normal_similarity_cos,
        plane_distance_threshold. random_numbers: the passes' random numbers in launch order."""
        s, r = settings, restir
        W, H = self.width, self.height
        si = np.array([W, H, s.nb_bounces, 1 if s.do_russian_roulette else 0, s.russian_roulette_min_depth,
                       1 if s.do_jittering else 0, getattr(s, "ris_light_candidates", 4),
                       getattr(s, "ris_bsdf_candidates", 1), r["light_candidates"], r["bsdf_candidates"],
                       r["do_temporal"], r["temporal_search_count"], r["temporal_search_radius"], r["do_spatial"],
                       r["spatial_passes"], r["spatial_neighbors"], r["spatial_radius"], r["m_cap"],
                       r["use_confidence_weights"]], np.int32)
        sf = np.array([s.russian_roulette_throughput_clamp, r["normal_similarity_cos"],
                       r["plane_distance_threshold"]], np.float32)
        iv = np.ascontiguousarray(s.inverse_view, np.float32).reshape(16)
        ip = np.ascontiguousarray(s.inverse_projection, np.float32).reshape(16)
        piv = np.ascontiguousarray(prev_inverse_view, np.float32).reshape(16)
        pvp = np.ascontiguousarray(prev_view_projection, np.float32).reshape(16)
        rn = np.ascontiguousarray(np.asarray(random_numbers, np.uint64) & 0xFFFFFFFF, np.uint32)
        out = dict(image=np.zeros((H, W, 3), np.float32), prim=np.zeros((H, W), np.int32),
                   pos=np.zeros((H, W, 3), np.float32))
        for k in ("initial", "temporal", "final"):
            out[k] = np.zeros((H * W, 8), np.float32)
        self._lib.refr_restir_frame(self._h, self._st, _ptr(si, _c_i), _ptr(sf, _c_f), _ptr(iv, _c_f), _ptr(ip, _c_f),
                                    _ptr(piv, _c_f), _ptr(pvp, _c_f), int(sample_number) & 0xFFFFFFFF,
                                    _ptr(rn, _u32p), _ptr(out["image"], _c_f), _ptr(out["initial"], _c_f),
                                    _ptr(out["temporal"], _c_f), _ptr(out["final"], _c_f), _ptr(out["prim"], _c_i),
                                    _ptr(out["pos"], _c_f))
        return out


def ref_pack_unpack_material(materials: np.ndarray) -> np.ndarray:
    """The reference's 8-bit material packing then unpacking (CPUMaterial::pack_to_GPU,
    DevicePackedEffectiveMaterial::unpack) of (M, 64) records."""
    lib = _ref_render_lib("lambert", "uniform")
    m = np.ascontiguousarray(materials, np.float32).reshape(-1, 64)
    out = np.zeros_like(m)
    for i in range(m.shape[0]):
        lib.refr_pack_unpack_material(_ptr(m[i], _c_f), _ptr(out[i], _c_f))
    return out


def ref_oct24(normals: np.ndarray):
    """Octahedral24BitNormalPadded32b pack + unpack of (N, 3) normals -> (unpacked (N, 3), packed (N,))."""
    lib = _ref_render_lib("lambert", "uniform")
    n = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
    out = np.zeros_like(n)
    packed = np.zeros(n.shape[0], np.uint32)
    lib.refr_oct24(_ptr(n, _c_f), n.shape[0], _ptr(out, _c_f), _ptr(packed, _u32p))
    return out, packed


def ref_alias_table(power: np.ndarray, total_sum: float):
    """The reference's own Utils::compute_alias_table (extracted from src/Utils/Utils.cpp)."""
    lib = _ref_render_lib("lambert", "uniform")
    p = np.ascontiguousarray(power, np.float32)
    prob = np.zeros(len(p), np.float32)
    alias = np.zeros(len(p), np.int32)
    lib.refr_alias_table(_ptr(p, _c_f), len(p), float(total_sum), _ptr(prob, _c_f), _ptr(alias, _c_i))
    return prob, alias


def wang_hash(x: int) -> int:
    """wang_hash (src/Device/includes/Hash.h:11-19) on uint32."""
    x &= 0xFFFFFFFF
    x = ((x ^ 61) ^ (x >> 16)) & 0xFFFFFFFF
    x = (x * 9) & 0xFFFFFFFF
    x ^= x >> 4
    x = (x * 0x27D4EB2D) & 0xFFFFFFFF
    x ^= x >> 15
    return x


def xorshift32(x: int) -> int:
    """One step of the reference's Xorshift32Generator (src/HostDeviceCommon/Xorshift.h:55-62)."""
    x ^= (x << 13) & 0xFFFFFFFF
    x ^= x >> 17
    x ^= (x << 5) & 0xFFFFFFFF
    return x & 0xFFFFFFFF
