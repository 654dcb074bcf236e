"""Scene, light table and wavefront renderer (host-side mirror of the reference's renderer API).

  * ``Scene(mesh, material_of_triangle, albedo, emission)`` <- GPURenderer::set_scene
    (src/Renderer/GPURenderer.cpp:952-958): BVH, emissive list, power alias table on the device.
  * ``Renderer(scene, settings)``                          <- GPURenderer + its render passes
  * ``Renderer.render(n)``                                 <- GPURendererThread::render_path_tracing
  * ``Renderer.pass_camera_rays / pass_bounce / pass_accumulate`` <- CameraRays / MegaKernel bounce /
    path_tracing_accumulate_color, for callers that schedule passes themselves.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import c_vp, i32, i64

LIGHT_UNIFORM = 0
LIGHT_POWER = 1
BSDF_LAMBERTIAN = 1
BSDF_PRINCIPLED = 3
DIRECT_MIS, DIRECT_RIS = 0, 1
RNG_PCG, RNG_REFERENCE = 0, 1
MATERIALS_FLOAT, MATERIALS_PACKED = 0, 1
GBPT_ALIAS_NOALLOC_MAX_EMITTERS = 131072  # include/gbpt_render.h


class Material(ctypes.Structure):
    _fields_ = [("base_color", ctypes.c_float * 3), ("emission", ctypes.c_float * 3)]


class SceneDesc(ctypes.Structure):
    _fields_ = [("positions", c_vp), ("n_vertices", i64), ("indices", c_vp), ("n_triangles", i64),
                ("material_indices", c_vp), ("materials", c_vp), ("n_materials", i32),
                ("principled_materials", c_vp), ("vertex_normals", c_vp), ("material_packing", i32)]


class RenderSettingsC(ctypes.Structure):
    _fields_ = [("width", i32), ("height", i32), ("samples_per_launch", i32), ("nb_bounces", i32),
                ("do_russian_roulette", i32), ("russian_roulette_min_depth", i32),
                ("russian_roulette_throughput_clamp", ctypes.c_float), ("light_sampling", i32), ("bsdf", i32),
                ("seed", ctypes.c_uint32), ("do_jittering", i32), ("ggx_height_correlated", i32),
                ("direct_lighting", i32), ("ris_light_candidates", i32), ("ris_bsdf_candidates", i32),
                ("rng_mode", i32),
                ("inverse_view", ctypes.c_float * 16), ("inverse_projection", ctypes.c_float * 16),
                ("random_number", ctypes.c_uint32)]


class RenderStatsC(ctypes.Structure):
    _fields_ = [("samples", i64), ("extension_rays", i64), ("shadow_rays", i64), ("bsdf_light_rays", i64)]


class RestirDISettingsC(ctypes.Structure):
    _fields_ = [("enabled", i32), ("light_candidates", i32), ("bsdf_candidates", i32), ("do_visibility_reuse", i32),
                ("do_temporal", i32), ("temporal_search_count", i32), ("temporal_search_radius", ctypes.c_float),
                ("do_spatial", i32), ("spatial_passes", i32), ("spatial_neighbors", i32),
                ("spatial_radius", ctypes.c_float), ("m_cap", i32), ("use_confidence_weights", i32),
                ("bias_correction_visibility", i32), ("do_final_shading_visibility", i32),
                ("normal_similarity_cos", ctypes.c_float), ("plane_distance_threshold", ctypes.c_float),
                ("do_fused_spatiotemporal", i32), ("do_light_presampling", i32), ("presampling_subsets", i32),
                ("presampling_subset_size", i32), ("presampling_tile_size", i32), ("reserved", i32 * 10)]


RESERVOIRS_INITIAL, RESERVOIRS_TEMPORAL, RESERVOIRS_FINAL, RESERVOIRS_PREVIOUS = 0, 1, 2, 3

AMBIENT_NONE, AMBIENT_UNIFORM, AMBIENT_ENVMAP = 0, 1, 2
ENVMAP_NO_SAMPLING, ENVMAP_BINARY_SEARCH, ENVMAP_ALIAS_TABLE = 0, 1, 2


class WorldDescC(ctypes.Structure):
    _fields_ = [("ambient", i32), ("uniform_color", ctypes.c_float * 3), ("envmap_rgb", c_vp),
                ("envmap_width", i32), ("envmap_height", i32), ("envmap_intensity", ctypes.c_float),
                ("envmap_scale_background", i32), ("envmap_to_world", ctypes.c_float * 9),
                ("world_to_envmap", ctypes.c_float * 9), ("envmap_sampling", i32), ("envmap_bsdf_mis", i32),
                ("envmap_bilinear", i32)]


class GltfCameraC(ctypes.Structure):
    _fields_ = [("present", i32), ("position", ctypes.c_float * 3), ("forward", ctypes.c_float * 3),
                ("up", ctypes.c_float * 3), ("yfov", ctypes.c_float), ("aspect_ratio", ctypes.c_float),
                ("znear", ctypes.c_float), ("zfar", ctypes.c_float)]


RENDER_SIGNATURES = [
    ("gbpt_material_pack_8bit", ctypes.c_int, [c_vp, i32, c_vp]),
    ("gbpt_gltf_load", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(c_vp)]),
    ("gbpt_gltf_scene_desc", ctypes.c_int, [c_vp, ctypes.POINTER(SceneDesc)]),
    ("gbpt_gltf_get_camera", ctypes.c_int, [c_vp, ctypes.POINTER(GltfCameraC)]),
    ("gbpt_gltf_destroy", ctypes.c_int, [c_vp]),
    ("gbpt_scene_create", ctypes.c_int, [ctypes.POINTER(SceneDesc), ctypes.POINTER(_lib.BvhParams),
                                         ctypes.POINTER(c_vp), c_vp]),
    ("gbpt_scene_destroy", ctypes.c_int, [c_vp]),
    ("gbpt_scene_get_bvh", ctypes.c_int, [c_vp, ctypes.POINTER(c_vp)]),
    ("gbpt_scene_get_light_table", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    ("gbpt_world_default", ctypes.c_int, [ctypes.POINTER(WorldDescC)]),
    ("gbpt_scene_set_world", ctypes.c_int, [c_vp, ctypes.POINTER(WorldDescC), c_vp]),
    ("gbpt_scene_get_envmap_tables", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    ("gbpt_renderer_create", ctypes.c_int, [c_vp, ctypes.POINTER(RenderSettingsC), ctypes.POINTER(c_vp)]),
    ("gbpt_renderer_destroy", ctypes.c_int, [c_vp]),
    ("gbpt_renderer_reset", ctypes.c_int, [c_vp, c_vp]),
    ("gbpt_render", ctypes.c_int, [c_vp, i32, c_vp]),
    ("gbpt_pass_camera_rays", ctypes.c_int, [c_vp, c_vp]),
    ("gbpt_pass_bounce", ctypes.c_int, [c_vp, i32, c_vp]),
    ("gbpt_pass_accumulate", ctypes.c_int, [c_vp, c_vp]),
    ("gbpt_renderer_get_image", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp]),
    ("gbpt_renderer_get_stats", ctypes.c_int, [c_vp, ctypes.POINTER(RenderStatsC), c_vp]),
    ("gbpt_alias_table_build_noalloc", ctypes.c_int, [c_vp, i32, c_vp, c_vp, c_vp, c_vp]),
    ("gbpt_restir_di_default_settings", ctypes.c_int, [ctypes.POINTER(RestirDISettingsC)]),
    ("gbpt_renderer_set_restir_di", ctypes.c_int, [c_vp, ctypes.POINTER(RestirDISettingsC)]),
    ("gbpt_renderer_set_camera", ctypes.c_int, [c_vp, c_vp, c_vp]),
    ("gbpt_pass_extend", ctypes.c_int, [c_vp, i32, c_vp]),
    ("gbpt_pass_shade", ctypes.c_int, [c_vp, i32, c_vp]),
    ("gbpt_pass_restir_di_initial", ctypes.c_int, [c_vp, c_vp]),
    ("gbpt_pass_restir_di_temporal", ctypes.c_int, [c_vp, c_vp]),
    ("gbpt_pass_restir_di_spatial", ctypes.c_int, [c_vp, i32, c_vp]),
    ("gbpt_pass_restir_di_spatiotemporal", ctypes.c_int, [c_vp, c_vp]),
    ("gbpt_restir_di_get_reservoirs", ctypes.c_int, [c_vp, i32, c_vp, c_vp]),
    ("gbpt_restir_di_set_reservoirs", ctypes.c_int, [c_vp, i32, c_vp, c_vp]),
    ("gbpt_guide_render_default_settings", ctypes.c_int, [c_vp]),
    ("gbpt_renderer_set_guide", ctypes.c_int, [c_vp, c_vp, c_vp]),
    ("gbpt_renderer_get_guide_records", ctypes.c_int, [c_vp, c_vp, i32, c_vp, c_vp]),
    ("gbpt_renderer_set_sample_index", ctypes.c_int, [c_vp, i64]),
    ("gbpt_batch_default_params", ctypes.c_int, [c_vp]),
    ("gbpt_batch_create", ctypes.c_int, [c_vp, i32, c_vp, c_vp]),
    ("gbpt_batch_destroy", ctypes.c_int, [c_vp]),
    ("gbpt_batch_render", ctypes.c_int, [c_vp, c_vp]),
    ("gbpt_batch_job_seconds", ctypes.c_int, [c_vp, c_vp]),
    ("gbpt_batch_get_image", ctypes.c_int, [c_vp, i32, c_vp, c_vp, c_vp]),
    ("gbpt_batch_get_stats", ctypes.c_int, [c_vp, c_vp, c_vp]),
]


class BatchJobC(ctypes.Structure):
    _fields_ = [("scene", c_vp), ("settings", RenderSettingsC)]


class BatchParamsC(ctypes.Structure):
    _fields_ = [("samples_per_iteration", i32), ("use_graph", i32), ("reserved", i32 * 6)]


class GuideRenderSettingsC(ctypes.Structure):
    _fields_ = [("enabled", i32), ("train", i32), ("guide_probability", ctypes.c_float), ("max_records", i32),
                ("weight_clamp", ctypes.c_float), ("reserved", i32 * 11)]


def guide_render_settings(**kw) -> GuideRenderSettingsC:
    """Defaults of gbpt_guide_render_default_settings with the given fields overridden."""
    lib = _load()
    c = GuideRenderSettingsC()
    _lib.check(lib.gbpt_guide_render_default_settings(ctypes.byref(c)))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise KeyError(k)
        setattr(c, k, v)
    return c


def restir_di_settings(**kw) -> RestirDISettingsC:
    """The reference's ReSTIR DI defaults with the given fields overridden."""
    lib = _load()
    c = RestirDISettingsC()
    _lib.check(lib.gbpt_restir_di_default_settings(ctypes.byref(c)))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise KeyError(k)
        setattr(c, k, v)
    return c


def _stream(stream) -> int:
    import torch
    if stream is None:
        return int(torch.cuda.current_stream().cuda_stream)
    return int(stream.cuda_stream)


def look_at_camera(eye, target, up=(0.0, 1.0, 0.0), vfov_deg=40.0, aspect=1.0, near=0.1, far=100.0):
    """(inverse_view, inverse_projection), row-major float32 4x4, points multiplied on the right.
    View space looks down -z (OpenGL convention); NDC (x, y, -1) maps to the near plane."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, np.asarray(up, np.float64))
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    inv_view = np.eye(4)
    inv_view[:3, 0], inv_view[:3, 1], inv_view[:3, 2], inv_view[:3, 3] = s, u, -f, eye
    t = np.tan(np.radians(vfov_deg) / 2)
    proj = np.zeros((4, 4))
    proj[0, 0] = 1 / (aspect * t)
    proj[1, 1] = 1 / t
    proj[2, 2] = -(far + near) / (far - near)
    proj[2, 3] = -2 * far * near / (far - near)
    proj[3, 2] = -1
    return inv_view.astype(np.float32), np.linalg.inv(proj).astype(np.float32)


@dataclass
class RenderSettings:
    width: int = 256
    height: int = 256
    samples_per_launch: int = 1
    nb_bounces: int = 4
    do_russian_roulette: bool = True
    russian_roulette_min_depth: int = 3
    russian_roulette_throughput_clamp: float = 0.0
    light_sampling: int = LIGHT_UNIFORM
    bsdf: int = BSDF_LAMBERTIAN
    seed: int = 1
    do_jittering: bool = True
    ggx_height_correlated: bool = False
    direct_lighting: int = 0  # DIRECT_MIS
    ris_light_candidates: int = 4
    ris_bsdf_candidates: int = 1
    rng_mode: int = RNG_PCG  # RNG_REFERENCE: the reference's generator and draw order (gbpt_render.h)
    random_number: int = 0   # RNG_REFERENCE: seed of the per-launch random numbers (0: 42)
    inverse_view: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))
    inverse_projection: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))

    def to_c(self) -> RenderSettingsC:
        c = RenderSettingsC()
        for k in ("width", "height", "samples_per_launch", "nb_bounces", "russian_roulette_min_depth",
                  "light_sampling", "bsdf", "seed", "direct_lighting", "ris_light_candidates", "ris_bsdf_candidates",
                  "rng_mode"):
            setattr(c, k, int(getattr(self, k)))
        c.random_number = int(self.random_number) & 0xFFFFFFFF
        c.do_russian_roulette = 1 if self.do_russian_roulette else 0
        c.do_jittering = 1 if self.do_jittering else 0
        c.ggx_height_correlated = 1 if self.ggx_height_correlated else 0
        c.russian_roulette_throughput_clamp = float(self.russian_roulette_throughput_clamp)
        c.inverse_view[:] = [float(v) for v in np.asarray(self.inverse_view, np.float32).reshape(16)]
        c.inverse_projection[:] = [float(v) for v in np.asarray(self.inverse_projection, np.float32).reshape(16)]
        return c


def _load():
    lib = _lib.load()
    if not getattr(lib, "_render_sigs", False):
        for name, res, args in RENDER_SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._render_sigs = True
    return lib


def material_pack_8bit(materials: np.ndarray) -> np.ndarray:
    """(M, 64) material records as the reference's packed records read them back
    (gbpt_material_pack_8bit; host code, no device needed)."""
    lib = _load()
    m = np.ascontiguousarray(materials, np.float32).reshape(-1, 64).copy()
    _lib.check(lib.gbpt_material_pack_8bit(m.ctypes.data, m.shape[0], m.ctypes.data))
    return m


class World:
    """The world around a scene (the reference's WorldSettings): ambient AMBIENT_NONE, AMBIENT_UNIFORM
    (uniform_color seen by every miss) or AMBIENT_ENVMAP (envmap: (H, W, 3) float texels, row 0 at
    the -y pole; rotation: 3x3 envmap-to-world matrix)."""

    def __init__(self, ambient=AMBIENT_NONE, uniform_color=(0.0, 0.0, 0.0), envmap=None, intensity=1.0,
                 scale_background=False, rotation=None, sampling=ENVMAP_ALIAS_TABLE, bsdf_mis=True, bilinear=False):
        self.ambient = int(ambient)
        self.uniform_color = tuple(float(c) for c in uniform_color)
        self.envmap = None if envmap is None else np.ascontiguousarray(envmap, np.float32)
        if self.envmap is not None and (self.envmap.ndim != 3 or self.envmap.shape[2] != 3):
            raise ValueError("envmap must be (H, W, 3)")
        self.intensity = float(intensity)
        self.scale_background = bool(scale_background)
        self.rotation = np.eye(3, dtype=np.float32) if rotation is None else np.asarray(rotation, np.float32).reshape(3, 3)
        self.inverse_rotation = np.linalg.inv(self.rotation.astype(np.float64)).astype(np.float32)
        self.sampling = int(sampling)
        self.bsdf_mis = bool(bsdf_mis)
        self.bilinear = bool(bilinear)

    def to_c(self) -> WorldDescC:
        w = WorldDescC()
        _lib.check(_load().gbpt_world_default(ctypes.byref(w)))
        w.ambient = self.ambient
        w.uniform_color[:] = list(self.uniform_color)
        if self.envmap is not None:
            w.envmap_rgb = self.envmap.ctypes.data
            w.envmap_height, w.envmap_width = self.envmap.shape[:2]
        w.envmap_intensity = self.intensity
        w.envmap_scale_background = int(self.scale_background)
        w.envmap_to_world[:] = [float(v) for v in self.rotation.reshape(-1)]
        w.world_to_envmap[:] = [float(v) for v in self.inverse_rotation.reshape(-1)]
        w.envmap_sampling = self.sampling
        w.envmap_bsdf_mis = int(self.bsdf_mis)
        w.envmap_bilinear = int(self.bilinear)
        return w


class Scene:
    def __init__(self, positions, indices, material_of_triangle, albedo=None, emission=None, stream=None, sah_bins=128,
                 max_leaf_size=1, principled=None, vertex_normals=None, material_packing=MATERIALS_FLOAT):
        """albedo/emission: (M, 3) plain materials; principled: (M, 64) gbpt.materials records (the
        reference's CPUMaterial parameters; base colour and emission come from them when albedo is
        None); vertex_normals: (V, 3) smooth-shading normals (a zero row: none at that vertex);
        material_packing: MATERIALS_PACKED stores the materials as the reference's 8-bit packed
        records."""
        lib = _load()
        self._pm = None
        if principled is not None:
            self._pm = np.ascontiguousarray(principled, np.float32).reshape(-1, 64)
            if albedo is None:
                albedo = self._pm[:, 0:3]
                emission = self._pm[:, 4:7]
        self._pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        self._idx = np.ascontiguousarray(indices, np.int32).reshape(-1, 3)
        self._mat_of = np.ascontiguousarray(material_of_triangle, np.int32).reshape(-1)
        alb = np.asarray(albedo, np.float32).reshape(-1, 3)
        emi = np.asarray(emission, np.float32).reshape(-1, 3)
        self._mats = (Material * len(alb))()
        for k in range(len(alb)):
            self._mats[k].base_color[:] = [float(v) for v in alb[k]]
            self._mats[k].emission[:] = [float(v) for v in emi[k]]
        self._nrm = None
        if vertex_normals is not None:
            self._nrm = np.ascontiguousarray(vertex_normals, np.float32).reshape(-1, 3)
            if self._nrm.shape[0] != self._pos.shape[0]:
                raise ValueError("vertex_normals needs one normal per vertex")
        desc = SceneDesc(self._pos.ctypes.data, self._pos.shape[0], self._idx.ctypes.data, self._idx.shape[0],
                         self._mat_of.ctypes.data, ctypes.addressof(self._mats), len(alb),
                         self._pm.ctypes.data if self._pm is not None else None,
                         self._nrm.ctypes.data if self._nrm is not None else None, int(material_packing))
        params = _lib.BvhParams(sah_bins, max_leaf_size, 0)
        h = c_vp()
        _lib.check(lib.gbpt_scene_create(ctypes.byref(desc), ctypes.byref(params), ctypes.byref(h), _stream(stream)))
        self._h = h
        self._lib = lib
        self.world = World()

    @classmethod
    def from_cornell(cls, cb, **kw):
        return cls(cb.mesh.positions, cb.mesh.indices, cb.material_of_triangle, cb.albedo, cb.emission, **kw)

    @property
    def handle(self):
        return self._h

    def light_table(self):
        n = ctypes.c_int32()
        _lib.check(self._lib.gbpt_scene_get_light_table(self._h, ctypes.addressof(n), None, None, None, None, None))
        e = np.zeros(n.value, np.int32)
        p = np.zeros(n.value, np.float32)
        a = np.zeros(n.value, np.int32)
        s32 = ctypes.c_float()
        s64 = ctypes.c_double()
        _lib.check(self._lib.gbpt_scene_get_light_table(self._h, None, e.ctypes.data, p.ctypes.data, a.ctypes.data,
                                                        ctypes.addressof(s32), ctypes.addressof(s64)))
        return {"emissive": e, "probas": p, "alias": a, "power_sum": s32.value, "power_sum64": s64.value}

    def set_world(self, world: "World", stream=None):
        """Sets the world (ambient light / envmap); builds the envmap tables on the device."""
        w = world.to_c()
        _lib.check(self._lib.gbpt_scene_set_world(self._h, ctypes.byref(w), _stream(stream)))
        self.world = world

    def envmap_tables(self):
        """Device envmap tables: RGB9E5 texels, CDF, alias probabilities and indices (H, W each)."""
        # the library answers first whether the scene's world has an envmap
        _lib.check(self._lib.gbpt_scene_get_envmap_tables(self._h, None, None, None, None, None, None))
        h, w = self.world.envmap.shape[:2]
        tex = np.zeros((h, w), np.uint32)
        cdf = np.zeros((h, w), np.float32)
        prob = np.zeros((h, w), np.float32)
        alias = np.zeros((h, w), np.int32)
        s32 = ctypes.c_float()
        s64 = ctypes.c_double()
        _lib.check(self._lib.gbpt_scene_get_envmap_tables(self._h, tex.ctypes.data, cdf.ctypes.data, prob.ctypes.data,
                                                          alias.ctypes.data, ctypes.addressof(s32),
                                                          ctypes.addressof(s64)))
        return {"texels": tex, "cdf": cdf, "probas": prob, "alias": alias, "total_sum": s32.value,
                "total_sum64": s64.value}

    def destroy(self):
        if getattr(self, "_h", None):
            _lib.check(self._lib.gbpt_scene_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


@dataclass
class GltfScene:
    """A glTF 2.0 file read by gbpt_gltf_load: world-space triangles, per-triangle material indices,
    principled material records (M, 64), the file's camera (None when it has none) and world-space
    vertex normals (None when no primitive has any)."""
    positions: np.ndarray
    indices: np.ndarray
    material_of_triangle: np.ndarray
    principled: np.ndarray
    camera: dict | None
    vertex_normals: np.ndarray | None = None

    def create_scene(self, **kw) -> "Scene":
        return Scene(self.positions, self.indices, self.material_of_triangle, principled=self.principled,
                     vertex_normals=self.vertex_normals, **kw)

    def camera_matrices(self, aspect=None, near=0.1, far=100.0):
        """(inverse_view, inverse_projection) of the file's camera with its vertical field of view
        (the glTF yfov; the reference's ASSIMP route widens it by 0.425 rad). near/far default to
        the reference's fixed clip planes (src/Scene/SceneParser.cpp:258-259)."""
        c = self.camera
        if c is None:
            raise ValueError("the glTF scene has no perspective camera")
        if aspect is None:
            aspect = c["aspect_ratio"] or 1.0
        eye = np.asarray(c["position"], np.float64)
        return look_at_camera(eye, eye + np.asarray(c["forward"], np.float64), c["up"],
                              vfov_deg=float(np.degrees(c["yfov"])), aspect=aspect, near=near, far=far)


def load_gltf(path) -> GltfScene:
    """Reads a .gltf/.glb file through gbpt_gltf_load (the library's own parser)."""
    lib = _load()
    h = c_vp()
    _lib.check(lib.gbpt_gltf_load(os.fsencode(os.fspath(path)), ctypes.byref(h)))
    try:
        d = SceneDesc()
        _lib.check(lib.gbpt_gltf_scene_desc(h, ctypes.byref(d)))
        nv, nt, nm = int(d.n_vertices), int(d.n_triangles), int(d.n_materials)

        def copy(ptr, n, dtype):
            if n == 0:
                return np.zeros(0, dtype)
            buf = (ctypes.c_char * (n * np.dtype(dtype).itemsize)).from_address(ptr)
            return np.frombuffer(buf, dtype).copy()

        pos = copy(d.positions, nv * 3, np.float32).reshape(nv, 3)
        idx = copy(d.indices, nt * 3, np.int32).reshape(nt, 3)
        mat = copy(d.material_indices, nt, np.int32)
        pm = copy(d.principled_materials, nm * 64, np.float32).reshape(nm, 64)
        nrm = copy(d.vertex_normals, nv * 3, np.float32).reshape(nv, 3) if d.vertex_normals else None
        cam = GltfCameraC()
        _lib.check(lib.gbpt_gltf_get_camera(h, ctypes.byref(cam)))
        camera = None
        if cam.present:
            camera = {"position": tuple(cam.position), "forward": tuple(cam.forward), "up": tuple(cam.up),
                      "yfov": cam.yfov, "aspect_ratio": cam.aspect_ratio, "znear": cam.znear, "zfar": cam.zfar}
        return GltfScene(pos, idx, mat, pm, camera, nrm)
    finally:
        lib.gbpt_gltf_destroy(h)


class Renderer:
    def __init__(self, scene: Scene, settings: RenderSettings):
        lib = _load()
        self.scene = scene  # keeps the scene alive
        self.settings = settings
        h = c_vp()
        c = settings.to_c()
        _lib.check(lib.gbpt_renderer_create(scene.handle, ctypes.byref(c), ctypes.byref(h)))
        self._h = h
        self._lib = lib

    def render(self, n_launches: int = 1, stream=None):
        _lib.check(self._lib.gbpt_render(self._h, n_launches, _stream(stream)))

    def reset(self, stream=None):
        _lib.check(self._lib.gbpt_renderer_reset(self._h, _stream(stream)))

    def set_sample_index(self, first_sample: int):
        """Sample index of the next launch (sample-range sharding across ranks)."""
        _lib.check(self._lib.gbpt_renderer_set_sample_index(self._h, int(first_sample)))

    def pass_camera_rays(self, stream=None):
        _lib.check(self._lib.gbpt_pass_camera_rays(self._h, _stream(stream)))

    def pass_bounce(self, bounce: int, stream=None):
        _lib.check(self._lib.gbpt_pass_bounce(self._h, bounce, _stream(stream)))

    def pass_extend(self, bounce: int, stream=None):
        _lib.check(self._lib.gbpt_pass_extend(self._h, bounce, _stream(stream)))

    def pass_shade(self, bounce: int, stream=None):
        _lib.check(self._lib.gbpt_pass_shade(self._h, bounce, _stream(stream)))

    def set_restir_di(self, settings: "RestirDISettingsC"):
        _lib.check(self._lib.gbpt_renderer_set_restir_di(self._h, ctypes.byref(settings)))

    def set_camera(self, inverse_view, inverse_projection):
        iv = np.ascontiguousarray(inverse_view, np.float32).reshape(16)
        ip = np.ascontiguousarray(inverse_projection, np.float32).reshape(16)
        _lib.check(self._lib.gbpt_renderer_set_camera(self._h, iv.ctypes.data, ip.ctypes.data))

    def pass_restir_initial(self, stream=None):
        _lib.check(self._lib.gbpt_pass_restir_di_initial(self._h, _stream(stream)))

    def pass_restir_temporal(self, stream=None):
        _lib.check(self._lib.gbpt_pass_restir_di_temporal(self._h, _stream(stream)))

    def pass_restir_spatiotemporal(self, stream=None):
        _lib.check(self._lib.gbpt_pass_restir_di_spatiotemporal(self._h, _stream(stream)))

    def pass_restir_spatial(self, pass_index: int = 0, stream=None):
        _lib.check(self._lib.gbpt_pass_restir_di_spatial(self._h, pass_index, _stream(stream)))

    def reservoirs(self, which: int, stream=None) -> np.ndarray:
        """(H*W, 8) float32 reservoir records (words 4-5 are int32 bit patterns)."""
        n = self.settings.width * self.settings.height
        out = np.zeros((n, 8), np.float32)
        _lib.check(self._lib.gbpt_restir_di_get_reservoirs(self._h, which, out.ctypes.data, _stream(stream)))
        return out

    def set_reservoirs(self, which: int, data: np.ndarray, stream=None):
        d = np.ascontiguousarray(data, np.float32).reshape(-1, 8)
        _lib.check(self._lib.gbpt_restir_di_set_reservoirs(self._h, which, d.ctypes.data, _stream(stream)))

    def set_guide(self, guide, settings: "GuideRenderSettingsC | None" = None):
        """Attaches a gbpt.guide.Guide (kept alive by the renderer) or detaches with None."""
        self._guide = guide
        s = settings if settings is not None else guide_render_settings()
        _lib.check(self._lib.gbpt_renderer_set_guide(self._h, guide.handle if guide is not None else None,
                                                     ctypes.byref(s)))

    def guide_records(self, capacity: int = 1 << 16, stream=None):
        """-> (count made by the last launch, (k, 15) float32 records: position, normal, view, direction,
        weight, BSDF pdf, slot (int32 bits))."""
        out = np.zeros((capacity, 15), np.float32)
        n = i32(0)
        _lib.check(self._lib.gbpt_renderer_get_guide_records(self._h, out.ctypes.data, capacity, ctypes.byref(n),
                                                             _stream(stream)))
        return n.value, out[:min(n.value, capacity)]

    def pass_accumulate(self, stream=None):
        _lib.check(self._lib.gbpt_pass_accumulate(self._h, _stream(stream)))

    def image_sums(self, stream=None):
        """(FP32 sums, FP64 sums) as (H, W, 3) arrays; row 0 is the bottom row."""
        w, h = self.settings.width, self.settings.height
        a32 = np.zeros((h, w, 3), np.float32)
        a64 = np.zeros((h, w, 3), np.float64)
        _lib.check(self._lib.gbpt_renderer_get_image(self._h, a32.ctypes.data, a64.ctypes.data, _stream(stream)))
        return a32, a64

    def stats(self, stream=None) -> dict:
        s = RenderStatsC()
        _lib.check(self._lib.gbpt_renderer_get_stats(self._h, ctypes.byref(s), _stream(stream)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def destroy(self):
        if getattr(self, "_h", None):
            _lib.check(self._lib.gbpt_renderer_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def cornell_settings(width=256, height=256, **kw) -> RenderSettings:
    """The Cornell-box configuration: camera at (2.75, 2.75, -8) looking +z, 40 degree vertical
    FOV, 4 bounces, Russian roulette from bounce 3, uniform light sampling, Lambertian BSDF."""
    iv, ip = look_at_camera((2.75, 2.75, -8.0), (2.75, 2.75, 0.0), vfov_deg=40.0, aspect=width / height)
    s = RenderSettings(width=width, height=height, inverse_view=iv, inverse_projection=ip)
    for k, v in kw.items():
        setattr(s, k, v)
    return s


class Batch:
    """Many independent render jobs in one wavefront (gbpt_batch_*): jobs is a list of
    (Scene, RenderSettings) whose samples_per_launch is each job's total samples per pixel."""

    def __init__(self, jobs, samples_per_iteration: int = 4, use_graph: bool = True):
        lib = _load()
        self._lib = lib
        self._scenes = [sc for sc, _ in jobs]  # keep the scenes alive
        self.settings = [st for _, st in jobs]
        arr = (BatchJobC * len(jobs))()
        for k, (sc, st) in enumerate(jobs):
            arr[k].scene = sc.handle
            arr[k].settings = st.to_c()
        p = BatchParamsC()
        _lib.check(lib.gbpt_batch_default_params(ctypes.byref(p)))
        p.samples_per_iteration = samples_per_iteration
        p.use_graph = 1 if use_graph else 0
        h = c_vp()
        _lib.check(lib.gbpt_batch_create(arr, len(jobs), ctypes.byref(p), ctypes.byref(h)))
        self._h = h

    def render(self, stream=None):
        _lib.check(self._lib.gbpt_batch_render(self._h, _stream(stream)))

    def job_seconds(self) -> np.ndarray:
        out = np.zeros(len(self.settings), np.float64)
        _lib.check(self._lib.gbpt_batch_job_seconds(self._h, out.ctypes.data))
        return out

    def image_sums(self, job: int, stream=None):
        st = self.settings[job]
        a32 = np.zeros((st.height, st.width, 3), np.float32)
        a64 = np.zeros((st.height, st.width, 3), np.float64)
        _lib.check(self._lib.gbpt_batch_get_image(self._h, job, a32.ctypes.data, a64.ctypes.data, _stream(stream)))
        return a32, a64

    def stats(self, stream=None) -> dict:
        s = RenderStatsC()
        _lib.check(self._lib.gbpt_batch_get_stats(self._h, ctypes.byref(s), _stream(stream)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def destroy(self):
        if getattr(self, "_h", None):
            _lib.check(self._lib.gbpt_batch_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

