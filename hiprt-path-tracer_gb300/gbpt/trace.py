"""Acceleration structure and ray queries (host-side mirror of the reference's traversal API).

Mirrors, over the C ABI:
  * ``BVH(indices, positions)``           <- HIPRTGeometry::build_bvh (src/HIPRT-Orochi/HIPRTScene.h:87-150)
  * ``BVH.closest(rays)``                 <- trace_main_path_ray's traversal (src/Device/includes/Intersect.h:200)
  * ``BVH.occluded(rays)``                <- evaluate_shadow_ray_occluded (src/Device/includes/Intersect.h:276)

Device buffers are torch CUDA tensors (torch is used for device memory and streams only; every
computation runs in libgbpt's CUDA kernels). Rays are SoA queues: origin_tmin (N,4) float32,
dir_tmax (N,4) float32, last_prim (N,) int32. Closest hits are (N,4) float32 records
(t, u, v, prim as int32 bits); ``hit_prim(hits)`` reinterprets the last column.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _stream_handle(stream) -> int:
    import torch
    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream)


def _ptr(t) -> int:
    return int(t.data_ptr()) if t is not None else 0


def hit_prim(hits):
    """Primitive indices of closest-hit records (int32 view of column 3)."""
    if isinstance(hits, np.ndarray):
        return hits[:, 3].view(np.int32)
    import torch
    return hits[:, 3].contiguous().view(torch.int32)


class BVH:
    """8-wide compressed BVH over a triangle mesh, resident on the current CUDA device."""

    def __init__(self, indices: np.ndarray, positions: np.ndarray, sah_bins: int = 128, max_leaf_size: int = 1,
                 num_threads: int = 0):
        lib = _lib.load()
        idx = np.ascontiguousarray(indices, dtype=np.int32).reshape(-1, 3)
        pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3)
        params = _lib.BvhParams(sah_bins, max_leaf_size, num_threads)
        handle = ctypes.c_void_p()
        _lib.check(lib.gbpt_bvh_build(idx.ctypes.data_as(_lib.c_i32), pos.ctypes.data_as(_lib.c_f), pos.shape[0],
                                      idx.shape[0], ctypes.byref(params), ctypes.byref(handle)))
        self._h = handle
        self._lib = lib

    @property
    def handle(self) -> ctypes.c_void_p:
        if not self._h:
            raise RuntimeError("BVH has been destroyed")
        return self._h

    def stats(self) -> dict:
        s = _lib.BvhStats()
        _lib.check(self._lib.gbpt_bvh_get_stats(self.handle, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_ if f != "reserved"}

    def destroy(self) -> None:
        if getattr(self, "_h", None):
            _lib.check(self._lib.gbpt_bvh_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    # ---- device-resident queues -------------------------------------------------------------
    def closest(self, origin_tmin, dir_tmax, last_prim=None, out=None, stream=None):
        import torch
        n = origin_tmin.shape[0]
        if out is None:
            out = torch.empty((n, 4), dtype=torch.float32, device=origin_tmin.device)
        _lib.check(self._lib.gbpt_trace_closest(self.handle, _ptr(origin_tmin), _ptr(dir_tmax), _ptr(last_prim), n,
                                                _ptr(out), _stream_handle(stream)))
        return out

    def occluded(self, origin_tmin, dir_tmax, last_prim=None, out=None, stream=None):
        import torch
        n = origin_tmin.shape[0]
        if out is None:
            out = torch.empty((n,), dtype=torch.uint8, device=origin_tmin.device)
        _lib.check(self._lib.gbpt_trace_any(self.handle, _ptr(origin_tmin), _ptr(dir_tmax), _ptr(last_prim), n,
                                            _ptr(out), _stream_handle(stream)))
        return out

    # ---- launch configuration and autotuning -------------------------------------------------
    def trace_config(self, any_hit: bool = False) -> dict:
        c = _lib.TraceConfig()
        _lib.check(self._lib.gbpt_bvh_get_trace_config(self.handle, 1 if any_hit else 0, ctypes.byref(c)))
        return {f: getattr(c, f) for f, _ in c._fields_ if f != "reserved"}

    def set_trace_config(self, any_hit: bool = False, **cfg) -> None:
        c = _lib.TraceConfig(**{**self.trace_config(any_hit), **cfg})
        _lib.check(self._lib.gbpt_bvh_set_trace_config(self.handle, 1 if any_hit else 0, ctypes.byref(c)))

    def autotune(self, origin_tmin, dir_tmax, last_prim=None, any_hit: bool = False, store: bool = True, stream=None):
        """Times candidate launch configurations on this device batch; returns (config, ms per launch)."""
        c = _lib.TraceConfig()
        ms = ctypes.c_float(0.0)
        n = origin_tmin.shape[0]
        _lib.check(self._lib.gbpt_trace_autotune(self.handle, _ptr(origin_tmin), _ptr(dir_tmax), _ptr(last_prim), n,
                                                 1 if any_hit else 0, 1 if store else 0, ctypes.byref(c),
                                                 ctypes.byref(ms), _stream_handle(stream)))
        return {f: getattr(c, f) for f, _ in c._fields_ if f != "reserved"}, ms.value

    def closest_cfg(self, origin_tmin, dir_tmax, last_prim=None, out=None, stream=None, **cfg):
        """Closest hits with an explicit launch configuration (fields of gbpt_trace_config)."""
        import torch
        n = origin_tmin.shape[0]
        if out is None:
            out = torch.empty((n, 4), dtype=torch.float32, device=origin_tmin.device)
        c = _lib.TraceConfig(**{**self.trace_config(False), **cfg})
        _lib.check(self._lib.gbpt_trace_closest_cfg(self.handle, _ptr(origin_tmin), _ptr(dir_tmax), _ptr(last_prim), n,
                                                    _ptr(out), ctypes.byref(c), _stream_handle(stream)))
        return out

    def occluded_cfg(self, origin_tmin, dir_tmax, last_prim=None, out=None, stream=None, **cfg):
        import torch
        n = origin_tmin.shape[0]
        if out is None:
            out = torch.empty((n,), dtype=torch.uint8, device=origin_tmin.device)
        c = _lib.TraceConfig(**{**self.trace_config(True), **cfg})
        _lib.check(self._lib.gbpt_trace_any_cfg(self.handle, _ptr(origin_tmin), _ptr(dir_tmax), _ptr(last_prim), n,
                                                _ptr(out), ctypes.byref(c), _stream_handle(stream)))
        return out

    def count(self, origin_tmin, dir_tmax, last_prim=None, any_hit: bool = False, stream=None):
        """(nodes visited, triangles tested) summed over the batch, from the counting kernels."""
        import torch
        n = origin_tmin.shape[0]
        counters = torch.zeros(2, dtype=torch.int64, device=origin_tmin.device)
        _lib.check(self._lib.gbpt_trace_count(self.handle, _ptr(origin_tmin), _ptr(dir_tmax), _ptr(last_prim), n,
                                              1 if any_hit else 0, _ptr(counters), _stream_handle(stream)))
        c = counters.cpu().numpy()
        return int(c[0]), int(c[1])

    # ---- host buffers (end-to-end: copies inside the call) ------------------------------------
    def closest_host(self, origin_tmin, dir_tmax, last_prim=None, out=None, stream=None):
        """Host arrays or (pinned) CPU tensors in, host results out; synchronous."""
        n = origin_tmin.shape[0]
        if out is None:
            out = np.empty((n, 4), np.float32)
        _lib.check(self._lib.gbpt_trace_closest_host(self.handle, _host_ptr(origin_tmin), _host_ptr(dir_tmax),
                                                     _host_ptr(last_prim), n, _host_ptr(out), _stream_handle(stream)))
        return out

    def occluded_host(self, origin_tmin, dir_tmax, last_prim=None, out=None, stream=None):
        n = origin_tmin.shape[0]
        if out is None:
            out = np.empty((n,), np.uint8)
        _lib.check(self._lib.gbpt_trace_any_host(self.handle, _host_ptr(origin_tmin), _host_ptr(dir_tmax),
                                                 _host_ptr(last_prim), n, _host_ptr(out), _stream_handle(stream)))
        return out


def _host_ptr(a) -> int:
    if a is None:
        return 0
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return int(a.ctypes.data)
    assert a.is_contiguous() and a.device.type == "cpu"
    return int(a.data_ptr())


def classify_hit_differences(mesh, rays, a, b, edge_rel=2.5e-7, mt_epsilon=1e-7):
    """Compares the closest-hit records a (Moller-Trumbore, the parity test) and b (watertight) of
    the same rays -> dict of counts {agree, edge, parallel, tie, other}:
      agree: both miss, or the same triangle at the same point: |t_a - t_b| cos(theta) <= 4e-6 s
        and the points their (u, v) address within 4e-6 s k / cos(theta), with s = max(t, |origin|)
        the magnitude of the coordinates both tests round (a bounce ray's t can be far below its
        origin's), theta the angle between the ray and the triangle's normal (the position of a
        grazing intersection along the ray is conditioned by 1 / cos(theta)) and k = max(1,
        longest edge^2 / (2 area)) the triangle's aspect (a sliver's barycentrics are conditioned
        by it: both tests divide edge functions of size ~area by the determinant);
      parallel (checked first): b hits a triangle whose Moller-Trumbore determinant e1 . (d x e2),
        in float as the reference computes it, is within +-mt_epsilon: the reference's test treats
        such a ray as parallel to the triangle and never reports it (src/Renderer/Triangle.h:22-31)
        - grazing hits on small triangles that only the watertight test keeps;
      edge: a different outcome where a hit lies within edge_rel s / max(cos(theta), 1e-3) of an
        edge of its triangle, measured in the plane perpendicular to the ray (the plane both tests
        decide in: a coordinate rounding decides which side of the edge the ray passes, and a
        grazing incidence stretches that rounding by 1 / cos(theta));
      tie: two different triangles hit at the same t (1e-6 relative);
      other: anything else."""
    pa, pb = a[:, 3].view(np.int32), b[:, 3].view(np.int32)
    soup = np.asarray(mesh.triangle_soup(), np.float32).reshape(-1, 3, 3)
    tri = soup.astype(np.float64)
    origin = np.asarray(rays.origin_tmin)[:, :3].astype(np.float64)
    direction = np.asarray(rays.dir_tmax)[:, :3].astype(np.float64)
    same = pa == pb
    both = np.nonzero(same & (pa >= 0))[0]
    T = tri[pa[both]]
    e1, e2 = T[:, 1] - T[:, 0], T[:, 2] - T[:, 0]
    n = np.cross(e1, e2)
    dn = direction[both] / np.linalg.norm(direction[both], axis=1, keepdims=True)
    cos = np.abs(np.einsum("ij,ij->i", n, dn)) / np.maximum(np.linalg.norm(n, axis=1), 1e-300)
    cos = np.maximum(cos, 1e-6)

    def at(h):
        return T[:, 0] + h[both, 1:2].astype(np.float64) * e1 + h[both, 2:3].astype(np.float64) * e2

    t = a[both, 0].astype(np.float64)
    scale = np.maximum(t, np.linalg.norm(origin[both], axis=1))
    e3 = T[:, 0] - T[:, 2]
    longest2 = np.maximum(np.maximum((e1 * e1).sum(1), (e2 * e2).sum(1)), ((T[:, 2] - T[:, 1]) ** 2).sum(1))
    longest2 = np.maximum(longest2, (e3 * e3).sum(1))
    aspect = np.maximum(1.0, longest2 / np.maximum(np.linalg.norm(n, axis=1), 1e-300))
    ok = (np.abs(t - b[both, 0]) * cos <= 4e-6 * scale) & \
         (np.linalg.norm(at(a) - at(b), axis=1) * cos <= 4e-6 * scale * aspect)
    counts = dict(agree=int((same & (pa < 0)).sum() + ok.sum()), edge=0, parallel=0, tie=0, other=int((~ok).sum()))

    def edge_distance(i, h):
        """(distance of the hit from its triangle's nearest edge, perpendicular to the ray;
        |cos| of the incidence)"""
        o, d = origin[i], direction[i] / np.linalg.norm(direction[i])
        v0, v1, v2 = tri[int(h[3:4].view(np.int32)[0])]
        nv = np.cross(v1 - v0, v2 - v0)
        c = abs(float(np.dot(nv, d))) / max(float(np.linalg.norm(nv)), 1e-300)
        p = v0 + float(h[1]) * (v1 - v0) + float(h[2]) * (v2 - v0)

        def perp(x):
            return x - np.dot(x - o, d) * d

        q, w = perp(p), [perp(v) for v in (v0, v1, v2)]
        best = np.inf
        for k in range(3):
            s0, s1 = w[k], w[(k + 1) % 3]
            e = s1 - s0
            s = np.clip(np.dot(q - s0, e) / max(np.dot(e, e), 1e-300), 0.0, 1.0)
            best = min(best, float(np.linalg.norm(q - (s0 + s * e))))
        return best, c

    def mt_determinant(i, prim):
        v0, v1, v2 = soup[prim]
        d = np.asarray(rays.dir_tmax)[i, :3].astype(np.float32)
        return float(np.dot(v1 - v0, np.cross(d, v2 - v0)))

    for i in np.nonzero(~same)[0]:
        if pb[i] >= 0 and abs(mt_determinant(i, pb[i])) < mt_epsilon:
            counts["parallel"] += 1
            continue
        o_len = float(np.linalg.norm(origin[i]))
        near = False
        for h, p in ((a, pa), (b, pb)):
            if p[i] >= 0:
                dist, c = edge_distance(i, h[i])
                near = near or dist <= edge_rel * max(float(h[i, 0]), o_len) / max(c, 1e-3)
        if near:
            counts["edge"] += 1
        elif pa[i] >= 0 and pb[i] >= 0 and abs(float(a[i, 0]) - float(b[i, 0])) <= 1e-6 * max(1.0, abs(float(a[i, 0]))):
            counts["tie"] += 1
        else:
            counts["other"] += 1
    return counts
