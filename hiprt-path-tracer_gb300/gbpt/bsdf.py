"""Principled BSDF entry points of libgbpt (include/gbpt_bsdf.h) over torch device tensors.

Material records are built with gbpt.materials; queries are (n, 20) float32 rows in the
gbpt_bsdf_query layout (inside and incident_lobe stored as int32 bit patterns, then the path's
wavelength and three reserved words).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

c_vp = ctypes.c_void_p
i32 = ctypes.c_int32
i64 = ctypes.c_int64


class BsdfOptions(ctypes.Structure):
    _fields_ = [("ggx_height_correlated", i32), ("reserved", i32 * 7)]


BSDF_SIGNATURES = [
    ("gbpt_bsdf_eval", ctypes.c_int, [c_vp, i32, c_vp, c_vp, i64, ctypes.POINTER(BsdfOptions), c_vp, c_vp]),
    ("gbpt_bsdf_pdf", ctypes.c_int, [c_vp, i32, c_vp, c_vp, i64, ctypes.POINTER(BsdfOptions), c_vp, c_vp]),
    ("gbpt_bsdf_sample", ctypes.c_int, [c_vp, i32, c_vp, c_vp, c_vp, i64, ctypes.POINTER(BsdfOptions), c_vp, c_vp, c_vp,
                                        c_vp]),
]

LOBES = {"none": 0, "coat": 2, "metal1": 4, "metal2": 8, "specular": 16, "glass_reflect": 32, "glass_refract": 64,
         "diffuse": 128, "diffuse_transmission": 256}


QUERY_WORDS = 20  # sizeof(gbpt_bsdf_query) / 4


def _check_queries(queries):
    if queries.dim() != 2 or queries.shape[1] != QUERY_WORDS:
        raise ValueError(f"queries must be (n, {QUERY_WORDS}) rows in the gbpt_bsdf_query layout, got "
                         f"{tuple(queries.shape)}")


def _load():
    lib = _lib.load()
    if not getattr(lib, "_bsdf_sigs", False):
        for name, res, args in BSDF_SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._bsdf_sigs = True
    return lib


def _opts(height_correlated: bool):
    o = BsdfOptions()
    o.ggx_height_correlated = 1 if height_correlated else 0
    return o


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def eval(materials, material_index, queries, height_correlated=False, stream=None):
    """f (rgb) and pdf per query -> (n, 4) float32 tensor on the queries' device."""
    import torch
    lib = _load()
    _check_queries(queries)
    n = queries.shape[0]
    out = torch.empty((n, 4), dtype=torch.float32, device=queries.device)
    _lib.check(lib.gbpt_bsdf_eval(materials.data_ptr(), materials.shape[0], material_index.data_ptr(),
                                  queries.data_ptr(), n, ctypes.byref(_opts(height_correlated)), out.data_ptr(),
                                  _stream(stream)))
    return out


def pdf(materials, material_index, queries, height_correlated=False, stream=None):
    import torch
    lib = _load()
    _check_queries(queries)
    n = queries.shape[0]
    out = torch.empty(n, dtype=torch.float32, device=queries.device)
    _lib.check(lib.gbpt_bsdf_pdf(materials.data_ptr(), materials.shape[0], material_index.data_ptr(),
                                 queries.data_ptr(), n, ctypes.byref(_opts(height_correlated)), out.data_ptr(),
                                 _stream(stream)))
    return out


def sample(materials, material_index, queries, seeds, height_correlated=False, stream=None):
    """-> (out (n, 8): direction, f, pdf, 0; lobe (n,) int32; rng state (n,) int32 bits)."""
    import torch
    lib = _load()
    _check_queries(queries)
    n = queries.shape[0]
    out = torch.empty((n, 8), dtype=torch.float32, device=queries.device)
    lobe = torch.empty(n, dtype=torch.int32, device=queries.device)
    rng = torch.empty(n, dtype=torch.int32, device=queries.device)
    _lib.check(lib.gbpt_bsdf_sample(materials.data_ptr(), materials.shape[0], material_index.data_ptr(),
                                    queries.data_ptr(), seeds.data_ptr(), n, ctypes.byref(_opts(height_correlated)),
                                    out.data_ptr(), lobe.data_ptr(), rng.data_ptr(), _stream(stream)))
    return out, lobe, rng


def as_uint32(t) -> np.ndarray:
    return t.cpu().numpy().view(np.uint32)
