"""Guiding network entry points of libgbpt (include/gbpt_guide.h) over torch device tensors.

The network maps (position, normal) to a mixture of 8 von Mises-Fisher lobes. It is trained
online on radiance-weighted directions. Forward, backward and Adam run in libgbpt's CUDA kernels:
the MLP uses the tcgen05 tensor cores.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

c_vp = ctypes.c_void_p
c_f = ctypes.POINTER(ctypes.c_float)
i32 = ctypes.c_int32
u32 = ctypes.c_uint32
i64 = ctypes.c_int64

LEVELS, TABLE, FEATURES = 16, 524288, 2
GRID_PARAMS = LEVELS * TABLE * FEATURES
IN, HIDDEN, OUT, LOBES, ROW = 64, 64, 48, 8, 44
WEIGHTS = 3 * HIDDEN * HIDDEN + HIDDEN * OUT


class GuideParams(ctypes.Structure):
    _fields_ = [("scene_min", ctypes.c_float * 3), ("scene_max", ctypes.c_float * 3), ("learning_rate", ctypes.c_float),
                ("beta1", ctypes.c_float), ("beta2", ctypes.c_float), ("epsilon", ctypes.c_float), ("seed", u32),
                ("max_batch", i32), ("wait_limit", i32), ("reserved", i32 * 5)]


GUIDE_SIGNATURES = [
    ("gbpt_guide_default_params", ctypes.c_int, [ctypes.POINTER(GuideParams)]),
    ("gbpt_guide_create", ctypes.c_int, [ctypes.POINTER(GuideParams), ctypes.POINTER(c_vp)]),
    ("gbpt_guide_destroy", ctypes.c_int, [c_vp]),
    ("gbpt_guide_train", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, i64, c_f, c_vp]),
    ("gbpt_guide_gradients", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, i64, c_f, c_f, c_f, c_vp]),
    ("gbpt_guide_infer", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, i64, c_vp, c_vp]),
    ("gbpt_guide_error_flag", ctypes.c_int, [c_vp, ctypes.POINTER(i32)]),
    ("gbpt_guide_get_params", ctypes.c_int, [c_vp, c_f, c_f]),
    ("gbpt_guide_set_params", ctypes.c_int, [c_vp, c_f, c_f]),
]


def _load():
    lib = _lib.load()
    if not getattr(lib, "_guide_sigs", False):
        for name, res, args in GUIDE_SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._guide_sigs = True
    return lib


def default_params(**kw) -> GuideParams:
    p = GuideParams()
    _lib.check(_load().gbpt_guide_default_params(ctypes.byref(p)))
    for k, v in kw.items():
        if k in ("scene_min", "scene_max"):
            getattr(p, k)[:] = [float(x) for x in v]
        else:
            setattr(p, k, v)
    return p


def split_rows(rows):
    """(n, ROW) inferred rows -> lobes (n, 8, 5) and alpha (n,) views."""
    return rows[:, :LOBES * 5].reshape(-1, LOBES, 5), rows[:, LOBES * 5]


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(c_f)


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _dev(t, n):
    import torch
    t = t.to(device="cuda", dtype=torch.float32).contiguous()
    assert t.numel() == n
    return t


class Guide:
    """Owns one gbpt_guide. Arrays passed to train/gradients/infer are torch CUDA tensors."""

    def __init__(self, params: GuideParams | None = None, **kw):
        self._lib = _load()
        p = params if params is not None else default_params(**kw)
        self.params = p
        h = c_vp()
        _lib.check(self._lib.gbpt_guide_create(ctypes.byref(p), ctypes.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            _lib.check(self._lib.gbpt_guide_destroy(self._h))
            self._h = c_vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def train(self, position, normal, view, direction, weight, bsdf_pdf=None, want_loss=True, stream=None):
        n = weight.numel()
        pos, nrm, v, d, w = (_dev(position, 3 * n), _dev(normal, 3 * n), _dev(view, 3 * n), _dev(direction, 3 * n),
                             _dev(weight, n))
        pb = None if bsdf_pdf is None else _dev(bsdf_pdf, n)
        loss = ctypes.c_float(0.0)
        _lib.check(self._lib.gbpt_guide_train(self._h, pos.data_ptr(), nrm.data_ptr(), v.data_ptr(), d.data_ptr(),
                                              w.data_ptr(), None if pb is None else pb.data_ptr(), n,
                                              ctypes.byref(loss) if want_loss else None, _stream(stream)))
        return loss.value if want_loss else None

    def gradients(self, position, normal, view, direction, weight, bsdf_pdf=None, stream=None):
        """-> (grad_weights (WEIGHTS,), grad_grid (GRID_PARAMS,), loss) as numpy float32."""
        n = weight.numel()
        pos, nrm, v, d, w = (_dev(position, 3 * n), _dev(normal, 3 * n), _dev(view, 3 * n), _dev(direction, 3 * n),
                             _dev(weight, n))
        pb = None if bsdf_pdf is None else _dev(bsdf_pdf, n)
        gw = np.zeros(WEIGHTS, np.float32)
        gg = np.zeros(GRID_PARAMS, np.float32)
        loss = ctypes.c_float(0.0)
        _lib.check(self._lib.gbpt_guide_gradients(self._h, pos.data_ptr(), nrm.data_ptr(), v.data_ptr(), d.data_ptr(),
                                                  w.data_ptr(), None if pb is None else pb.data_ptr(), n, _fptr(gw),
                                                  _fptr(gg), ctypes.byref(loss), _stream(stream)))
        return gw, gg, loss.value

    def infer(self, position, normal, view, stream=None):
        """-> (n, ROW) float32 CUDA tensor: 8 x (mu xyz, kappa, weight), alpha, 3 unused."""
        import torch
        n = position.numel() // 3
        pos, nrm, v = _dev(position, 3 * n), _dev(normal, 3 * n), _dev(view, 3 * n)
        out = torch.empty((n, ROW), dtype=torch.float32, device="cuda")
        _lib.check(self._lib.gbpt_guide_infer(self._h, pos.data_ptr(), nrm.data_ptr(), v.data_ptr(), n, out.data_ptr(),
                                              _stream(stream)))
        return out

    def error_flag(self) -> int:
        f = i32(0)
        _lib.check(self._lib.gbpt_guide_error_flag(self._h, ctypes.byref(f)))
        return f.value

    def get_params(self):
        w = np.zeros(WEIGHTS, np.float32)
        g = np.zeros(GRID_PARAMS, np.float32)
        _lib.check(self._lib.gbpt_guide_get_params(self._h, _fptr(w), _fptr(g)))
        return w, g

    def set_params(self, weights=None, grid=None):
        w = None if weights is None else np.ascontiguousarray(weights, np.float32)
        g = None if grid is None else np.ascontiguousarray(grid, np.float32)
        assert w is None or w.size == WEIGHTS
        assert g is None or g.size == GRID_PARAMS
        _lib.check(self._lib.gbpt_guide_set_params(self._h, None if w is None else _fptr(w),
                                                   None if g is None else _fptr(g)))
