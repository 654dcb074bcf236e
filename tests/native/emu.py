"""TEST INFRASTRUCTURE ONLY — ctypes wrapper of tests/native/libtraverse_emu.so."""
import ctypes

import numpy as np

from . import build_emu

_lib = None


def lib():
    global _lib
    if _lib is None:
        l = ctypes.CDLL(build_emu.build())
        l.emu_build.restype = ctypes.c_void_p
        l.emu_build.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                                ctypes.c_int]
        l.emu_free.argtypes = [ctypes.c_void_p]
        l.emu_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        l.emu_export.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        l.emu_trace.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int64, ctypes.c_int, ctypes.c_void_p,
                                                        ctypes.c_void_p]
        l.emu_last_error.restype = ctypes.c_char_p
        _lib = l
    return _lib


class EmuBVH:
    def __init__(self, mesh, max_leaf=1, bins=128):  # the library's defaults (csrc/bvh.h BuildParams)
        self.idx = np.ascontiguousarray(mesh.indices, np.int32)
        self.pos = np.ascontiguousarray(mesh.positions, np.float32)
        self.h = lib().emu_build(self.idx.ctypes.data, self.pos.ctypes.data, self.pos.shape[0], self.idx.shape[0],
                                 max_leaf, bins)
        if not self.h:
            raise RuntimeError(lib().emu_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().emu_free(self.h)

    def stats(self):
        s = np.zeros(4, np.int64)
        lib().emu_stats(self.h, s.ctypes.data)
        return dict(n_nodes=int(s[0]), n_tris=int(s[1]), wide_depth=int(s[2]), n_binary_nodes=int(s[3]))

    def export(self):
        st = self.stats()
        nodes = np.zeros(st["n_nodes"] * 80, np.uint8)
        tris = np.zeros((st["n_tris"], 12), np.float32)
        lib().emu_export(self.h, nodes.ctypes.data, tris.ctypes.data)
        return nodes.reshape(-1, 80), tris

    def trace(self, rays, any_hit=False, watertight=False):
        o = np.ascontiguousarray(rays.origin_tmin, np.float32)
        d = np.ascontiguousarray(rays.dir_tmax, np.float32)
        lp = np.ascontiguousarray(rays.last_prim, np.int32)
        out = np.zeros((len(o), 4), np.float32)
        cnt = np.zeros(2, np.int64)
        lib().emu_trace(self.h, o.ctypes.data, d.ctypes.data, lp.ctypes.data, len(o), (1 if any_hit else 0) | (2 if watertight else 0),
                        out.ctypes.data, cnt.ctypes.data)
        return out, cnt
