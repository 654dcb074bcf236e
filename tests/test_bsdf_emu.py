"""CPU: the principled BSDF source shared with the CUDA kernels (csrc/principled.h), built for the
host, against golden vectors written by the reference's own principled BSDF (eval, pdf and
sampling with the same Xorshift32 stream)."""
import ctypes

import numpy as np

import bsdf_golden as G
from native import build_emu


def _lib():
    lib = ctypes.CDLL(build_emu.build())
    vp = ctypes.c_void_p
    lib.emu_bsdf_eval.argtypes = [vp, vp, vp, ctypes.c_int64, ctypes.c_int, vp]
    lib.emu_bsdf_sample.argtypes = [vp, vp, vp, vp, ctypes.c_int64, ctypes.c_int, vp, vp, vp]
    return lib


def test_golden_vectors_cover_every_lobe():
    g = G.load()
    lobes = set(np.unique(g["sample_info"]).tolist())
    assert {2, 4, 8, 16, 32, 64, 128, 256} <= lobes
    assert (g["eval_out"][:, 3] > 0).mean() > 0.5
    assert np.isfinite(g["eval_out"]).all() and np.isfinite(g["sample_out"]).all()


def test_host_build_eval_and_pdf_match_reference():
    g = G.load()
    lib = _lib()
    mats = np.ascontiguousarray(g["materials"])
    q = G.queries(g["eval_q"])
    mi = np.ascontiguousarray(g["eval_mat"], np.int32)
    out = np.zeros((len(q), 4), np.float32)
    lib.emu_bsdf_eval(mats.ctypes.data, mi.ctypes.data, q.ctypes.data, len(q), 0, out.ctypes.data)
    G.check_eval(out, g, max_flips=2)
    assert G.close(out[:, 3:4], g["pdf_out"][:, None], rtol=1e-4).mean() > 0.999


def test_host_build_sampling_matches_reference():
    g = G.load()
    lib = _lib()
    mats = np.ascontiguousarray(g["materials"])
    q = G.queries(g["sample_q"])
    mi = np.ascontiguousarray(g["sample_mat"], np.int32)
    seeds = np.ascontiguousarray(g["seeds"], np.uint32)
    out = np.zeros((len(q), 8), np.float32)
    lobe = np.zeros(len(q), np.int32)
    rng = np.zeros(len(q), np.uint32)
    lib.emu_bsdf_sample(mats.ctypes.data, mi.ctypes.data, q.ctypes.data, seeds.ctypes.data, len(q), 0,
                        out.ctypes.data, lobe.ctypes.data, rng.ctypes.data)
    G.check_sample(out, lobe, rng, g, max_flips=2)
