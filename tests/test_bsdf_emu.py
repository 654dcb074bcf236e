"""CPU: the principled BSDF source shared with the CUDA kernels (csrc/principled.h), built for the
host, against golden vectors written by the reference's own principled BSDF (eval, pdf and
sampling with the same Xorshift32 stream)."""
import ctypes

import numpy as np
import pytest

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


def test_oren_nayar_vectors_differ_from_lambertian_where_the_lobe_shows():
    """The Oren-Nayar set selects the lobe on every material (word 45) and its values differ from
    what a Lambertian lobe gives: the host build with the selector cleared disagrees on a good share
    of the diffuse queries, and agrees on the sigma = 0 material, where A = 1 and B = 0."""
    g = G.load("oren_nayar")
    mats = np.ascontiguousarray(g["materials"])
    assert (mats[:, 45].view(np.int32) == 1).all()
    lamb = mats.copy()
    lamb[:, 45] = np.zeros(len(mats), np.int32).view(np.float32)
    lib = _lib()
    q = G.queries(g["eval_q"], g.get("eval_w"))
    mi = np.ascontiguousarray(g["eval_mat"], np.int32)
    out = np.zeros((len(q), 4), np.float32)
    lib.emu_bsdf_eval(lamb.ctypes.data, mi.ctypes.data, q.ctypes.data, len(q), 0, out.ctypes.data)
    same = G.close(out, g["eval_out"], 1e-5)
    assert same[mi == 0].all()
    assert (~same).mean() > 0.2


@pytest.mark.parametrize("which", sorted(G.SETS))
def test_host_build_eval_and_pdf_match_reference(which):
    g = G.load(which)
    lib = _lib()
    mats = np.ascontiguousarray(g["materials"])
    q = G.queries(g["eval_q"], g.get("eval_w"))
    mi = np.ascontiguousarray(g["eval_mat"], np.int32)
    out = np.zeros((len(q), 4), np.float32)
    lib.emu_bsdf_eval(mats.ctypes.data, mi.ctypes.data, q.ctypes.data, len(q), 0, out.ctypes.data)
    G.check_eval(out, g, max_flips=2)
    assert G.close(out[:, 3:4], g["pdf_out"][:, None], rtol=1e-4).mean() > 0.999


@pytest.mark.parametrize("which", sorted(G.SETS))
def test_host_build_sampling_matches_reference(which):
    g = G.load(which)
    lib = _lib()
    mats = np.ascontiguousarray(g["materials"])
    q = G.queries(g["sample_q"], g.get("sample_w"))
    mi = np.ascontiguousarray(g["sample_mat"], np.int32)
    seeds = np.ascontiguousarray(g["seeds"], np.uint32)
    out = np.zeros((len(q), 8), np.float32)
    lobe = np.zeros(len(q), np.int32)
    rng = np.zeros(len(q), np.uint32)
    lib.emu_bsdf_sample(mats.ctypes.data, mi.ctypes.data, q.ctypes.data, seeds.ctypes.data, len(q), 0,
                        out.ctypes.data, lobe.ctypes.data, rng.ctypes.data)
    G.check_sample(out, lobe, rng, g, max_flips=2)
