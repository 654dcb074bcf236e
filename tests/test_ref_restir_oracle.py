"""CPU: the ReSTIR DI oracle's reference-RNG mode against ReSTIR DI frames of the REFERENCE's own
kernels (tests/golden/ref_restir_cornell.npz, made by tests/golden/make_ref_restir_golden.py:
CameraRays, ReSTIR_DI_InitialCandidates, ReSTIR_DI_TemporalReuse, ReSTIR_DI_SpatialReuse in the
reference GPU renderer's pass order and random numbers, on a many-light principled Cornell box
whose camera orbits, so that the temporal pass backprojects).

Every pass is checked twice: on the reference's own inputs (this frame's reference G-buffer
positions, the reference's reservoirs of the previous pass) and chained through the oracle's own
outputs for all frames. A reservoir agrees when its triangle, M and flags are equal and its
point, target function, weight sum and UCW agree to 1e-4 relative."""
import numpy as np
import pytest

import pyoracle
from conftest import GOLDEN
from gbpt import materials as M

REF = pytest.mark.skipif(not (pyoracle.ref_render_available("principled", "power_restir")
                               and pyoracle.ref_render_available("lambert", "uniform")),
                         reason="needs the reference tree (oracle/_ref)")


def _agree(a, b):
    same = (a[:, 4].view(np.int32) == b[:, 4].view(np.int32)) & (a[:, 5].view(np.int32) == b[:, 5].view(np.int32))
    f = [0, 1, 2, 3, 6, 7]
    rel = np.abs(a[:, f] - b[:, f]) / np.maximum(np.abs(b[:, f]), 1e-6)
    return same & (rel.max(axis=1) < 1e-4)


def _setup():
    g = np.load(f"{GOLDEN}/ref_restir_cornell.npz")
    raw, mo = g["materials"], g["material_of"]
    q = pyoracle.ref_pack_unpack_material(raw)
    eff = M.pack_many([M.coat_roughened(M.unpack(q[i])) for i in range(len(q))])
    pm = np.concatenate([eff, pyoracle.ref_pack_unpack_material(eff)])
    lt = pyoracle.RefRender("principled", "power", g["positions"], g["indices"], mo, raw).light_table()
    soup = g["positions"][g["indices"]].reshape(-1, 9)
    sc = dict(soup=soup, material_of=mo, emission=raw[:, 4:7], emissive=lt["emissive"], alias_prob=lt["probas"],
              alias_idx=lt["alias"], power_sum=lt["power_sum"])
    return g, pm, sc, soup


def _cam(iv):
    iv = np.asarray(iv, np.float32).reshape(4, 4)
    return [iv[0, 3], iv[1, 3], iv[2, 3]]


def _view_projection(iv, ip):
    prod = np.asarray(iv, np.float64).reshape(4, 4) @ np.asarray(ip, np.float64).reshape(4, 4)
    return np.linalg.inv(prod).astype(np.float32)


def _settings(g, f, n_raw):
    ri, rf = g["restir_i"], g["restir_f"]
    S = int(g["size"])
    rn = g["random_numbers"][f]
    iv, ip = g["inverse_view"][f], g["inverse_projection"][f]
    piv = g["inverse_view"][f - 1] if f > 0 else iv
    # light, bsdf candidates, temporal on, search count, search radius, spatial on, passes,
    # neighbours, radius, M-cap, confidence weights
    si = [S, S, 0, f, 1 if f > 0 else 0, 1, ri[0], ri[1], 1, ri[2], ri[3], ri[6], ri[7], ri[9], ri[10], 1,
          1, f, int(rn[1]), int(rn[2]), int(rn[4]), 0, 0, 0, n_raw]
    sf = [float(ri[4]), float(ri[8]), float(rf[0]), float(rf[1]), *_cam(iv), *_cam(piv)]
    return si, sf, _view_projection(piv, ip), iv, ip, rn


@REF
def test_restir_oracle_matches_reference_passes():
    g, pm, sc, soup = _setup()
    S, F, n_raw = int(g["size"]), int(g["frames"]), len(g["materials"])
    prev_gb, chain_prev = None, None
    for f in range(F):
        si, sf, vp, iv, ip, rn = _settings(g, f, n_raw)
        gb = pyoracle.restir_gbuffer(soup, g["material_of"], pm, S, S, 0, f, True, iv, ip, random_number=int(rn[0]))
        assert np.array_equal(gb[:, 3].view(np.int32), g["prim"][f].reshape(-1)), f
        assert np.array_equal(gb[:, 0:3], g["pos"][f].reshape(-1, 3)), f
        gbp = prev_gb if prev_gb is not None else gb
        zero = np.zeros((S * S, 8), np.float32)
        # on the reference's own inputs
        init = pyoracle.restir_pass(0, sc, pm, si, sf, vp, gb)
        assert _agree(init, g["initial"][f]).all(), f
        ref_prev = g["final"][f - 1] if f > 0 else zero
        temp = pyoracle.restir_pass(1, sc, pm, si, sf, vp, gb, gb_prev=gbp, inp=g["initial"][f], prev=ref_prev)
        assert _agree(temp, g["temporal"][f]).all(), f
        spat = pyoracle.restir_pass(2, sc, pm, si, sf, vp, gb, inp=g["temporal"][f], spatial_index=0)
        assert _agree(spat, g["final"][f]).all(), f
        # chained through the oracle's own reservoirs
        t2 = pyoracle.restir_pass(1, sc, pm, si, sf, vp, gb, gb_prev=gbp, inp=init,
                                  prev=chain_prev if chain_prev is not None else zero)
        chain_prev = pyoracle.restir_pass(2, sc, pm, si, sf, vp, gb, inp=t2, spatial_index=0)
        assert _agree(chain_prev, g["final"][f]).mean() > 0.999, f
        prev_gb = gb
