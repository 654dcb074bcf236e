"""GPU: ReSTIR DI passes (initial candidates, temporal reuse, spatial reuse with pairwise MIS)
against the CPU oracle's reservoirs (tests/golden/restir_di_cornell.npz, shaded with the
reference's own principled BSDF), pass by pass, both end to end and on injected input reservoirs
("given identical candidates"); and unbiasedness of ReSTIR DI direct lighting against plain NEE.

Reservoir tolerance: same light triangle, M and flags; target function, weight sum and UCW within
1e-4 relative. The G-buffer is the GPU's own (its camera rays are FMA-contracted, the oracle's
not), and a pixel whose candidate selection u < w/w_sum sits within rounding of the threshold
picks another sample on one side only; such pixels are counted and allowed up to 2%.
"""
import os

import numpy as np
import pytest
import torch

import gbpt
from gbpt import render
from gbpt.render import BSDF_PRINCIPLED, LIGHT_POWER, RenderSettings

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "restir_di_cornell.npz")
RTOL = 1e-4
RESTIR = dict(light_candidates=8, bsdf_candidates=1, do_visibility_reuse=1, do_temporal=1, temporal_search_count=8,
              spatial_passes=1, spatial_neighbors=5, m_cap=20, use_confidence_weights=1, bias_correction_visibility=1,
              temporal_search_radius=4.0, spatial_radius=8.0, normal_similarity_cos=0.906307787,
              plane_distance_threshold=0.1)
W = H = 32
SEED = 5


def _fields(r):
    iw = r[:, 4:6].view(np.int32)
    return dict(point=r[:, 0:3], p_hat=r[:, 3], tri=iw[:, 0], M=iw[:, 1] >> 9, flags=iw[:, 1] & 0x1FF, w_sum=r[:, 6],
                ucw=r[:, 7])


def _rel_ok(a, b, rtol=RTOL, floor=1e-12):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) <= rtol * np.maximum(np.abs(a), np.abs(b)) + floor


def compare_reservoirs(got, want, min_fraction):
    g, w = _fields(got), _fields(want)
    same = (g["tri"] == w["tri"]) & (g["M"] == w["M"]) & (g["flags"] == w["flags"])
    same &= _rel_ok(g["p_hat"], w["p_hat"]) & _rel_ok(g["w_sum"], w["w_sum"]) & _rel_ok(g["ucw"], w["ucw"])
    same &= np.all(np.abs(g["point"] - w["point"]) <= 1e-4 * (1 + np.abs(w["point"])), axis=1)
    frac = float(same.mean())
    assert frac >= min_fraction, (frac, np.nonzero(~same)[0][:10])
    return frac


def _renderer(g):
    scene = gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=g["materials"])
    lt = scene.light_table()
    assert np.array_equal(lt["emissive"], g["emissive"])
    assert lt["power_sum64"] == float(g["power_sum64"])
    assert np.array_equal(lt["probas"], g["alias_prob"]) and np.array_equal(lt["alias"], g["alias_idx"])
    st = RenderSettings(width=W, height=H, samples_per_launch=1, nb_bounces=0, light_sampling=LIGHT_POWER,
                        bsdf=BSDF_PRINCIPLED, seed=SEED, inverse_view=g["f0_inverse_view"],
                        inverse_projection=g["f0_inverse_projection"])
    r = gbpt.Renderer(scene, st)
    r.set_restir_di(render.restir_di_settings(**RESTIR))
    return scene, r


def _frame_to_reservoirs(r, g, frame, inject=None):
    """Runs one ReSTIR frame pass by pass; returns the reservoirs after each pass."""
    r.set_camera(g[f"f{frame}_inverse_view"], g[f"f{frame}_inverse_projection"])
    r.pass_camera_rays()
    r.pass_extend(0)
    r.pass_restir_initial()
    out = {"initial": r.reservoirs(render.RESERVOIRS_INITIAL)}
    if inject is not None:
        r.set_reservoirs(render.RESERVOIRS_INITIAL, inject["initial"])
        r.set_reservoirs(render.RESERVOIRS_PREVIOUS, inject["previous"])
    r.pass_restir_temporal()
    out["temporal"] = r.reservoirs(render.RESERVOIRS_TEMPORAL)
    if inject is not None:
        r.set_reservoirs(render.RESERVOIRS_TEMPORAL, inject["temporal"])
    r.pass_restir_spatial(0)
    out["final"] = r.reservoirs(render.RESERVOIRS_FINAL)
    r.pass_shade(0)
    r.pass_accumulate()
    torch.cuda.synchronize()
    return out


def test_restir_passes_match_oracle_end_to_end(cuda):
    g = np.load(GOLDEN)
    _, r = _renderer(g)
    for frame in range(2):
        out = _frame_to_reservoirs(r, g, frame)
        for stage in ("initial", "temporal", "final"):
            frac = compare_reservoirs(out[stage], g[f"f{frame}_{stage}"], 0.98)
            print(f"frame {frame} {stage}: {frac:.4f} of pixels match")


def test_restir_reuse_passes_match_oracle_on_given_candidates(cuda):
    g = np.load(GOLDEN)
    _, r = _renderer(g)
    _frame_to_reservoirs(r, g, 0)
    inject = {"initial": g["f1_initial"], "previous": g["f0_final"], "temporal": g["f1_temporal"]}
    out = _frame_to_reservoirs(r, g, 1, inject)
    assert compare_reservoirs(out["temporal"], g["f1_temporal"], 0.99) >= 0.99
    assert compare_reservoirs(out["final"], g["f1_final"], 0.99) >= 0.99


def test_restir_direct_lighting_unbiased_against_nee(cuda):
    """Static camera: the mean over frames of ReSTIR DI direct lighting (temporal + spatial reuse,
    pairwise MIS, visibility reuse) equals plain NEE + MIS direct lighting (nb_bounces = 0) within
    a few standard errors of the frame means."""
    g = np.load(GOLDEN)
    scene = gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=g["materials"])
    base = dict(width=W, height=H, nb_bounces=0, light_sampling=LIGHT_POWER, bsdf=BSDF_PRINCIPLED,
                inverse_view=g["f0_inverse_view"], inverse_projection=g["f0_inverse_projection"])
    ref_st = RenderSettings(samples_per_launch=1024, seed=99, **base)
    ref = gbpt.Renderer(scene, ref_st)
    ref.render(16)
    torch.cuda.synchronize()
    want = ref.image_sums()[1] / (1024 * 16)
    frames = []
    r = gbpt.Renderer(scene, RenderSettings(samples_per_launch=1, seed=7, **base))
    r.set_restir_di(render.restir_di_settings(**RESTIR))
    prev = np.zeros_like(want)
    for f in range(256):
        r.render(1)
        cur = r.image_sums()[1]
        frames.append((cur - prev).mean())
        prev = cur
    frames = np.array(frames)
    # frames are correlated through temporal reuse: use batch means of 16 frames for the error
    batches = frames.reshape(16, 16).mean(axis=1)
    sigma = batches.std(ddof=1) / np.sqrt(len(batches))
    assert abs(frames.mean() - want.mean()) < 4 * sigma + 2e-3 * want.mean(), (frames.mean(), want.mean(), sigma)


def _frame_fused(r, g, frame, inject=None):
    """One frame with the fused spatiotemporal pass; returns the initial and final reservoirs."""
    r.set_camera(g[f"f{frame}_inverse_view"], g[f"f{frame}_inverse_projection"])
    r.pass_camera_rays()
    r.pass_extend(0)
    r.pass_restir_initial()
    out = {"initial": r.reservoirs(render.RESERVOIRS_INITIAL)}
    if inject is not None:
        r.set_reservoirs(render.RESERVOIRS_INITIAL, inject["initial"])
        r.set_reservoirs(render.RESERVOIRS_PREVIOUS, inject["previous"])
    r.pass_restir_spatiotemporal()
    out["final"] = r.reservoirs(render.RESERVOIRS_FINAL)
    r.pass_shade(0)
    r.pass_accumulate()
    torch.cuda.synchronize()
    return out


def test_fused_spatiotemporal_matches_oracle_on_given_candidates(cuda):
    """ReSTIR_DI_SpatiotemporalReuse (FusedSpatiotemporalReuse.h): frame 1's fused pass on frame 1's
    initial and frame 0's final reservoirs of the oracle, against the oracle's fused output."""
    g = np.load(GOLDEN)
    scene, _ = _renderer(g)
    st = RenderSettings(width=W, height=H, samples_per_launch=1, nb_bounces=0, light_sampling=LIGHT_POWER,
                        bsdf=BSDF_PRINCIPLED, seed=SEED, inverse_view=g["f0_inverse_view"],
                        inverse_projection=g["f0_inverse_projection"])
    r = gbpt.Renderer(scene, st)
    r.set_restir_di(render.restir_di_settings(**RESTIR, do_fused_spatiotemporal=1))
    _frame_fused(r, g, 0)
    out = _frame_fused(r, g, 1, {"initial": g["f1_initial"], "previous": g["f0_final"]})
    assert compare_reservoirs(out["final"], g["fused_f1"], 0.99) >= 0.99


def test_presampled_initial_candidates_match_oracle(cuda):
    """Light presampling (ReSTIR_DI_LightsPresampling + use_presampled_light_candidate): frame 0's
    initial candidates drawn from 16 presampled subsets of 64 lights, tiles of 8 x 8 pixels."""
    g = np.load(GOLDEN)
    scene, _ = _renderer(g)
    st = RenderSettings(width=W, height=H, samples_per_launch=1, nb_bounces=0, light_sampling=LIGHT_POWER,
                        bsdf=BSDF_PRINCIPLED, seed=SEED, inverse_view=g["f0_inverse_view"],
                        inverse_projection=g["f0_inverse_projection"])
    r = gbpt.Renderer(scene, st)
    r.set_restir_di(render.restir_di_settings(**RESTIR, do_light_presampling=1, presampling_subsets=16,
                                              presampling_subset_size=64, presampling_tile_size=8))
    out = _frame_to_reservoirs(r, g, 0)
    compare_reservoirs(out["initial"], g["ps_f0_initial"], 0.98)


@pytest.mark.parametrize("fused,presampled", [(1, 0), (1, 1), (0, 1)])
def test_fused_and_presampled_restir_unbiased_against_nee(cuda, fused, presampled):
    """As the separate-pass test: the mean over frames of ReSTIR DI direct lighting with the fused
    spatiotemporal pass and / or light presampling equals plain NEE + MIS within a few standard
    errors."""
    g = np.load(GOLDEN)
    scene = gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=g["materials"])
    base = dict(width=W, height=H, nb_bounces=0, light_sampling=LIGHT_POWER, bsdf=BSDF_PRINCIPLED,
                inverse_view=g["f0_inverse_view"], inverse_projection=g["f0_inverse_projection"])
    ref = gbpt.Renderer(scene, RenderSettings(samples_per_launch=1024, seed=99, **base))
    ref.render(16)
    torch.cuda.synchronize()
    want = ref.image_sums()[1] / (1024 * 16)
    r = gbpt.Renderer(scene, RenderSettings(samples_per_launch=1, seed=7, **base))
    r.set_restir_di(render.restir_di_settings(**RESTIR, do_fused_spatiotemporal=fused, do_light_presampling=presampled,
                                              presampling_subsets=16, presampling_subset_size=64))
    frames, prev = [], np.zeros_like(want)
    for f in range(256):
        r.render(1)
        cur = r.image_sums()[1]
        frames.append((cur - prev).mean())
        prev = cur
    frames = np.array(frames)
    batches = frames.reshape(16, 16).mean(axis=1)
    sigma = batches.std(ddof=1) / np.sqrt(len(batches))
    assert abs(frames.mean() - want.mean()) < 4 * sigma + 2e-3 * want.mean(), (frames.mean(), want.mean(), sigma)


def test_restir_settings_validation(cuda):
    from gbpt import GbptError
    g = np.load(GOLDEN)
    _, r = _renderer(g)
    for bad in (dict(do_light_presampling=1, presampling_subsets=0), dict(do_light_presampling=1, presampling_subset_size=-1),
                dict(do_light_presampling=1, presampling_subsets=1 << 13, presampling_subset_size=1 << 12),
                dict(do_fused_spatiotemporal=1, spatial_neighbors=40)):
        with pytest.raises(GbptError):
            r.set_restir_di(render.restir_di_settings(**{**RESTIR, **bad}))
