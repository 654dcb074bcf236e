"""GPU: the wavefront path tracer's ReSTIR DI in GBPT_RNG_REFERENCE mode against ReSTIR DI frames
of the REFERENCE's own kernels (tests/golden/ref_restir_cornell.npz, made by
tests/golden/make_ref_restir_golden.py: CameraRays, ReSTIR_DI_InitialCandidates,
ReSTIR_DI_TemporalReuse, ReSTIR_DI_SpatialReuse and the MegaKernel's ReSTIR DI final shading with
RIS at later bounces, in the reference GPU renderer's pass order and random numbers).

Four frames of a many-light principled Cornell box under an orbiting camera: per frame the
initial, temporal and final reservoirs and the image. The GPU contracts multiply-adds and uses its
own sqrt/sin/cos, so a reservoir whose selection draw lands within a rounding of its threshold
(or a neighbour search on a heuristic's edge) may keep another sample, and the next frames' reuse
carries that on; the test requires 97% of the reservoirs (same triangle, M and flags, the floats
within 1e-3 relative) and 95% of the pixels (1e-3 relative) of every frame to agree. (Measured:
every reservoir of every pass agrees; 98.3-98.8% of the pixels, the rest being paths whose later
RIS bounces crossed a branch threshold on one side only. The frame means are not compared: one
such path that reaches a small bright emitter moves the mean of a 48 x 48 frame by several
percent.)"""
import os

import numpy as np
import pytest
import torch

import gbpt
from gbpt.render import (BSDF_PRINCIPLED, DIRECT_RIS, LIGHT_POWER, MATERIALS_PACKED, RESERVOIRS_FINAL,
                         RESERVOIRS_INITIAL, RESERVOIRS_TEMPORAL, RNG_REFERENCE, RenderSettings, restir_di_settings)

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_restir_cornell.npz")


def _agree(a, b):
    same = (a[:, 4].view(np.int32) == b[:, 4].view(np.int32)) & (a[:, 5].view(np.int32) == b[:, 5].view(np.int32))
    f = [0, 1, 2, 3, 6, 7]
    rel = np.abs(a[:, f] - b[:, f]) / np.maximum(np.abs(b[:, f]), 1e-6)
    return same & (rel.max(axis=1) < 1e-3)


def test_restir_di_matches_reference_passes_and_frames(cuda):
    g = np.load(GOLDEN)
    S, F = int(g["size"]), int(g["frames"])
    ri, rf = g["restir_i"], g["restir_f"]
    scene = gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=g["materials"],
                       material_packing=MATERIALS_PACKED)
    st = RenderSettings(width=S, height=S, samples_per_launch=1, nb_bounces=3, russian_roulette_min_depth=3,
                        russian_roulette_throughput_clamp=0.0, light_sampling=LIGHT_POWER, bsdf=BSDF_PRINCIPLED,
                        direct_lighting=DIRECT_RIS, ris_light_candidates=4, ris_bsdf_candidates=1,
                        inverse_view=g["inverse_view"][0], inverse_projection=g["inverse_projection"][0],
                        rng_mode=RNG_REFERENCE, random_number=0)
    r = gbpt.Renderer(scene, st)
    r.set_restir_di(restir_di_settings(
        enabled=1, light_candidates=int(ri[0]), bsdf_candidates=int(ri[1]), do_visibility_reuse=1,
        do_temporal=int(ri[2]), temporal_search_count=int(ri[3]), temporal_search_radius=float(ri[4]),
        do_spatial=int(ri[5]), spatial_passes=int(ri[6]), spatial_neighbors=int(ri[7]), spatial_radius=float(ri[8]),
        m_cap=int(ri[9]), use_confidence_weights=int(ri[10]), bias_correction_visibility=1,
        do_final_shading_visibility=1, normal_similarity_cos=float(rf[0]), plane_distance_threshold=float(rf[1])))
    prev = 0.0
    for f in range(F):
        r.set_camera(g["inverse_view"][f], g["inverse_projection"][f])
        r.render(1)
        torch.cuda.synchronize()
        img = r.image_sums()[1]
        frame, prev = img - prev, img
        for which, key in ((RESERVOIRS_INITIAL, "initial"), (RESERVOIRS_TEMPORAL, "temporal"),
                           (RESERVOIRS_FINAL, "final")):
            ok = _agree(r.reservoirs(which), g[key][f])
            print(f"frame {f} {key}: {ok.mean():.4f}")
            assert ok.mean() >= 0.97, (f, key, ok.mean())
        ref = g["image"][f]
        rel = np.abs(frame - ref) / np.maximum(np.abs(ref), 1e-3)
        frac = (rel.max(axis=-1) < 1e-3).mean()
        print(f"frame {f} image: {frac:.4f}, mean {frame.mean():.5f} vs {ref.mean():.5f}")
        assert frac >= 0.95, (f, frac)
