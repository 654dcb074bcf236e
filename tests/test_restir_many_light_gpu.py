"""GPU: ReSTIR DI on the many-light benchmark scene at full size (16,777,216 heightfield triangles,
10,000 emitters, one random principled material per instance), with the benchmark's ReSTIR
settings (32 light + 1 BSDF candidates, visibility reuse, M-cap 20, temporal reuse, one spatial
pass of 5 neighbours in 30 px), against the CPU oracle's reservoirs pass by pass over two frames.

The image is a 96 x 96 crop of the benchmark's 1920 x 1080 view around its centre (the same
camera with the field of view narrowed to those rows); frame 1 orbits the camera by half a degree,
as the benchmark's frames do. The oracle traces through its octree (a restatement of the
reference's CPU BVH) and shades with the library's principled BSDF built for the host, which the
BSDF golden vectors pin to the reference's own; the estimator is the restatement pinned to the
reference's ReSTIR DI passes on the Cornell golden frames. Tolerance as the Cornell ReSTIR test:
light triangle, M and flags equal, target function, weight sum and UCW within 1e-4 relative, on at
least 97% of the pixels (the GPU's G-buffer comes from FMA-contracted camera rays and a candidate
pick sitting within rounding of its threshold differs on one side only)."""
import math

import numpy as np
import pytest
import torch

import gbpt
from gbpt import render, scenes
from gbpt import materials as M
from gbpt.render import BSDF_PRINCIPLED, LIGHT_POWER, RenderSettings, look_at_camera

from test_restir_gpu import compare_reservoirs

pytestmark = pytest.mark.gpu

W = H = 96
SEED = 9
FULL_H, FULL_VFOV = 1080, 45.0


def _orbit(eye, target, deg):
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    ex, ez = eye[0] - target[0], eye[2] - target[2]
    return (target[0] + c * ex + s * ez, eye[1], target[2] - s * ex + c * ez)


def _camera(S, frame):
    vfov = math.degrees(2.0 * math.atan(math.tan(math.radians(FULL_VFOV) / 2.0) * H / FULL_H))
    return look_at_camera(_orbit(S.eye, S.target, 0.5 * frame), S.target, vfov_deg=vfov, aspect=W / H)


def _camera_pos(iv):
    iv = np.asarray(iv, np.float32).reshape(4, 4)
    return [float(iv[0, 3]), float(iv[1, 3]), float(iv[2, 3])]


def _view_projection(iv, ip):
    prod = np.asarray(iv, np.float64).reshape(4, 4) @ np.asarray(ip, np.float64).reshape(4, 4)
    return np.linalg.inv(prod).astype(np.float32)


def test_restir_many_light_crop_matches_oracle(cuda):
    import pyoracle
    S = scenes.many_light_scene()
    assert S.mesh.n_triangles == 16_777_216 + 10_000
    scene = gbpt.Scene(S.mesh.positions, S.mesh.indices, S.material_of_triangle, principled=S.materials)
    lt = scene.light_table()
    rs = render.restir_di_settings(light_candidates=32, bsdf_candidates=1, m_cap=20, spatial_passes=1,
                                   spatial_neighbors=5, spatial_radius=30)
    iv0, ip = _camera(S, 0)
    r = gbpt.Renderer(scene, RenderSettings(width=W, height=H, samples_per_launch=1, nb_bounces=0,
                                            light_sampling=LIGHT_POWER, bsdf=BSDF_PRINCIPLED, seed=SEED,
                                            inverse_view=iv0, inverse_projection=ip))
    r.set_restir_di(rs)

    soup = np.ascontiguousarray(S.mesh.triangle_soup(), np.float32)
    eff = M.pack_many([M.coat_roughened(M.unpack(S.materials[i])) for i in range(len(S.materials))])
    sc = dict(soup=soup, material_of=np.ascontiguousarray(S.material_of_triangle, np.int32),
              emission=np.ascontiguousarray(S.materials[:, 4:7], np.float32), emissive=lt["emissive"],
              alias_prob=lt["probas"], alias_idx=lt["alias"], power_sum=np.float32(lt["power_sum64"]))
    oc = pyoracle.Oracle().octree(soup)
    pyoracle.set_scene_accel(oc)
    try:
        prev_gb = prev_final = prev_iv = None
        for frame in range(2):
            iv, ip = _camera(S, frame)
            # GPU, pass by pass
            r.set_camera(iv, ip)
            r.pass_camera_rays()
            r.pass_extend(0)
            r.pass_restir_initial()
            got = {"initial": r.reservoirs(render.RESERVOIRS_INITIAL)}
            r.pass_restir_temporal()
            got["temporal"] = r.reservoirs(render.RESERVOIRS_TEMPORAL)
            r.pass_restir_spatial(0)
            got["final"] = r.reservoirs(render.RESERVOIRS_FINAL)
            r.pass_shade(0)
            r.pass_accumulate()
            torch.cuda.synchronize()
            # oracle
            piv = prev_iv if prev_iv is not None else iv
            vp = _view_projection(piv, ip)
            si = np.array([W, H, SEED, frame, 1 if frame > 0 else 0, 1, rs.light_candidates, rs.bsdf_candidates,
                           rs.do_visibility_reuse, rs.do_temporal, rs.temporal_search_count, rs.spatial_passes,
                           rs.spatial_neighbors, rs.m_cap, rs.use_confidence_weights, rs.bias_correction_visibility],
                          np.int32)
            sf = np.array([rs.temporal_search_radius, rs.spatial_radius, rs.normal_similarity_cos,
                           rs.plane_distance_threshold, *_camera_pos(iv), *_camera_pos(piv)], np.float32)
            gb = pyoracle.restir_gbuffer(soup, sc["material_of"], eff, W, H, SEED, frame, True, iv, ip)
            init = pyoracle.restir_pass(0, sc, eff, si, sf, vp, gb, bsdf="host")
            temp = pyoracle.restir_pass(1, sc, eff, si, sf, vp, gb, gb_prev=prev_gb if prev_gb is not None else gb,
                                        inp=init, prev=prev_final, bsdf="host")
            final = pyoracle.restir_pass(2, sc, eff, si, sf, vp, gb, inp=temp, spatial_index=0,
                                         spatial_seed=pyoracle.restir_spatial_seed(frame, 0, SEED), bsdf="host")
            hit = (gb[:, 3].view(np.int32) >= 0).mean()
            assert hit > 0.9, hit
            assert (final[:, 7] > 0).mean() > 0.2
            for stage, want in (("initial", init), ("temporal", temp), ("final", final)):
                frac = compare_reservoirs(got[stage], want, 0.97)
                print(f"frame {frame} {stage}: {frac:.4f} of pixels match")
            prev_gb, prev_final, prev_iv = gb, final, iv
    finally:
        pyoracle.set_scene_accel(None)
        del oc
