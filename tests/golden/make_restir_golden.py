"""Generates tests/golden/restir_di_cornell.npz: ReSTIR DI reservoirs of two frames of a principled
Cornell box with 16 extra small emitters, computed by the CPU oracle (oracle/restir_oracle.cpp)
shading with the REFERENCE's own principled BSDF (oracle/_ref/libref.so).

Per frame it stores the camera G-buffer and the reservoirs after the initial-candidates, temporal
and spatial passes; frame 1 moves the camera by half a degree so that the temporal pass
backprojects. The GPU test runs the same passes (same PCG streams and Xorshift32 BSDF seeds) and,
separately, each reuse pass on these stored input reservoirs ("given identical candidates").
Also: the fused spatiotemporal pass of frame 1 on frame 1's initial and frame 0's final
reservoirs (fused_f1), and frame 0's initial candidates drawn from presampled lights
(PRESAMPLE subsets x size, tiles of 8 pixels; ps_f0_initial).
Usage (where the reference tree is present):  python tests/golden/make_restir_golden.py
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "hiprt-path-tracer_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, HERE)

from gbpt import materials as M, scenes  # noqa: E402
from gbpt.render import look_at_camera  # noqa: E402
import pyoracle  # noqa: E402
from make_pt_principled_golden import MATERIALS  # noqa: E402

OUT = os.path.join(HERE, "restir_di_cornell.npz")
W = H = 32
SEED = 5
N_EMIT = 16
# light candidates, bsdf candidates, visibility reuse, temporal, temporal search, spatial passes,
# spatial neighbours, m cap, confidence weights, bias-correction visibility
RESTIR_I = dict(light_candidates=8, bsdf_candidates=1, do_visibility_reuse=1, do_temporal=1, temporal_search_count=8,
                spatial_passes=1, spatial_neighbors=5, m_cap=20, use_confidence_weights=1, bias_correction_visibility=1)
RESTIR_F = dict(temporal_search_radius=4.0, spatial_radius=8.0, normal_similarity_cos=0.906307787,
                plane_distance_threshold=0.1)
PRESAMPLE = dict(presampling_subsets=16, presampling_subset_size=64, presampling_tile_size=8)


def scene():
    """Principled Cornell box (materials of the principled golden image) plus N_EMIT small emitters
    of log-uniform radiance; returns mesh, material per triangle, raw and effective materials."""
    cb = scenes.cornell_box()
    rng = np.random.Generator(np.random.PCG64(11))
    em = scenes.random_triangles(N_EMIT, seed=12, lo=(0.8, 1.0, 0.8), hi=(4.7, 4.5, 4.7), sigma=0.25)
    mesh = scenes.merge(cb.mesh, em)
    mat_of = np.concatenate([cb.material_of_triangle.copy(), len(MATERIALS) + np.arange(N_EMIT, dtype=np.int32)])
    mat_of[10:22] = 4
    mat_of[22:34] = 5
    mats = list(MATERIALS)
    rad = np.exp(rng.uniform(0.0, math.log(50.0), N_EMIT))
    for k in range(N_EMIT):
        col = rng.uniform(0.3, 1.0, 3)
        mats.append(dict(base_color=(0.0, 0.0, 0.0), emission=tuple(float(v) for v in rad[k] * col)))
    raw = M.pack_many(mats)
    eff = M.pack_many([M.coat_roughened(m) for m in mats])
    return mesh, mat_of.astype(np.int32), raw, eff


def camera(frame):
    """Orbit of the Cornell camera about the box centre, 0.5 degree per frame."""
    a = math.radians(0.5 * frame)
    cx, cz = 2.75, 2.75
    ex, ez = 2.75 - cx, -8.0 - cz
    eye = (cx + ex * math.cos(a) - ez * math.sin(a), 2.75, cz + ex * math.sin(a) + ez * math.cos(a))
    return look_at_camera(eye, (2.75, 2.75, 2.75), vfov_deg=40.0, aspect=W / H)


def camera_pos(iv):
    iv = np.asarray(iv, np.float32).reshape(4, 4)
    w = iv[3, 3] if iv[3, 3] != 0 else np.float32(1)
    return np.array([iv[0, 3] / w, iv[1, 3] / w, iv[2, 3] / w], np.float32)


def view_projection(iv, ip):
    prod = np.asarray(iv, np.float64).reshape(4, 4) @ np.asarray(ip, np.float64).reshape(4, 4)
    return np.linalg.inv(prod).astype(np.float32)


def device_sum64(x):
    """The library's deterministic FP64 sum order (render.cu sum_f64_kernel + sum_partials_kernel):
    64 blocks of contiguous chunks, 256 strided lanes per block, shared-memory tree, then the same
    over the 64 partials."""
    x = np.asarray(x, np.float32).astype(np.float64)
    n = len(x)

    def block(vals, lanes=256):
        acc = [0.0] * lanes
        for i, v in enumerate(vals):
            acc[i % lanes] += v
        w = lanes // 2
        while w > 0:
            for t in range(w):
                acc[t] += acc[t + w]
            w //= 2
        return acc[0]

    chunk = (n + 63) // 64
    partials = [block(x[b * chunk:min(n, (b + 1) * chunk)]) if b * chunk < n else 0.0 for b in range(64)]
    return block(partials)


def light_table(mesh, mat_of, emission):
    emissive = np.nonzero(np.any(emission[mat_of] != 0, axis=1))[0].astype(np.int32)
    power = pyoracle.emissive_power(mesh.triangle_soup(), mat_of, emission, emissive)
    s64 = device_sum64(power)
    prob, alias = pyoracle.vose_alias(power, s64)
    return emissive, prob, alias, s64


def settings_arrays(frame, has_prev, cam, prev_cam):
    si = np.array([W, H, SEED, frame, has_prev, 1, RESTIR_I["light_candidates"], RESTIR_I["bsdf_candidates"],
                   RESTIR_I["do_visibility_reuse"], RESTIR_I["do_temporal"], RESTIR_I["temporal_search_count"],
                   RESTIR_I["spatial_passes"], RESTIR_I["spatial_neighbors"], RESTIR_I["m_cap"],
                   RESTIR_I["use_confidence_weights"], RESTIR_I["bias_correction_visibility"]], np.int32)
    sf = np.array([RESTIR_F["temporal_search_radius"], RESTIR_F["spatial_radius"], RESTIR_F["normal_similarity_cos"],
                   RESTIR_F["plane_distance_threshold"], *cam, *prev_cam], np.float32)
    return si, sf


def main():
    pyoracle.build(ref=True)
    mesh, mat_of, raw, eff = scene()
    emission = raw[:, 4:7]
    emissive, prob, alias, s64 = light_table(mesh, mat_of, emission)
    sc = dict(soup=mesh.triangle_soup(), material_of=mat_of, emission=emission, emissive=emissive, alias_prob=prob,
              alias_idx=alias, power_sum=np.float32(s64))
    out = dict(positions=mesh.positions, indices=mesh.indices, material_of=mat_of, materials=raw, effective=eff,
               emissive=emissive, alias_prob=prob, alias_idx=alias, power_sum64=np.float64(s64))
    prev_gb = prev_final = None
    prev_iv = None
    for frame in range(2):
        iv, ip = camera(frame)
        cam = camera_pos(iv)
        pcam = camera_pos(prev_iv if prev_iv is not None else iv)
        vp = view_projection(prev_iv if prev_iv is not None else iv, ip)
        si, sf = settings_arrays(frame, 1 if frame > 0 else 0, cam, pcam)
        gb = pyoracle.restir_gbuffer(sc["soup"], mat_of, eff, W, H, SEED, frame, True, iv, ip)
        init = pyoracle.restir_pass(0, sc, eff, si, sf, vp, gb)
        temp = pyoracle.restir_pass(1, sc, eff, si, sf, vp, gb, gb_prev=prev_gb if prev_gb is not None else gb,
                                    inp=init, prev=prev_final)
        seed = pyoracle.restir_spatial_seed(frame, 0, SEED)
        final = pyoracle.restir_pass(2, sc, eff, si, sf, vp, gb, inp=temp, spatial_index=0, spatial_seed=seed)
        out.update({f"f{frame}_inverse_view": iv, f"f{frame}_inverse_projection": ip, f"f{frame}_gbuffer": gb,
                    f"f{frame}_initial": init, f"f{frame}_temporal": temp, f"f{frame}_final": final})
        valid = final[:, 7] > 0
        print(f"frame {frame}: hit {np.mean(gb[:, 3].view(np.int32) >= 0):.2f}, valid reservoirs {valid.mean():.2f}, "
              f"mean M {final[:, 5].view(np.int32).__rshift__(9).mean():.2f}")
        if frame == 0:
            recs = pyoracle.restir_presample(sc, 1, PRESAMPLE["presampling_subsets"],
                                             PRESAMPLE["presampling_subset_size"], frame, SEED)
            pi = (PRESAMPLE["presampling_subsets"], PRESAMPLE["presampling_subset_size"],
                  PRESAMPLE["presampling_tile_size"], pyoracle.restir_presample_seed(frame, SEED))
            out["ps_f0_initial"] = pyoracle.restir_pass(0, sc, eff, si, sf, vp, gb, presampled=recs, presample_i=pi)
        else:
            out["fused_f1"] = pyoracle.restir_pass(3, sc, eff, si, sf, vp, gb, gb_prev=prev_gb, inp=init,
                                                   prev=prev_final)
        prev_gb, prev_final, prev_iv = gb, final, iv
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
