"""Generates tests/golden/ref_restir_cornell.npz: ReSTIR DI frames rendered by the REFERENCE's own
CPU kernels (oracle/ref_render.cpp built with REF_DIRECT = LSS_RESTIR_DI, `make -C oracle ref`):
CameraRays, ReSTIR_DI_InitialCandidates, ReSTIR_DI_TemporalReuse, ReSTIR_DI_SpatialReuse and the
MegaKernel's ReSTIR DI final shading, in the reference GPU renderer's pass order, with its
per-pass random numbers (the renderer's Xorshift32 seeded with 42 gives one number to the
G-buffer pass, the initial candidates, two to the temporal pass (random number, permutation
bits), one per spatial pass and one to the MegaKernel; GPURenderer.cpp:750-751,
ReSTIRDIRenderPass.cpp:449-578, MegaKernelRenderPass.cpp:53).

Scene: the principled Cornell box (the materials of the principled golden image) with 16 small
emissive triangles of log-uniform radiance just below the ceiling, facing down. The camera looks
down into the box and sees neither the ceiling nor a light: the reference's light candidates get
a 0/0 weight (NaN) at a shading point behind a light's plane (a zero cosine at the light in the
solid-angle pdf of the MIS weight, InitialCandidates.h:229-248), so every camera hit lies below
every emitter. The camera orbits the box by half a degree per frame, so the temporal pass
backprojects. Per frame it stores the
camera, the random numbers, the frame's image and the reservoirs after the initial-candidates,
temporal and spatial passes (8 words per pixel: point xyz, target function, triangle,
(M << 9) | flags, weight sum, UCW).
Usage (where the reference tree is present):  python tests/golden/make_ref_restir_golden.py
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

OUT = os.path.join(HERE, "ref_restir_cornell.npz")
SIZE = 48
FRAMES = 4
N_EMIT = 16
RESTIR = dict(light_candidates=8, bsdf_candidates=1, do_temporal=1, temporal_search_count=8, temporal_search_radius=4,
              do_spatial=1, spatial_passes=1, spatial_neighbors=5, spatial_radius=8, m_cap=20,
              use_confidence_weights=1, normal_similarity_cos=0.906307787, plane_distance_threshold=0.1)


class Settings:
    def __init__(self, frame):
        self.width = self.height = SIZE
        self.nb_bounces = 3
        self.do_russian_roulette = True
        self.russian_roulette_min_depth = 3
        self.russian_roulette_throughput_clamp = 0.0
        self.do_jittering = True
        self.ris_light_candidates, self.ris_bsdf_candidates = 4, 1
        self.inverse_view, self.inverse_projection = camera(frame)


def camera(frame):
    """A camera looking down into the box (no ceiling or light in view: every camera hit lies
    below every emitter's plane), orbiting the box's vertical axis by half a degree per frame."""
    a = math.radians(0.5 * frame)
    cx, cz = 2.75, 2.75
    ex, ez = 0.0, -6.0 - cz
    eye = (cx + ex * math.cos(a) - ez * math.sin(a), 3.2, cz + ex * math.sin(a) + ez * math.cos(a))
    return look_at_camera(eye, (2.75, 1.2, 2.75), vfov_deg=30.0, aspect=1.0)


def view_projection(iv, ip):
    """World -> NDC of a camera given its inverse view and inverse projection (row-major)."""
    prod = np.asarray(iv, np.float64).reshape(4, 4) @ np.asarray(ip, np.float64).reshape(4, 4)
    return np.linalg.inv(prod).astype(np.float32)


def scene():
    """Principled Cornell box plus N_EMIT ceiling emitters -> mesh, material per triangle, records."""
    cb = scenes.cornell_box()
    rng = np.random.Generator(np.random.PCG64(21))
    tris = []
    for _ in range(N_EMIT):
        x, z = rng.uniform(0.3, 4.9, 2)
        s = rng.uniform(0.15, 0.35)
        y = 5.48
        tris.append([(x, y, z), (x + s, y, z), (x + s, y, z + s)])  # normal -y
    pos = np.asarray(tris, np.float32).reshape(-1, 3)
    em = scenes.Mesh(pos, np.arange(3 * N_EMIT, dtype=np.int32).reshape(-1, 3))
    mesh = scenes.merge(cb.mesh, em)
    mat_of = np.concatenate([cb.material_of_triangle.copy(), len(MATERIALS) + np.arange(N_EMIT, dtype=np.int32)])
    mat_of[10:22] = 4
    mat_of[22:34] = 5
    mats = list(MATERIALS)
    rad = np.exp(rng.uniform(0.0, math.log(40.0), N_EMIT))
    for k in range(N_EMIT):
        col = rng.uniform(0.3, 1.0, 3)
        mats.append(dict(base_color=(0.0, 0.0, 0.0), emission=tuple(float(v) for v in rad[k] * col)))
    return mesh, mat_of.astype(np.int32), M.pack_many(mats)


def pass_random_numbers(frames, restir=RESTIR, seed=42):
    """Per frame, the passes' random numbers in launch order (see the module docstring)."""
    n = 2 + (2 if restir["do_temporal"] else 0) + (restir["spatial_passes"] if restir["do_spatial"] else 0) + 1 - 1
    x, out = seed, []
    for _ in range(frames):
        row = []
        for _ in range(n + 1):
            x = pyoracle.xorshift32(x)
            row.append(x)
        out.append(row)
    return np.asarray(out, np.uint32)


def main():
    pyoracle.build(ref=True)
    mesh, mat_of, raw = scene()
    r = pyoracle.RefRestir(SIZE, SIZE, mesh.positions, mesh.indices, mat_of, raw)
    rn = pass_random_numbers(FRAMES)
    out = dict(size=np.int32(SIZE), frames=np.int32(FRAMES), positions=mesh.positions, indices=mesh.indices,
               material_of=mat_of, materials=raw, random_numbers=rn,
               restir_i=np.array([RESTIR[k] for k in ("light_candidates", "bsdf_candidates", "do_temporal",
                                                     "temporal_search_count", "temporal_search_radius", "do_spatial",
                                                     "spatial_passes", "spatial_neighbors", "spatial_radius", "m_cap",
                                                     "use_confidence_weights")], np.int32),
               restir_f=np.array([RESTIR["normal_similarity_cos"], RESTIR["plane_distance_threshold"]], np.float32))
    keys = ("image", "initial", "temporal", "final", "prim", "pos")
    acc = {k: [] for k in keys}
    ivs, ips = [], []
    prev_iv = None
    for f in range(FRAMES):
        st = Settings(f)
        iv, ip = st.inverse_view, st.inverse_projection
        piv = prev_iv if prev_iv is not None else iv
        o = r.frame(st, RESTIR, f, rn[f], piv, view_projection(piv, ip))
        for k in keys:
            acc[k].append(o[k])
        ivs.append(np.asarray(iv, np.float32).reshape(16))
        ips.append(np.asarray(ip, np.float32).reshape(16))
        prev_iv = iv
        m = o["final"][:, 5].view(np.int32) >> 9
        print(f"frame {f}: image mean {o['image'].mean():.5f}, final M mean {m.mean():.2f}, "
              f"UCW > 0 {np.mean(o['final'][:, 7] > 0):.3f}")
    for k in keys:
        out[k] = np.stack(acc[k])
    out["inverse_view"], out["inverse_projection"] = np.stack(ivs), np.stack(ips)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes)")


if __name__ == "__main__":
    main()
