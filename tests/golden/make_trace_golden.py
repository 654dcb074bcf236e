"""Generates tests/golden/trace_*.npz from the REFERENCE's own CPU intersection code.

Runs oracle/_ref/libref.so (the reference's src/Renderer/BVH.cpp + Triangle.h and
src/Device/includes/Intersect.h's shadow test, compiled behind clean-room shims by
`make -C oracle ref`) on seeded scenes and stores inputs and outputs:
  closest: rays -> hits (t, u, v, prim)         [BVH::intersect, src/Renderer/BVH.h:132-223]
  shadow:  rays + light distance -> occluded   [evaluate_shadow_ray_occluded, Intersect.h:276-324]
Usage (where the reference tree is present):  python tests/golden/make_trace_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "hiprt-path-tracer_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from gbpt import scenes  # noqa: E402
import pyoracle  # noqa: E402


def make(name, mesh, width, height, eye, target, vfov, seed):
    ref = pyoracle.RefBVH(mesh.triangle_soup())
    prim_rays = scenes.pinhole_rays(width, height, eye=eye, target=target, vfov_deg=vfov)
    prim_hits = ref.closest(prim_rays)
    pts, nrm, prim = scenes.hit_points_normals(mesh, prim_rays, prim_hits)
    m = prim >= 0
    b = scenes.bounce_rays(pts[m], nrm[m], prim[m], seed=seed)
    b_hits = ref.closest(b)
    s, light_dist = scenes.shadow_rays(pts[m], prim[m], seed=seed + 1,
                                       centre=(float(target[0]), float(eye[1]) + 0.5, float(target[2])))
    s_occ = ref.shadow_occluded(s, light_dist)
    closest = scenes.RayBatch.concat([prim_rays, b])
    np.savez_compressed(os.path.join(HERE, f"trace_{name}.npz"),
                        positions=mesh.positions, indices=mesh.indices,
                        c_origin_tmin=closest.origin_tmin, c_dir_tmax=closest.dir_tmax, c_last_prim=closest.last_prim,
                        c_hits=np.concatenate([prim_hits, b_hits]),
                        s_origin_tmin=s.origin_tmin, s_dir_tmax=s.dir_tmax, s_last_prim=s.last_prim,
                        s_light_dist=light_dist, s_occluded=s_occ)
    print(name, mesh.n_triangles, "tris", len(closest), "closest rays", len(s), "shadow rays",
          "hit frac", float((prim_hits[:, 3].view(np.int32) >= 0).mean()))


if __name__ == "__main__":
    pyoracle.build(ref=True)
    cb = scenes.cornell_box()
    make("cornell", cb.mesh, 96, 96, (2.75, 2.75, -8.0), (2.75, 2.75, 0.0), 40.0, seed=11)
    make("terrain", scenes.traversal_scene(cells=48, n_random=1500, seed=5), 128, 64, (0.0, 1.5, -2.5),
         (0.0, 0.0, 0.0), 30.0, seed=12)
