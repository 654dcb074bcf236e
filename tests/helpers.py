"""Shared test helpers: fixture loading and the tie/edge classifier for hit-ID mismatches."""
import os

import numpy as np

from conftest import GOLDEN
from gbpt import scenes


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, f"trace_{name}.npz"))
    mesh = scenes.Mesh(z["positions"], z["indices"])
    closest = scenes.RayBatch(z["c_origin_tmin"], z["c_dir_tmax"], z["c_last_prim"])
    shadow = scenes.RayBatch(z["s_origin_tmin"], z["s_dir_tmax"], z["s_last_prim"])
    return mesh, closest, z["c_hits"], shadow, z["s_light_dist"], z["s_occluded"]


def classify_mismatches(oracle, mesh, rays, got, want):
    """Compares closest-hit records. Returns (n_mismatch, n_ties, n_other). A mismatch is a tie
    when the Moller-Trumbore test of both candidate triangles gives the same t (bit-equal):
    the reference keeps the first one found in its traversal order, these kernels keep the
    lowest primitive index."""
    gp, wp = got[:, 3].view(np.int32), want[:, 3].view(np.int32)
    bad = np.nonzero((got.view(np.uint32) != want.view(np.uint32)).any(axis=1))[0]
    soup = mesh.triangle_soup()
    ties = 0
    for i in bad:
        if gp[i] < 0 or wp[i] < 0:
            continue
        ok_g, tg = oracle.mt(soup[gp[i]], rays.origin_tmin[i, :3], rays.dir_tmax[i, :3])
        ok_w, tw = oracle.mt(soup[wp[i]], rays.origin_tmin[i, :3], rays.dir_tmax[i, :3])
        if ok_g and ok_w and tg[0] == tw[0] and got[i, 0] == want[i, 0]:
            ties += 1
    return len(bad), ties, len(bad) - ties
