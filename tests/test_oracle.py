"""CPU: the oracle restatement pinned against the reference's own code and its golden vectors."""
import numpy as np
import pytest

import pyoracle
from gbpt import scenes
from helpers import load_golden


@pytest.mark.parametrize("name", ["cornell", "terrain"])
def test_restatement_matches_reference_golden(oracle, name):
    """Golden vectors come from the reference's BVH::intersect / evaluate_shadow_ray_occluded."""
    mesh, closest, c_hits, shadow, light_dist, s_occ = load_golden(name)
    oc = oracle.octree(mesh.triangle_soup())
    got = oc.closest(closest)
    assert np.array_equal(got.view(np.uint32), c_hits.view(np.uint32))
    occ = oc.occluded(shadow)
    assert np.array_equal(occ, s_occ)
    # the shadow batch's tmax is the reference's own 't_max - 1e-4' in float32
    assert np.array_equal(shadow.dir_tmax[:, 3], (light_dist - np.float32(1e-4)).astype(np.float32))


@pytest.mark.parametrize("name", ["cornell", "terrain"])
def test_brute_force_agrees_up_to_ties(oracle, name):
    """Exhaustive Moller-Trumbore (lowest-index tie rule) vs the reference's first-found rule."""
    from helpers import classify_mismatches
    mesh, closest, c_hits, *_ = load_golden(name)
    got = oracle.brute_closest(mesh.triangle_soup(), closest)
    n, ties, other = classify_mismatches(oracle, mesh, closest, got, c_hits)
    assert other == 0, f"{other} non-tie mismatches of {n}"


@pytest.mark.skipif(not pyoracle.ref_available(), reason="reference build (oracle/_ref) not present")
def test_restatement_matches_reference_live():
    """Live comparison on a fresh seed (only where the reference tree was compiled)."""
    orc = pyoracle.Oracle()
    mesh = scenes.traversal_scene(cells=64, n_random=3000, seed=9)
    soup = mesh.triangle_soup()
    ref = pyoracle.RefBVH(soup)
    oc = orc.octree(soup)
    rays = scenes.pinhole_rays(128, 64, vfov_deg=30)
    h_ref, h_orc = ref.closest(rays), oc.closest(rays)
    assert np.array_equal(h_ref.view(np.uint32), h_orc.view(np.uint32))
    pts, nrm, prim = scenes.hit_points_normals(mesh, rays, h_ref)
    m = prim >= 0
    s, ld = scenes.shadow_rays(pts[m], prim[m], seed=7)
    assert np.array_equal(ref.shadow_occluded(s, ld), oc.occluded(s))


def test_mt_known_answers(oracle):
    """Moller-Trumbore edge cases of src/Renderer/Triangle.h:20-63."""
    tri = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    ok, tuv = oracle.mt(tri, [0.25, 0.25, -1], [0, 0, 1])
    assert ok and tuv[0] == 1.0 and tuv[1] == 0.25 and tuv[2] == 0.25
    ok, _ = oracle.mt(tri, [0.25, 0.25, -1], [1, 0, 0])  # parallel
    assert not ok
    ok, _ = oracle.mt(tri, [0.25, 0.25, 1], [0, 0, 1])  # behind the origin
    assert not ok
    ok, tuv = oracle.mt(tri, [0.0, 0.0, -1], [0, 0, 1])  # exactly on a vertex: u = v = 0 accepted
    assert ok and tuv[1] == 0.0 and tuv[2] == 0.0
    ok, _ = oracle.mt(tri, [0.6, 0.6, -1], [0, 0, 1])  # u + v > 1
    assert not ok
