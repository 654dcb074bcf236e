"""GPU: the CUDA traversal kernels through the C ABI against the oracle and the reference's
golden vectors. Closest-hit records must be bit-identical (t, u, v, prim) except for exact ties
on t, which resolve to the lowest primitive index; shadow decisions must be identical."""
import numpy as np
import pytest
import torch

import gbpt
from gbpt import scenes
from helpers import classify_mismatches, load_golden

pytestmark = pytest.mark.gpu


def _dev(rays, device):
    return (torch.from_numpy(np.ascontiguousarray(rays.origin_tmin)).to(device),
            torch.from_numpy(np.ascontiguousarray(rays.dir_tmax)).to(device),
            torch.from_numpy(np.ascontiguousarray(rays.last_prim)).to(device))


def _closest(bvh, rays, device):
    o, d, lp = _dev(rays, device)
    h = bvh.closest(o, d, lp)
    torch.cuda.synchronize()
    return h.cpu().numpy()


def _occluded(bvh, rays, device):
    o, d, lp = _dev(rays, device)
    r = bvh.occluded(o, d, lp)
    torch.cuda.synchronize()
    return r.cpu().numpy()


@pytest.mark.parametrize("name", ["cornell", "terrain"])
def test_golden_closest_and_shadow(cuda, oracle, name):
    mesh, closest, c_hits, shadow, _, s_occ = load_golden(name)
    bvh = gbpt.BVH(mesh.indices, mesh.positions)
    got = _closest(bvh, closest, cuda)
    n, ties, other = classify_mismatches(oracle, mesh, closest, got, c_hits)
    assert other == 0, f"{other} non-tie mismatches of {n}"
    assert np.array_equal(_occluded(bvh, shadow, cuda), s_occ)


def test_random_scene_against_oracle(cuda, oracle):
    mesh = scenes.traversal_scene(cells=128, n_random=8000, seed=21)
    oc = oracle.octree(mesh.triangle_soup())
    bvh = gbpt.BVH(mesh.indices, mesh.positions)
    rays = scenes.pinhole_rays(256, 128, vfov_deg=30)
    want = oc.closest(rays)
    got = _closest(bvh, rays, cuda)
    n, ties, other = classify_mismatches(oracle, mesh, rays, got, want)
    assert other == 0, f"{other} non-tie mismatches of {n}"
    pts, nrm, prim = scenes.hit_points_normals(mesh, rays, want)
    m = prim >= 0
    b = scenes.bounce_rays(pts[m], nrm[m], prim[m], seed=5)
    n, ties, other = classify_mismatches(oracle, mesh, b, _closest(bvh, b, cuda), oc.closest(b))
    assert other == 0
    s, _ = scenes.shadow_rays(pts[m], prim[m], seed=6)
    assert np.array_equal(_occluded(bvh, s, cuda), oc.occluded(s))


def test_matches_host_emulation_bits(cuda):
    """The CUDA build and the host build of the same traversal source agree bit for bit."""
    from native.emu import EmuBVH
    mesh = scenes.traversal_scene(cells=96, n_random=4000, seed=8)
    rays = scenes.pinhole_rays(192, 96, vfov_deg=35)
    got = _closest(gbpt.BVH(mesh.indices, mesh.positions), rays, cuda)
    want, _ = EmuBVH(mesh).trace(rays)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_host_buffer_entry_points_match_device(cuda):
    mesh, closest, c_hits, shadow, _, s_occ = load_golden("terrain")
    bvh = gbpt.BVH(mesh.indices, mesh.positions)
    dev = _closest(bvh, closest, cuda)
    host = bvh.closest_host(np.ascontiguousarray(closest.origin_tmin), np.ascontiguousarray(closest.dir_tmax),
                            np.ascontiguousarray(closest.last_prim))
    assert np.array_equal(dev.view(np.uint32), host.view(np.uint32))
    occ = bvh.occluded_host(np.ascontiguousarray(shadow.origin_tmin), np.ascontiguousarray(shadow.dir_tmax),
                            np.ascontiguousarray(shadow.last_prim))
    assert np.array_equal(occ, s_occ)


def test_count_kernel_matches_emulation(cuda):
    from native.emu import EmuBVH
    mesh = scenes.traversal_scene(cells=64, n_random=2000, seed=4)
    rays = scenes.pinhole_rays(128, 64, vfov_deg=30)
    bvh = gbpt.BVH(mesh.indices, mesh.positions)
    o, d, lp = _dev(rays, cuda)
    nodes, tris = bvh.count(o, d, lp)
    _, cnt = EmuBVH(mesh).trace(rays)
    assert (nodes, tris) == (int(cnt[0]), int(cnt[1]))


def test_empty_and_zero_rays(cuda):
    bvh = gbpt.BVH(np.zeros((0, 3), np.int32), np.zeros((0, 3), np.float32))
    rays = scenes.pinhole_rays(16, 8)
    got = _closest(bvh, rays, cuda)
    assert (got[:, 3].view(np.int32) == -1).all()
    o, d, lp = _dev(rays.slice(slice(0, 0)), cuda)
    assert bvh.closest(o, d, lp).shape == (0, 4)


def test_full_size_scene_sampled(cuda, oracle):
    """The benchmark scene at full size (2,297,152 triangles): strided samples of primary, bounce
    (closest hit) and shadow (any hit) rays against the oracle, the secondary rays generated from
    the primary hits as the benchmark does (cosine bounces off the hit normal, shadow rays to an
    area light), plus size-independent properties over the whole batch."""
    mesh = scenes.traversal_scene()
    assert mesh.n_triangles == 2_297_152
    bvh = gbpt.BVH(mesh.indices, mesh.positions)
    st = bvh.stats()
    assert st["n_bvh_triangles"] == mesh.n_triangles and st["wide_depth"] < 48
    rays = scenes.pinhole_rays(1024, 512, vfov_deg=30)
    got = _closest(bvh, rays, cuda)
    sample = rays.slice(slice(0, None, 97))
    oc = oracle.octree(mesh.triangle_soup())
    n, ties, other = classify_mismatches(oracle, mesh, sample, got[::97], oc.closest(sample))
    assert other == 0, f"{other} non-tie mismatches of {n}"
    prim = got[:, 3].view(np.int32)
    hit = prim >= 0
    assert (got[hit, 0] > 0).all() and (prim < mesh.n_triangles).all()
    # determinism: a second launch returns identical bits
    assert np.array_equal(got.view(np.uint32), _closest(bvh, rays, cuda).view(np.uint32))
    pts, nrm, prims = scenes.hit_points_normals(mesh, rays, got)
    m = np.nonzero(prims >= 0)[0]
    b = scenes.bounce_rays(pts[m], nrm[m], prims[m], seed=3)
    gb = _closest(bvh, b, cuda)
    bs = b.slice(slice(0, None, 41))
    n, ties, other = classify_mismatches(oracle, mesh, bs, gb[::41], oc.closest(bs))
    assert other == 0, f"bounce: {other} non-tie mismatches of {n}"
    sh, _ = scenes.shadow_rays(pts[m], prims[m], seed=4)
    occ = _occluded(bvh, sh, cuda)
    ss = sh.slice(slice(0, None, 41))
    assert np.array_equal(occ[::41], oc.occluded(ss))
    assert 0.05 < occ.mean() < 0.95


@pytest.mark.parametrize("any_hit", [False, True])
def test_every_launch_configuration_gives_identical_results(cuda, any_hit):
    """Per-ray and persistent kernels over block sizes, refill / postpone thresholds, shared-memory
    stack depths and the top BVH levels in shared memory return the same hits bit for bit
    (the closest hit does not depend on the visiting order), and the autotuner returns a valid
    configuration whose results are again identical."""
    mesh, closest, _, shadow, _, _ = load_golden("terrain")
    bvh = gbpt.BVH(mesh.indices, mesh.positions)
    rays = shadow if any_hit else closest
    o, d, lp = _dev(rays, cuda)
    run = bvh.occluded_cfg if any_hit else bvh.closest_cfg
    base = run(o, d, lp, kernel=1, block=128).cpu().numpy()
    configs = [dict(kernel=1, block=b, shared_stack=sh) for b in (32, 64, 256) for sh in (0, 8, 16)]
    configs += [dict(kernel=2, block=b, refill_below=r, postpone_below=p, blocks_per_sm=s, shared_stack=sh)
                for b, r, p, s in [(128, 12, 8, 8), (64, 1, 0, 2), (256, 32, 32, 16), (128, 4, 24, 1), (32, 20, 4, 64)]
                for sh in (0, 8, 16)]
    configs += [dict(kernel=3, block=b, blocks_per_sm=s, shared_stack=sh)
                for b, s in [(128, 8), (256, 4), (32, 64), (64, 1)] for sh in (0, 8, 16)]
    # the top levels of the BVH staged in shared memory, in every kernel
    configs += [dict(c, top_levels=1) for c in configs if c.get("shared_stack", 0) == 0]
    for cfg in configs:
        got = run(o, d, lp, **cfg).cpu().numpy()
        assert np.array_equal(got.view(np.uint8), base.view(np.uint8)), cfg
    best, ms = bvh.autotune(o, d, lp, any_hit=any_hit)
    assert ms > 0 and best["kernel"] in (1, 2, 3) and bvh.trace_config(any_hit) == best
    got = (bvh.occluded if any_hit else bvh.closest)(o, d, lp).cpu().numpy()
    assert np.array_equal(got.view(np.uint8), base.view(np.uint8))


def test_trace_config_validation(cuda):
    from gbpt import GbptError
    mesh, *_ = load_golden("cornell")
    bvh = gbpt.BVH(mesh.indices, mesh.positions)
    for bad in (dict(kernel=4), dict(block=96), dict(refill_below=0), dict(postpone_below=33), dict(blocks_per_sm=0),
                dict(shared_stack=4), dict(shared_stack=-8), dict(top_levels=2), dict(top_levels=1, shared_stack=8)):
        with pytest.raises(GbptError):
            bvh.set_trace_config(False, **bad)


@pytest.mark.parametrize("any_hit", [False, True])
def test_watertight_kernels_match_host_build_and_autotune(cuda, any_hit):
    """The watertight triangle test in every kernel variant returns, bit for bit, what the host build
    of the same traversal core returns; the autotuner keeps the triangle test it is given."""
    import sys
    sys.path.insert(0, __file__.rsplit("/", 1)[0])
    from native.emu import EmuBVH
    mesh = scenes.traversal_scene(cells=96, n_random=3000, seed=4)
    rays = scenes.pinhole_rays(256, 128, eye=(0.0, 1.5, -2.5), target=(0.0, 0.0, 0.0), vfov_deg=30.0)
    if any_hit:
        pts, _, prim = scenes.hit_points_normals(mesh, rays, EmuBVH(mesh).trace(rays)[0])
        m = prim >= 0
        rays, _ = scenes.shadow_rays(pts[m], prim[m], seed=6)
    want, _ = EmuBVH(mesh).trace(rays, any_hit=any_hit, watertight=True)
    bvh = gbpt.BVH(mesh.indices, mesh.positions)
    o, d, lp = _dev(rays, cuda)
    run = bvh.occluded_cfg if any_hit else bvh.closest_cfg
    for cfg in (dict(kernel=1, block=128), dict(kernel=1, block=64, shared_stack=8),
                dict(kernel=2, block=128, refill_below=12, postpone_below=8, blocks_per_sm=8, shared_stack=16),
                dict(kernel=3, block=256, blocks_per_sm=4)):
        got = run(o, d, lp, triangle_test=1, **cfg).cpu().numpy()
        if any_hit:
            assert np.array_equal(got, (want[:, 3].view(np.int32) >= 0).astype(np.uint8)), cfg
        else:
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), cfg
    bvh.set_trace_config(any_hit, triangle_test=1)
    best, _ = bvh.autotune(o, d, lp, any_hit=any_hit)
    assert best["triangle_test"] == 1


def test_watertight_against_moller_trumbore_on_benchmark_scene(cuda):
    """The traversal benchmark scene (2,297,152 triangles): Moller-Trumbore (parity) and watertight
    closest hits of 2M primary rays and of bounce rays; every disagreement is a ray within a
    rounding of an edge or an exact tie (classified as in tests/test_watertight.py)."""
    import sys
    sys.path.insert(0, __file__.rsplit("/", 1)[0])
    from test_watertight import classify
    mesh = scenes.traversal_scene()
    bvh = gbpt.BVH(mesh.indices, mesh.positions)
    rays = scenes.pinhole_rays(2048, 1024, vfov_deg=30)
    o, d, lp = _dev(rays, cuda)
    mt = bvh.closest_cfg(o, d, lp, kernel=1, block=128).cpu().numpy()
    wt = bvh.closest_cfg(o, d, lp, kernel=1, block=128, triangle_test=1).cpu().numpy()
    agree, edge, parallel, tie, other = classify(mesh, rays, mt, wt)
    assert other == 0, (agree, edge, parallel, tie, other)
    assert agree >= 0.999 * len(rays), (agree, edge, tie)
    pts, nrm, prim = scenes.hit_points_normals(mesh, rays, mt)
    m = np.nonzero(prim >= 0)[0][::4]
    b = scenes.bounce_rays(pts[m], nrm[m], prim[m], seed=9)
    o, d, lp = _dev(b, cuda)
    mt = bvh.closest_cfg(o, d, lp, kernel=1, block=128).cpu().numpy()
    wt = bvh.closest_cfg(o, d, lp, kernel=1, block=128, triangle_test=1).cpu().numpy()
    agree, edge, parallel, tie, other = classify(mesh, b, mt, wt)
    assert other == 0, (agree, edge, parallel, tie, other)
