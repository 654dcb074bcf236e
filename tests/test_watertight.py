"""CPU: the watertight triangle test (Woop, Benthin and Wald 2013), host build of the traversal
core the CUDA kernels compile, against the reference's Moller-Trumbore (the parity mode).

* Watertightness: near-vertical rays aimed at the interior edges and vertices of a height-field
  surface never pass through it with the watertight test; Moller-Trumbore lets some through.
* Agreement: on a scene of random and heightfield triangles the two tests give the same closest
  hit, with t/u/v equal to float rounding, except rays that pass within a rounding of an edge
  (the two tests may pick either neighbour, or only one of them finds a hit), grazing hits on
  small triangles that the reference's test rejects as parallel (its determinant epsilon,
  src/Renderer/Triangle.h:22-31) and exact ties; every disagreement is classified
  (gbpt.trace.classify_hit_differences) and no other kind is allowed.
"""
import numpy as np

from gbpt import scenes
from gbpt.trace import classify_hit_differences
from native.emu import EmuBVH


def _rays(origins, targets, last=-1):
    d = targets - origins
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    o4 = np.concatenate([origins, np.zeros((len(origins), 1))], axis=1).astype(np.float32)
    d4 = np.concatenate([d, np.full((len(d), 1), np.inf)], axis=1).astype(np.float32)
    return scenes.RayBatch(o4, d4, np.full(len(d), last, np.int32))


def _edge_targets(mesh, cells):
    """Points on every interior edge of the heightfield grid (midpoints and vertices)."""
    n = cells + 1
    pos = mesh.positions.astype(np.float64).reshape(n, n, 3)
    inner = pos[1:-1, 1:-1].reshape(-1, 3)  # interior vertices (shared by six triangles)
    h = 0.5 * (pos[1:-1, :-1] + pos[1:-1, 1:])  # horizontal edge midpoints away from the border rows
    v = 0.5 * (pos[:-1, 1:-1] + pos[1:, 1:-1])
    d = 0.5 * (pos[:-1, 1:] + pos[1:, :-1])  # the diagonals the two triangles of a cell share
    d = d[1:-1, 1:-1]
    return np.concatenate([inner, h[:, 1:-1].reshape(-1, 3), v[1:-1].reshape(-1, 3), d.reshape(-1, 3)])


def test_watertight_test_closes_shared_edges():
    cells = 48
    mesh = scenes.heightfield(cells=cells, amplitude=0.2, seed=5)
    targets = _edge_targets(mesh, cells)
    rng = np.random.default_rng(1)
    misses = {"mt": 0, "wt": 0}
    bvh = EmuBVH(mesh)
    for _ in range(4):
        # origins above the points, rays nearly straight down: each crosses the height field
        # exactly once (a grazing ray could touch it at a silhouette vertex without crossing)
        up = np.concatenate([rng.normal(scale=1e-3, size=(len(targets), 1)), np.ones((len(targets), 1)),
                             rng.normal(scale=1e-3, size=(len(targets), 1))], axis=1)
        origins = targets + 2.0 * up / np.linalg.norm(up, axis=1, keepdims=True)
        rays = _rays(origins, targets)
        mt, _ = bvh.trace(rays)
        wt, _ = bvh.trace(rays, watertight=True)
        misses["mt"] += int((mt[:, 3].view(np.int32) < 0).sum())
        misses["wt"] += int((wt[:, 3].view(np.int32) < 0).sum())
    assert misses["wt"] == 0, misses
    print(f"rays through {4 * len(targets)} interior edge / vertex points: Moller-Trumbore misses "
          f"{misses['mt']}, watertight misses 0")


def classify(mesh, rays, mt, wt):
    c = classify_hit_differences(mesh, rays, mt, wt)
    return c["agree"], c["edge"], c["parallel"], c["tie"], c["other"]


def test_watertight_agrees_with_moller_trumbore_away_from_edges():
    mesh = scenes.traversal_scene(cells=96, n_random=3000, seed=4)
    rays = scenes.pinhole_rays(256, 128, eye=(0.0, 1.5, -2.5), target=(0.0, 0.0, 0.0), vfov_deg=30.0)
    bvh = EmuBVH(mesh)
    mt, _ = bvh.trace(rays)
    wt, _ = bvh.trace(rays, watertight=True)
    agree, edge, parallel, tie, other = classify(mesh, rays, mt, wt)
    assert other == 0, (agree, edge, parallel, tie, other)
    assert agree >= 0.99 * len(rays), (agree, edge, tie)
    # any-hit decisions: a disagreement needs a hit near an edge
    so, _ = bvh.trace(rays, any_hit=True)
    sw, _ = bvh.trace(rays, any_hit=True, watertight=True)
    assert ((so[:, 3].view(np.int32) >= 0) != (sw[:, 3].view(np.int32) >= 0)).sum() <= edge + parallel + tie
