"""GPU: gbpt_alias_table_build_noalloc, the light-table build for callers that cannot allocate
device memory (an interactive loop that must not stall on cudaMalloc/cudaFree after an emission
edit, or a host that gives the library a fixed memory budget). It must write the same table as the
light-table build inside gbpt_scene_create, from the same power list, with all of its scratch in a
fixed array inside the library. Calls in a row (3000 emitters, the maximum count, 700) check that
the shared scratch left by one call does not leak into the next, and that the maximum fills it
without overrunning its end. This file is named so that pytest collects it last."""
import numpy as np
import pytest
import torch

import gbpt
import pyoracle
from gbpt import render, scenes

pytestmark = pytest.mark.gpu


def _emitter_scene(n_emit, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    hf = scenes.heightfield(cells=16, amplitude=0.2, seed=seed)
    em = scenes.random_triangles(n_emit, seed=seed + 1, lo=(-0.8, 0.35, -0.8), hi=(0.8, 0.9, 0.8), sigma=0.05)
    mesh = scenes.merge(hf, em)
    mat_of = np.concatenate([np.zeros(hf.n_triangles, np.int32), 1 + np.arange(n_emit, dtype=np.int32)])
    albedo = np.full((n_emit + 1, 3), 0.5, np.float32)
    rad = np.exp(rng.uniform(0, np.log(1000), n_emit))
    emission = np.concatenate([[[0, 0, 0]], rad[:, None] * rng.uniform(0.2, 1.0, (n_emit, 3))]).astype(np.float32)
    return mesh, mat_of, albedo, emission


def _noalloc(lib, power_dev, n, stream):
    probas = torch.full((max(n, 1),), -1.0, dtype=torch.float32, device=power_dev.device)
    alias = torch.full((max(n, 1),), -7, dtype=torch.int32, device=power_dev.device)
    sum64 = torch.zeros(1, dtype=torch.float64, device=power_dev.device)
    st = lib.gbpt_alias_table_build_noalloc(power_dev.data_ptr(), n, probas.data_ptr(), alias.data_ptr(),
                                            sum64.data_ptr(), stream.cuda_stream)
    assert st == 0, lib.gbpt_last_error()
    stream.synchronize()
    return probas[:n].cpu().numpy(), alias[:n].cpu().numpy(), float(sum64.item())


def test_noalloc_alias_table_matches_scene_light_table(cuda, oracle):
    lib = render._load()
    stream = torch.cuda.Stream()
    # two different scenes, one call each, back to back: the second call runs on scratch that
    # still holds the first call's (larger) table
    for n_emit, seed in ((3000, 11), (700, 12)):
        mesh, mat_of, albedo, emission = _emitter_scene(n_emit, seed)
        scene = gbpt.Scene(mesh.positions, mesh.indices, mat_of, albedo, emission)
        want = scene.light_table()
        power = pyoracle.emissive_power(mesh.triangle_soup(), mat_of, emission, want["emissive"])
        power_dev = torch.from_numpy(power).to(cuda)
        prob, alias, s64 = _noalloc(lib, power_dev, len(power), stream)
        assert s64 == want["power_sum64"]
        assert np.array_equal(prob, want["probas"])
        assert np.array_equal(alias, want["alias"])
        scene.destroy()
        if n_emit == 3000:
            # the maximum count between the two scenes: the queues fill the fixed array to its end
            n = gbpt.render.GBPT_ALIAS_NOALLOC_MAX_EMITTERS
            rng = np.random.Generator(np.random.PCG64(13))
            big = np.exp(rng.uniform(0.0, np.log(1.0e4), n)).astype(np.float32)
            prob, alias, s64 = _noalloc(lib, torch.from_numpy(big).to(cuda), n, stream)
            assert abs(s64 - float(np.sum(big.astype(np.float64)))) <= 1e-12 * s64
            want_p, want_a = pyoracle.vose_alias(big, s64)
            assert np.array_equal(prob, want_p) and np.array_equal(alias, want_a)


def test_noalloc_rejects_oversized_and_empty(cuda):
    lib = render._load()
    big = gbpt.render.GBPT_ALIAS_NOALLOC_MAX_EMITTERS + 1
    assert lib.gbpt_alias_table_build_noalloc(None, big, None, None, None, None) == 1
    assert b"exceeds the no-allocation maximum" in lib.gbpt_last_error()
    assert lib.gbpt_alias_table_build_noalloc(None, 0, None, None, None, None) == 0
