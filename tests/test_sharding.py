"""CPU: the multi-GPU sharding of the render path with world_size-2 gloo process groups. Each rank
renders its sample range with the oracle (the same PCG streams as the GPU kernels, seeded by pixel
and sample index); the all-reduced FP64 image equals the single-process render."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from gbpt import sharding


def test_sample_ranges_cover_every_launch_once():
    for n in (0, 1, 7, 64):
        for world in (1, 2, 3, 8):
            got = [sharding.sample_range(r, world, n) for r in range(world)]
            flat = [i for first, count in got for i in range(first, first + count)]
            assert flat == list(range(n))
            assert max(c for _, c in got) - min(c for _, c in got) <= 1
    with pytest.raises(ValueError):
        sharding.sample_range(2, 2, 10)


def test_job_assignment_balances_cost():
    rng = np.random.default_rng(0)
    costs = rng.uniform(1, 100, 48)
    parts = sharding.assign_jobs(costs, 4)
    assert sorted(j for p in parts for j in p) == list(range(48))
    loads = [costs[p].sum() for p in parts]
    assert max(loads) - min(loads) <= costs.max()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, n_launches, spp, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    import pyoracle
    import gbpt
    from gbpt import scenes
    cb = scenes.cornell_box()
    st = gbpt.cornell_settings(24, 24, samples_per_launch=spp, seed=3)
    lt = _light_table(cb)
    first, count = sharding.sample_range(rank, world, n_launches)
    img = pyoracle.pt_render(cb.mesh.triangle_soup(), cb.material_of_triangle, cb.albedo, cb.emission, lt[0], lt[1],
                             lt[2], lt[3], st, count * spp, iteration_base=first * spp, nthreads=2)
    total = sharding.reduce_image(img)
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), total)
    dist.barrier()
    dist.destroy_process_group()


def _light_table(cb):
    """Uniform light sampling needs only the emissive list (the alias arrays are unused)."""
    em = np.asarray(cb.emissive_triangles, np.int32)
    return em, np.ones(len(em), np.float32), np.arange(len(em), dtype=np.int32), 1.0


def test_two_rank_sample_sharding_reproduces_the_single_render(tmp_path, oracle):
    import pyoracle
    import gbpt
    from gbpt import scenes
    n_launches, spp, world = 5, 2, 2
    port = _free_port()
    mp.start_processes(_rank_main, args=(world, port, n_launches, spp, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    cb = scenes.cornell_box()
    st = gbpt.cornell_settings(24, 24, samples_per_launch=spp, seed=3)
    lt = _light_table(cb)
    full = pyoracle.pt_render(cb.mesh.triangle_soup(), cb.material_of_triangle, cb.albedo, cb.emission, lt[0], lt[1],
                              lt[2], lt[3], st, n_launches * spp, nthreads=2)
    for r in range(world):
        got = np.load(tmp_path / f"rank{r}.npy")
        np.testing.assert_allclose(got, full, rtol=1e-12, atol=1e-12)
    assert full.sum() > 0


def test_band_order_is_a_bijection_of_4x8_tiles():
    from gbpt import scenes
    for w, h in ((4096, 2048), (13, 11), (17, 23), (3, 5), (8, 8), (1, 1)):
        p = scenes.band_order(w, h)
        assert np.array_equal(np.sort(p), np.arange(w * h))
    p = scenes.band_order(64, 16)
    x, y = p % 64, p // 64
    for k in range(0, 64 * 16, 32):  # every 32 consecutive rays form a 4 x 8 tile
        assert x[k:k + 32].max() - x[k:k + 32].min() == 3 and y[k:k + 32].max() - y[k:k + 32].min() == 7
