"""GPU: batched rendering. Jobs with different scenes, resolutions, bounce depths, seeds and sample
counts share every wavefront launch; each job's image must equal, bit for bit, the image of a
single renderer tracing the same pixel samples (a path depends only on its scene, pixel, sample
index and seed), with and without the CUDA graph; and each job's image agrees sample by sample
with the path-tracing oracle's rendering of that job (same PCG streams; the principled jobs
shaded by the library's BSDF built for the host, which the BSDF golden vectors pin to the
reference's), to the tolerance of the single-renderer oracle tests."""
import os

import numpy as np
import pytest
import torch

import gbpt
from gbpt import materials as M, scenes
from gbpt.render import BSDF_PRINCIPLED, LIGHT_POWER, RenderSettings, look_at_camera

pytestmark = pytest.mark.gpu


def _single(scene, st):
    """The reference image: one renderer, one sample per launch, st.samples_per_launch launches."""
    one = RenderSettings(**{**st.__dict__, "samples_per_launch": 1})
    r = gbpt.Renderer(scene, one)
    r.render(st.samples_per_launch)
    torch.cuda.synchronize()
    return r.image_sums()


def _lambert_jobs(with_oracle=False):
    cb = scenes.cornell_box()
    scene = gbpt.Scene.from_cornell(cb)
    if with_oracle:
        return cb, _lambert_jobs()
    return [(scene, gbpt.cornell_settings(48, 32, samples_per_launch=9, nb_bounces=4, seed=3)),
            (scene, gbpt.cornell_settings(17, 23, samples_per_launch=4, nb_bounces=2, seed=8)),
            (scene, gbpt.cornell_settings(64, 64, samples_per_launch=13, nb_bounces=7, seed=1))]


def _principled_jobs(with_oracle=False):
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pt_principled_cornell.npz"))
    w, h, _, nb, rr, _ = (int(v) for v in g["settings"])
    cornell = gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=g["materials"])
    jobs = [(cornell, RenderSettings(width=w, height=h, samples_per_launch=6, nb_bounces=nb, russian_roulette_min_depth=rr,
                                     bsdf=BSDF_PRINCIPLED, seed=4, inverse_view=g["inverse_view"],
                                     inverse_projection=g["inverse_projection"]))]
    # a heightfield with emitters above it and random principled materials
    rng = np.random.default_rng(2)
    hf = scenes.heightfield(cells=32, amplitude=0.2, seed=5)
    em = scenes.random_triangles(40, seed=6, lo=(-0.8, 0.4, -0.8), hi=(0.8, 0.9, 0.8), sigma=0.06)
    mesh = scenes.merge(hf, em)
    mats = M.pack_many(M.random_principled(rng, 4) + [dict(base_color=(0, 0, 0), emission=(30.0, 25.0, 20.0))])
    mat_of = np.concatenate([rng.integers(0, 4, hf.n_triangles), np.full(40, 4)]).astype(np.int32)
    hscene = gbpt.Scene(mesh.positions, mesh.indices, mat_of, principled=mats)
    iv, ip = look_at_camera((0.0, 1.2, -2.2), (0.0, 0.1, 0.0), vfov_deg=45.0, aspect=40 / 24)
    jobs.append((hscene, RenderSettings(width=40, height=24, samples_per_launch=11, nb_bounces=5, light_sampling=LIGHT_POWER,
                                        bsdf=BSDF_PRINCIPLED, seed=9, inverse_view=iv, inverse_projection=ip)))
    if with_oracle:
        # per job: triangle soup, material per triangle, raw records
        return [(g["positions"][g["indices"]].reshape(-1, 9), g["material_of"], g["materials"]),
                (mesh.triangle_soup(), mat_of, mats)], jobs
    return jobs


@pytest.mark.parametrize("kind", ["lambert", "principled"])
@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_jobs_equal_single_renders(cuda, kind, use_graph):
    jobs = _lambert_jobs() if kind == "lambert" else _principled_jobs()
    b = gbpt.Batch(jobs, samples_per_iteration=4, use_graph=use_graph)
    b.render()
    torch.cuda.synchronize()
    for k, (scene, st) in enumerate(jobs):
        got32, got64 = b.image_sums(k)
        want32, want64 = _single(scene, st)
        assert np.array_equal(got32, want32), k
        assert np.array_equal(got64, want64), k
    st = b.stats()
    assert st["samples"] == sum(s.width * s.height * s.samples_per_launch for _, s in jobs)
    assert st["extension_rays"] >= st["samples"]
    # a second render starts from zero and gives the same images
    b.render()
    torch.cuda.synchronize()
    assert np.array_equal(b.image_sums(0)[0], _single(*jobs[0])[0])


def _close_to_oracle(gpu, orc, min_close):
    rel = np.abs(gpu - orc) / np.maximum(np.abs(orc), 1e-3)
    close = rel.max(axis=-1) < 1e-3
    assert close.mean() > min_close, close.mean()
    assert abs(gpu[close].mean() - orc[close].mean()) / orc[close].mean() < 1e-4


def test_batch_jobs_match_oracle(cuda):
    import pyoracle
    cb, jobs = _lambert_jobs(with_oracle=True)
    b = gbpt.Batch(jobs, samples_per_iteration=4)
    b.render()
    torch.cuda.synchronize()
    for k, (scene, st) in enumerate(jobs):
        lt = scene.light_table()
        orc = pyoracle.pt_render(cb.mesh.triangle_soup(), cb.material_of_triangle, cb.albedo, cb.emission,
                                 lt["emissive"], lt["probas"], lt["alias"], lt["power_sum"], st, st.samples_per_launch)
        _close_to_oracle(b.image_sums(k)[1], orc, 0.97)
    data, jobs = _principled_jobs(with_oracle=True)
    b = gbpt.Batch(jobs, samples_per_iteration=4)
    b.render()
    torch.cuda.synchronize()
    for k, ((scene, st), (soup, mat_of, raw)) in enumerate(zip(jobs, data)):
        lt = scene.light_table()
        eff = M.pack_many([M.coat_roughened(M.unpack(m)) for m in raw])
        orc = pyoracle.pt_render_principled(np.ascontiguousarray(soup, np.float32), mat_of, eff, raw[:, 4:7],
                                            lt["emissive"], lt["probas"], lt["alias"], lt["power_sum"], st,
                                            st.samples_per_launch, bsdf="host")
        _close_to_oracle(b.image_sums(k)[1], orc, 0.93)


def test_job_completion_times_follow_iterations(cuda):
    jobs = _lambert_jobs()
    b = gbpt.Batch(jobs, samples_per_iteration=4)
    b.render()
    torch.cuda.synchronize()
    t = b.job_seconds()
    assert (t > 0).all()
    iters = [-(-s.samples_per_launch // 4) for _, s in jobs]  # 3, 1, 4
    order = np.argsort(iters)
    assert t[order[0]] <= t[order[1]] <= t[order[2]]


def test_batch_rejects_mixed_bsdf_modes(cuda):
    from gbpt import GbptError
    lam = _lambert_jobs()[:1]
    pri = _principled_jobs()[:1]
    with pytest.raises(GbptError):
        gbpt.Batch(lam + pri)
