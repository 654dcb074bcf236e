"""GPU: learned path guiding inside the wavefront path tracer. The continuation is one-sample MIS of
the network's vMF mixture and BSDF sampling, so the image must stay unbiased whatever the network
has learned; after online training it must also be less noisy than BSDF sampling at equal samples
per pixel on a scene lit indirectly. Training records must be well formed."""
import numpy as np
import pytest
import torch

import gbpt
from gbpt import guide, scenes
from gbpt.render import guide_render_settings

pytestmark = pytest.mark.gpu

BOX = ((0.0, 0.0, 0.0), (5.5, 5.5, 5.5))


def _indirect_cornell():
    """The Cornell box with its light lowered to y = 4.5 and turned to face the ceiling: the room is
    lit almost only by the bright patch the light makes on the ceiling, which cosine sampling of a
    continuation rarely finds."""
    cb = scenes.cornell_box()
    pos = cb.mesh.positions.copy()
    for t in cb.emissive_triangles:
        i = cb.mesh.indices[t]
        pos[i, 1] = 4.5
        pos[[i[1], i[2]]] = pos[[i[2], i[1]]]  # reverse the winding: the emitting side faces +y
    return gbpt.Scene(pos, cb.mesh.indices, cb.material_of_triangle, cb.albedo, cb.emission)


def _image(r):
    torch.cuda.synchronize()
    return r.image_sums()[1]


def _plain(scene, spp, launches, seed, w=32, h=32):
    r = gbpt.Renderer(scene, gbpt.cornell_settings(w, h, samples_per_launch=spp, seed=seed))
    r.render(launches)
    return _image(r) / (spp * launches)


def _trained_guided(scene, spp, train_launches, seed, w=32, h=32, **kw):
    r = gbpt.Renderer(scene, gbpt.cornell_settings(w, h, samples_per_launch=spp, seed=seed))
    g = guide.Guide(scene_min=BOX[0], scene_max=BOX[1], seed=seed)
    r.set_guide(g, guide_render_settings(**kw))
    r.render(train_launches)
    return r, g


def _launch_images(r, n, launches_each=1):
    """n consecutive images of launches_each launches, as differences of the accumulated sums (the
    renderer is not reset, so every launch draws fresh random numbers, independent of the samples
    the network was trained on)."""
    prev = _image(r)
    out = []
    for _ in range(n):
        r.render(launches_each)
        cur = _image(r)
        out.append(cur - prev)
        prev = cur
    return out


def _relmse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


@pytest.fixture(scope="module")
def indirect_reference(cuda):
    scene = _indirect_cornell()
    return scene, _plain(scene, 1024, 32, seed=1000)


def test_training_records_are_well_formed(cuda, indirect_reference):
    scene, _ = indirect_reference
    r, g = _trained_guided(scene, 4, 0, seed=3)
    r.render(1)
    n, rec = r.guide_records()
    assert n > 1000 and rec.shape[0] == min(n, 1 << 16)
    pos, nrm, view, d, w, pb = rec[:, 0:3], rec[:, 3:6], rec[:, 6:9], rec[:, 9:12], rec[:, 12], rec[:, 13]
    slot = rec[:, 14].view(np.int32)
    assert (pos >= -1e-3).all() and (pos <= 5.5 + 1e-3).all()
    for v in (nrm, view, d):
        np.testing.assert_allclose(np.linalg.norm(v, axis=1), 1.0, atol=1e-4)
    assert ((nrm * view).sum(1) >= -1e-6).all()  # the normal faces the viewer
    # Lambertian continuations leave above the surface (the shading normal may be bent slightly)
    assert ((nrm * d).sum(1) > -0.1).all() and ((nrm * d).sum(1) > 0).mean() > 0.99
    assert np.isfinite(w).all() and (w >= 0).all() and (w <= 50.0).all() and (w > 0).mean() > 0.05
    # continuation records carry their path slot, light-sample records -1
    assert ((slot >= 0) | (slot == -1)).all() and (slot < 32 * 32 * 4).all()
    assert (slot == -1).any() and (slot >= 0).any()
    # the recorded BSDF pdf is the Lambertian cos / pi of the recorded direction (about the shading
    # normal, which equals the recorded geometric normal unless it was bent)
    close = np.abs(pb - np.maximum((nrm * d).sum(1), 0) / np.pi) < 2e-3
    assert close.mean() > 0.99, close.mean()
    assert g.error_flag() == 0


def test_guided_rendering_is_unbiased(cuda, indirect_reference):
    """Mean radiance of independent guided renders (network still training, probability 0.5)
    agrees with the 32768-spp plain image within 3 sigma."""
    scene, ref = indirect_reference
    r, g = _trained_guided(scene, 16, 20, seed=5)
    means = np.array([(img / 16).mean() for img in _launch_images(r, 48)])
    sigma = means.std(ddof=1) / np.sqrt(len(means))
    assert abs(means.mean() - ref.mean()) < 3 * sigma + 1e-6, (means.mean(), ref.mean(), sigma)
    assert g.error_flag() == 0


def test_guiding_reduces_error_at_equal_spp(cuda, indirect_reference):
    """After 300 training launches, 64 spp of guided rendering have a lower relMSE than 64 spp of
    BSDF sampling against the high-spp reference (averaged over 4 seeds each)."""
    scene, ref = indirect_reference
    r, _ = _trained_guided(scene, 4, 300, seed=9)
    guided = [_relmse(img / 64, ref) for img in _launch_images(r, 4, 16)]
    plain = [_relmse(_plain(scene, 4, 16, seed=100 + k), ref) for k in range(4)]
    assert np.mean(guided) < 0.8 * np.mean(plain), (guided, plain)


def test_guided_principled_scene_is_unbiased(cuda):
    """The principled Cornell box (coated, rough dielectric and anisotropic-metal walls are guided;
    the rough glass box and the mirror are not) stays unbiased with guiding on."""
    import os
    from gbpt.render import BSDF_PRINCIPLED, LIGHT_UNIFORM, RenderSettings
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pt_principled_cornell.npz"))
    w, h, _, nb, rr, _ = (int(v) for v in g["settings"])
    scene = gbpt.Scene(g["positions"], g["indices"], g["material_of"], principled=g["materials"])

    def settings(spp, seed):
        return RenderSettings(width=w, height=h, samples_per_launch=spp, nb_bounces=nb, russian_roulette_min_depth=rr,
                              light_sampling=LIGHT_UNIFORM, bsdf=BSDF_PRINCIPLED, seed=seed,
                              inverse_view=g["inverse_view"], inverse_projection=g["inverse_projection"])

    rp = gbpt.Renderer(scene, settings(512, 1000))
    rp.render(32)
    ref = _image(rp) / (512 * 32)
    r = gbpt.Renderer(scene, settings(16, 3))
    gd = guide.Guide(scene_min=BOX[0], scene_max=BOX[1], seed=2)
    r.set_guide(gd, guide_render_settings())
    r.render(20)
    means = np.array([(img / 16).mean() for img in _launch_images(r, 48)])
    sigma = means.std(ddof=1) / np.sqrt(len(means))
    assert abs(means.mean() - ref.mean()) < 3 * sigma + 1e-6, (means.mean(), ref.mean(), sigma)


def test_set_guide_validates_and_detaches(cuda):
    from gbpt import GbptError
    scene = _indirect_cornell()
    r = gbpt.Renderer(scene, gbpt.cornell_settings(16, 16, samples_per_launch=2, seed=1))
    g = guide.Guide(scene_min=BOX[0], scene_max=BOX[1], max_batch=1024)
    with pytest.raises(GbptError):
        r.set_guide(g, guide_render_settings(guide_probability=1.0))
    with pytest.raises(GbptError):
        r.set_guide(g, guide_render_settings(max_records=4096))  # above the guide's max_batch
    r.set_guide(g, guide_render_settings(max_records=1024))
    r.render(2)
    n, rec = r.guide_records()
    assert n > 0 and rec.shape[0] == min(n, 1024)
    r.set_guide(None)
    with pytest.raises(GbptError):
        r.guide_records()
    # detached: the plain estimator again, bit for bit
    r.reset()
    r.render(1)
    a = _image(r)
    b = gbpt.Renderer(scene, gbpt.cornell_settings(16, 16, samples_per_launch=2, seed=1))
    b.render(3)
    b.reset()
    b.render(1)
    assert np.array_equal(a, _image(b))
