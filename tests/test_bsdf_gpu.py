"""GPU: the CUDA principled BSDF (gbpt_bsdf_eval / _pdf / _sample through the C ABI) against the
golden vectors of the reference's own BSDF, plus a consistency check of sampling against
evaluation that needs no reference: the one-sample estimate of the directional albedo
E[f |cos| / pdf] equals the albedo integrated from gbpt_bsdf_eval on a dense sphere grid."""
import numpy as np
import pytest
import torch

import bsdf_golden as G
from gbpt import bsdf, materials as M

pytestmark = pytest.mark.gpu


def _dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    return t.cuda() if dtype is None else t.to(dtype).cuda()


@pytest.mark.parametrize("which", sorted(G.SETS))
def test_eval_and_pdf_match_reference_golden(cuda, which):
    g = G.load(which)
    mats = _dev(g["materials"])
    q = _dev(G.queries(g["eval_q"], g.get("eval_w")))
    mi = _dev(g["eval_mat"].astype(np.int32))
    out = bsdf.eval(mats, mi, q).cpu().numpy()
    frac, flips = G.check_eval(out, g, max_flips=8)
    pdf = bsdf.pdf(mats, mi, q).cpu().numpy()
    assert np.array_equal(pdf, out[:, 3])
    assert G.close(pdf[:, None], g["pdf_out"][:, None], rtol=1e-4).mean() > 0.998
    print(f"eval: {frac:.4%} within 1e-5, {flips} beyond 2e-4 of {len(out)}")


@pytest.mark.parametrize("which", sorted(G.SETS))
def test_sampling_matches_reference_golden(cuda, which):
    g = G.load(which)
    mats = _dev(g["materials"])
    q = _dev(G.queries(g["sample_q"], g.get("sample_w")))
    mi = _dev(g["sample_mat"].astype(np.int32))
    seeds = _dev(g["seeds"].view(np.int32))
    out, lobe, rng = bsdf.sample(mats, mi, q, seeds)
    frac, flips = G.check_sample(out.cpu().numpy(), lobe.cpu().numpy(), bsdf.as_uint32(rng), g, max_flips=16)
    print(f"sample: {frac:.4%} within 1e-5, {flips} beyond 2e-4 of {len(out)}")


def _albedo_by_quadrature(mats, m_idx, view, normal, eta_out, n_theta=512, n_phi=1024):
    """Integral of f |cos| over the sphere, midpoint rule in (cos theta, phi) around the normal.

    Directions below the surface are evaluated as coming from the diffuse-transmission lobe (the
    only transmission lobe sampled there for the rough materials below): the reference applies the
    specular layer's fresnel attenuation to a refracted direction only when it was sampled from
    that lobe (Principled.h:1305-1318), so a transmitted direction's value depends on that tag."""
    ct = (np.arange(n_theta) + 0.5) / n_theta * 2.0 - 1.0
    ph = (np.arange(n_phi) + 0.5) / n_phi * 2.0 * np.pi
    c, p = np.meshgrid(ct, ph, indexing="ij")
    s = np.sqrt(1 - c * c)
    # frame around the normal
    n = normal / np.linalg.norm(normal)
    a = np.array([1.0, 0, 0]) if abs(n[0]) < 0.9 else np.array([0, 1.0, 0])
    t = np.cross(a, n)
    t /= np.linalg.norm(t)
    b = np.cross(n, t)
    dirs = (s * np.cos(p))[..., None] * t + (s * np.sin(p))[..., None] * b + c[..., None] * n
    dirs = dirs.reshape(-1, 3).astype(np.float32)
    k = len(dirs)
    q = np.zeros((k, 16), np.float32)
    q[:, 0:3] = view
    q[:, 3:6] = normal
    q[:, 6:9] = normal
    q[:, 9:12] = dirs
    q[:, 12] = 1.0
    q[:, 13] = eta_out
    below = c.reshape(-1) < 0
    q[below, 15] = bsdf.LOBES["diffuse_transmission"]
    rows = G.queries(q)
    f = bsdf.eval(mats, _dev(np.full(k, m_idx, np.int32)), _dev(rows)).cpu().numpy().astype(np.float64)
    cosv = np.abs(c.reshape(-1))
    dA = (2.0 / n_theta) * (2.0 * np.pi / n_phi)
    return (f[:, :3] * cosv[:, None]).sum(axis=0) * dA


@pytest.mark.parametrize("mat", [
    dict(base_color=(0.8, 0.4, 0.2), roughness=0.6, specular=0.0),
    dict(base_color=(0.8, 0.4, 0.2), roughness=0.5),
    dict(base_color=(0.9, 0.7, 0.4), roughness=0.45, metallic=1.0, anisotropy=0.5, anisotropy_rotation=0.25),
    dict(base_color=(0.5, 0.6, 0.3), roughness=0.5, coat=1.0, coat_roughness=0.35),
    dict(base_color=(0.9, 0.9, 0.9), roughness=0.5, specular_transmission=1.0, ior=1.5),
    dict(base_color=(0.3, 0.6, 0.8), roughness=0.5, diffuse_transmission=0.6),
])
def test_sampling_estimator_matches_quadrature(cuda, mat):
    """Unbiasedness of sampling + pdf: mean of f|cos|/pdf over 2M samples equals the quadrature
    of f|cos| within 4 sigma (plus 1% for the quadrature of the peaky lobes)."""
    rec = M.pack(**M.coat_roughened(mat))
    mats = _dev(rec[None, :])
    normal = np.array([0.2, 0.3, 0.93], np.float32)
    normal /= np.linalg.norm(normal)
    view = np.array([0.6, -0.2, 0.77], np.float32)
    view /= np.linalg.norm(view)
    ior = float(M.get(rec, "ior"))
    want = _albedo_by_quadrature(mats, 0, view, normal, ior)
    n = 1 << 21
    q = np.zeros((n, 16), np.float32)
    q[:, 0:3], q[:, 3:6], q[:, 6:9] = view, normal, normal
    q[:, 12], q[:, 13] = 1.0, ior
    rng = np.random.Generator(np.random.PCG64(7))
    seeds = rng.integers(1, 2**31 - 1, n).astype(np.int32)
    out, lobe, _ = bsdf.sample(mats, _dev(np.zeros(n, np.int32)), _dev(G.queries(q)), _dev(seeds))
    out = out.cpu().numpy().astype(np.float64)
    d, f, pdf = out[:, 0:3], out[:, 3:6], out[:, 6]
    w = np.where(pdf[:, None] > 0, f * np.abs(d @ normal.astype(np.float64))[:, None] / np.maximum(pdf, 1e-30)[:, None], 0.0)
    got, sigma = w.mean(axis=0), w.std(axis=0) / np.sqrt(n)
    assert np.all(np.abs(got - want) <= 4 * sigma + 0.01 * want + 1e-4), (got, want, sigma)
