"""CPU: the path-tracing oracle's reference-RNG mode (the reference's Xorshift32 + wang_hash seeds,
draw order and packed G-buffer) against frames rendered by the REFERENCE's own CameraRays +
MegaKernel (tests/golden/ref_render_cornell.npz, tests/golden/make_ref_render_golden.py), and the
restated pieces of that mode against the reference's own code where the reference tree is
present: octahedral-24 normals, the 8-bit material packing (the library's host code), and
Utils::compute_alias_table."""
import numpy as np
import pytest

import pyoracle
from conftest import GOLDEN
from gbpt import materials as M
from gbpt.render import LIGHT_POWER, LIGHT_UNIFORM, RNG_REFERENCE, RenderSettings

REF = pytest.mark.skipif(not pyoracle.ref_render_available(), reason="needs the reference tree (oracle/_ref)")


def _golden():
    return np.load(f"{GOLDEN}/ref_render_cornell.npz")


def _settings(g, light):
    n = int(g["size"])
    return RenderSettings(width=n, height=n, samples_per_launch=1, nb_bounces=4, russian_roulette_min_depth=3,
                          light_sampling=light, inverse_view=g["inverse_view"],
                          inverse_projection=g["inverse_projection"], rng_mode=RNG_REFERENCE)


def _soup(g):
    return g["positions"][g["indices"]].reshape(-1, 9)


def test_lambert_oracle_matches_reference_megakernel_frames(oracle):
    """The restated estimator, seeded and drawing as the reference does, reproduces every pixel of
    the reference's own frames (float32 rounding of the sums aside)."""
    g = _golden()
    lam = g["lambert_materials"]
    q = pyoracle.ref_pack_unpack_material(lam) if pyoracle.ref_render_available() else None
    albedo = (q if q is not None else _packed_host(lam))[:, 0:3]
    emission = lam[:, 4:7]
    emissive = np.nonzero(np.any(emission[g["lambert_material_of"]] != 0, axis=1))[0].astype(np.int32)
    st = _settings(g, LIGHT_UNIFORM)
    for k, (rn_cam, rn_mk) in enumerate(g["random_numbers"]):
        st.random_number, st.random_number_shade = int(rn_cam), int(rn_mk)
        img = pyoracle.pt_render(_soup(g), g["lambert_material_of"], albedo, emission, emissive, None, None, 1.0, st, 1,
                                 iteration_base=k)
        ref = g["lambert"][k]
        rel = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
        # association of the float sums differs (the reference adds light + BSDF samples before the
        # throughput product), so a few pixels differ in the last bits
        assert (rel.max(axis=-1) < 1e-4).mean() == 1.0, k


def _packed_host(mats):
    from gbpt import render
    return render.material_pack_8bit(mats)


def test_library_material_packing_matches_reference_layout():
    """gbpt_material_pack_8bit (host code of the library) on the golden materials gives the
    records the reference's kernels read (8-bit fields truncated, green through its << 8 path)."""
    g = _golden()
    for key in ("lambert_materials", "principled_materials", "principled_glass_materials",
                "principled_thin_film_materials"):
        got = _packed_host(g[key])
        if pyoracle.ref_render_available():
            want = pyoracle.ref_pack_unpack_material(g[key])
            assert np.array_equal(got[:, :54].view(np.uint32), want[:, :54].view(np.uint32)), key


@REF
def test_material_packing_random_records_bit_exact():
    rng = np.random.default_rng(5)
    recs = M.pack_many(M.random_principled(rng, 200))
    for w in (0, 1, 2, 8, 9, 10, 12, 13, 14, 20, 21, 22, 28, 29, 30, 40, 41, 42):
        recs[:, w] = rng.uniform(0, 1, len(recs)).astype(np.float32)
    for w in (17, 18, 19, 23, 24, 25, 26, 27, 32, 33, 34, 36, 38, 39):
        recs[:, w] = rng.uniform(0, 1, len(recs)).astype(np.float32)
    recs[:, 36] = 0.0
    recs[:5, 0:3] = [[k / 255.0] * 3 for k in (0, 1, 127, 254, 255)]
    # thin film: weight and hue shift are 8-bit fields, the rest full floats
    recs[:, 47] = rng.uniform(0, 1, len(recs)).astype(np.float32)
    recs[:, 48] = rng.uniform(1.1, 2.2, len(recs)).astype(np.float32)
    recs[:, 49] = rng.uniform(50.0, 1500.0, len(recs)).astype(np.float32)
    recs[:, 50] = rng.uniform(0.0, 3.0, len(recs)).astype(np.float32)
    recs[:, 51] = rng.uniform(0, 1, len(recs)).astype(np.float32)
    recs[:, 52] = rng.uniform(1.0, 3.0, len(recs)).astype(np.float32)
    recs[:, 53] = (rng.random(len(recs)) < 0.5).astype(np.int32).view(np.float32)
    got = _packed_host(recs)
    want = pyoracle.ref_pack_unpack_material(recs)
    assert np.array_equal(got[:, :54].view(np.uint32), want[:, :54].view(np.uint32))


@REF
def test_oct24_restatement_matches_reference():
    rng = np.random.default_rng(3)
    n = rng.normal(size=(200_000, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    n[:6] = [[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, -1], [-1, 0, 0], [0.6, 0, -0.8]]
    want, _ = pyoracle.ref_oct24(n)
    got = pyoracle.oct24(n)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@REF
def test_alias_restatement_matches_reference_utils():
    """orc_vose_alias reproduces the reference's own Utils::compute_alias_table bit for bit given the
    same divisor. The library divides by the FP64 sum of the powers where the reference divides by
    its float running sum (CPURenderer.cpp:437-456): measured here, the reference's table then
    differs in the last bits of most probabilities and its implied distribution drifts from the
    exact power distribution by about the float sum's relative error (total variation 1.7e-6 at
    10,000 emitters, 4e-5 at 100,000), while the FP64 table stays within 1e-7."""
    rng = np.random.default_rng(11)
    for n in (1, 2, 3, 17, 1000, 10_000, 100_000):
        p = (rng.uniform(0, 1, n) ** 4 * 1000).astype(np.float32)
        s32 = np.float32(0)
        for v in p:
            s32 = np.float32(s32 + v)
        want_p, want_a = pyoracle.ref_alias_table(p, float(s32))
        got_p, got_a = pyoracle.vose_alias(p, float(s32))
        assert np.array_equal(got_p.view(np.uint32), want_p.view(np.uint32)) and np.array_equal(got_a, want_a), n
        s64 = float(np.sum(p.astype(np.float64)))
        f_p, f_a = pyoracle.vose_alias(p, s64)
        exact = p.astype(np.float64) / s64
        tv_ref = 0.5 * np.abs(pyoracle.alias_distribution(want_p, want_a) - exact).sum()
        tv_f64 = 0.5 * np.abs(pyoracle.alias_distribution(f_p, f_a) - exact).sum()
        sum_err = abs(float(s32) - s64) / s64
        assert tv_f64 < 1e-7, (n, tv_f64)
        assert tv_ref <= 2.0 * sum_err + 1e-7, (n, tv_ref, sum_err)
        assert tv_f64 <= tv_ref + 1e-8, (n, tv_f64, tv_ref)


@REF
@pytest.mark.parametrize("name", ["principled", "principled_glass", "principled_ris", "principled_thin_film"])
def test_principled_oracle_matches_reference_megakernel_frames(name):
    """The restated estimator with the reference's own BSDF (through callbacks that hand back the
    generator's state) on the principled Cornell box, with and without a rough glass box whose
    faces wind inwards: only the restated nested-dielectric stack (volume parity, not face
    orientation) enters and leaves it as the reference does; and with RIS direct lighting over
    4 light and 1 BSDF candidates (the reference's default strategy)."""
    g = _golden()
    raw = g[f"{name}_materials"]
    q = pyoracle.ref_pack_unpack_material(raw)
    eff = M.pack_many([M.coat_roughened(M.unpack(q[i])) for i in range(len(q))])
    pm = np.concatenate([eff, pyoracle.ref_pack_unpack_material(eff)])
    emission = raw[:, 4:7]
    mo = g[f"{name}_material_of"]
    emissive = np.nonzero(np.any(emission[mo] != 0, axis=1))[0].astype(np.int32)
    r = pyoracle.RefRender("principled", "power", g["positions"], g["indices"], mo, raw)
    lt = r.light_table()
    st = _settings(g, LIGHT_POWER)
    st.gbuffer_materials = len(raw)
    st.direct_lighting = 1 if name.endswith("_ris") else 0
    st.ris_light_candidates, st.ris_bsdf_candidates = 4, 1
    for k, (rn_cam, rn_mk) in enumerate(g["random_numbers"]):
        st.random_number, st.random_number_shade = int(rn_cam), int(rn_mk)
        img = pyoracle.pt_render_principled(_soup(g), mo, pm, emission, emissive, lt["probas"], lt["alias"],
                                            lt["power_sum"], st, 1, iteration_base=k)
        ref = g[name][k]
        rel = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
        assert (rel.max(axis=-1) < 1e-4).mean() > 0.995, k
