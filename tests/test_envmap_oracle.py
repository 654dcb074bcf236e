"""CPU: the envmap oracle (oracle/pt_oracle.cpp) against golden vectors from the reference's own
envmap code (tests/golden/envmap_ref.npz, made by tests/golden/make_envmap_golden.py from
RGBE9995Packed, eval_envmap_no_pdf, envmap_eval, envmap_sample and envmap_cdf_search compiled from
the reference's sources), and the oracle's table builds against their definitions."""
import os

import numpy as np
import pytest

import pyoracle
from gbpt import scenes

G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "envmap_ref.npz"))


def _env(tag):
    bil = tag == "bil"
    return pyoracle.OracleEnv(texels=G["texels"], cdf=G["cdf"], probas=G["probas"], alias=G["alias"],
                              intensity=float(G[f"{tag}_intensity"]), total_sum=float(G["total_sum"]),
                              rotation=G["rotation"] if bil else None, bilinear=bil)


def test_rgb9e5_packing_matches_reference_bit_for_bit():
    tex, _ = pyoracle.env_pack(G["pack_in"].reshape(1, -1, 3))
    np.testing.assert_array_equal(tex.reshape(-1), G["pack_out"])


def test_rgb9e5_round_trip_error_is_within_the_shared_exponent_step():
    x = G["pack_in"]
    y = pyoracle.env_unpack(G["pack_out"]).reshape(-1, 3)
    m = np.clip(x, 0, 65408).max(axis=1, keepdims=True)
    # each channel rounds to a 9-bit mantissa of the largest channel's exponent (plus its carry)
    assert (np.abs(y - np.clip(x, 0, 65408)) <= np.maximum(m, 2.0 ** -16) * 2.0 ** -8 + 1e-30).all()
    assert (y >= 0).all() and np.isfinite(y).all()


def test_tables_are_the_oracle_build_of_the_golden_sky():
    tb = pyoracle.env_tables(G["sky"])
    np.testing.assert_array_equal(tb["texels"], G["texels"])
    np.testing.assert_array_equal(tb["cdf"], G["cdf"])
    np.testing.assert_array_equal(tb["probas"], G["probas"])
    np.testing.assert_array_equal(tb["alias"], G["alias"])
    assert tb["total_sum64"] == float(G["total_sum64"])


def test_tables_follow_their_definitions():
    sky = G["sky"]
    tb = pyoracle.env_tables(sky)
    lum = ((sky[..., 0] * np.float32(0.3086)) + (sky[..., 1] * np.float32(0.6094))) + (sky[..., 2] * np.float32(0.0820))
    np.testing.assert_array_equal(tb["luminance"], lum.astype(np.float32))
    run = np.cumsum(lum.reshape(-1).astype(np.float64))
    np.testing.assert_array_equal(tb["cdf"].reshape(-1), run.astype(np.float32))
    assert (np.diff(tb["cdf"].reshape(-1)) >= 0).all()
    # the alias table samples texels in proportion to their luminance
    dist = pyoracle.alias_distribution(tb["probas"].reshape(-1), tb["alias"].reshape(-1))
    np.testing.assert_allclose(dist, lum.reshape(-1) / run[-1], rtol=1e-5, atol=1e-9)


@pytest.mark.parametrize("tag", ["near", "bil"])
def test_lookup_and_eval_match_reference(tag):
    env = _env(tag)
    np.testing.assert_array_equal(pyoracle.env_lookup(env, G["dirs"]), G[f"{tag}_lookup"])
    rgb, pdf = pyoracle.env_eval(env, G["dirs"])
    np.testing.assert_array_equal(rgb, G[f"{tag}_eval_rgb"])
    np.testing.assert_array_equal(pdf, G[f"{tag}_eval_pdf"])


@pytest.mark.parametrize("tag", ["near", "bil"])
def test_alias_sampling_matches_reference_from_its_draws(tag):
    env = _env(tag)
    d, c, p, xy = pyoracle.env_sample(env, index=G[f"{tag}_sample_index"], u=G[f"{tag}_sample_u"])
    np.testing.assert_array_equal(d, G[f"{tag}_sample_dir"])
    np.testing.assert_array_equal(c, G[f"{tag}_sample_rgb"])
    np.testing.assert_array_equal(p, G[f"{tag}_sample_pdf"])
    assert (xy[:, 0] < G["texels"].shape[1]).all() and (xy[:, 1] < G["texels"].shape[0]).all()


def test_cdf_search_matches_reference():
    env = _env("near")
    _, _, _, xy = pyoracle.env_sample(env, values=G["cdf_values"])
    np.testing.assert_array_equal(xy, G["cdf_xy"])


def test_sky_generator_is_seeded_and_positive():
    a, b = scenes.sky_envmap(32, 16, seed=5), scenes.sky_envmap(32, 16, seed=5)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, G["sky"])
    assert (a >= 0).all() and a.max() > 10 * np.median(a)  # a sun brighter than the sky
