"""Generates the envmap golden fixtures from the REFERENCE's own envmap code and BSDF:

* tests/golden/envmap_ref.npz — vectors from oracle/_ref/libref_env.so and libref_env_bilinear.so
  (RGBE9995Packed::pack, eval_envmap_no_pdf, envmap_eval, envmap_sample with the alias table,
  envmap_cdf_search, compiled from the reference's sources): RGB9E5 words of edge-case and random
  texels; for a seeded 32 x 16 sky envmap and its tables, lookups and evals of random directions
  (nearest texel with identity rotation; bilinear with a rotation), samples from Xorshift32 seeds
  with the two draws each made, and CDF searches. The tables (texels, CDF, alias table) are the
  oracle's restatement of Image32Bit::compute_cdf / compute_alias_table: the reference's
  Image.cpp needs ImGui and OIDN and does not build here.
* tests/golden/pt_principled_env_cornell.npz — the principled Cornell box of
  make_pt_principled_golden.py under that sky (sun shining in through the open side), rendered by
  the path-tracing oracle with the reference's principled BSDF, with one-light MIS and with RIS
  direct lighting, envmap importance sampled by alias table.

Usage (where the reference tree is present):  python tests/golden/make_envmap_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "hiprt-path-tracer_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, HERE)

from gbpt import scenes  # noqa: E402
import pyoracle  # noqa: E402
import make_pt_principled_golden as P  # noqa: E402

OUT = os.path.join(HERE, "envmap_ref.npz")
OUT_PT = os.path.join(HERE, "pt_principled_env_cornell.npz")
ROTATION = np.array([[0.8, 0.0, 0.6], [0.0, 1.0, 0.0], [-0.6, 0.0, 0.8]], np.float32)


def pack_inputs(rng):
    edge = np.array([0.0, 1.0, 65408.0, 65407.9, 70000.0, 2.0 ** -16, 2.0 ** -17, 1e-20, 511.0 / 512, 0.5, 3.0e-5,
                     1.0e4], np.float32)
    rand = np.concatenate([rng.random(600) * 10.0, 10.0 ** rng.uniform(-9, 6, 600)]).astype(np.float32)
    v = np.concatenate([edge, rand])
    v = v[: (len(v) // 3) * 3].reshape(-1, 3)
    return np.concatenate([v, np.stack([edge, edge[::-1], np.roll(edge, 3)], -1)]).astype(np.float32)


def main():
    pyoracle.build(ref=True)
    rng = np.random.Generator(np.random.PCG64(20240607))
    out = {}
    x = pack_inputs(rng)
    out["pack_in"] = x
    out["pack_out"] = pyoracle.ref_env_pack(x)

    sky = scenes.sky_envmap(32, 16, seed=5)
    tb = pyoracle.env_tables(sky)
    out["sky"] = sky
    for k in ("texels", "cdf", "probas", "alias"):
        out[k] = tb[k]
    out["total_sum"] = np.float32(tb["total_sum"])
    out["total_sum64"] = np.float64(tb["total_sum64"])
    out["rotation"] = ROTATION
    dirs = rng.normal(size=(2000, 3)).astype(np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    # poles and seams: straight up/down, the u = 0/1 seam (-x), and directions just off them
    special = np.array([[0, 1, 0], [0, -1, 0], [-1, 0, 0], [1, 0, 0], [0, 0, 1], [0, 0, -1],
                        [-1, 1e-7, 0], [-1, 0, 1e-7], [-1, 0, -1e-7]], np.float32)
    dirs = np.concatenate([special / np.linalg.norm(special, axis=1, keepdims=True), dirs]).astype(np.float32)
    out["dirs"] = dirs
    seeds = rng.integers(1, 2 ** 32 - 1, 2000, dtype=np.uint32)
    out["seeds"] = seeds
    values = np.concatenate([[0.0, tb["total_sum"] * (1 - 1e-7)], rng.random(1000) * tb["total_sum"]]).astype(np.float32)
    out["cdf_values"] = values
    out["cdf_xy"] = pyoracle.ref_env_cdf_search(pyoracle.OracleEnv(texels=tb["texels"], cdf=tb["cdf"],
                                                                   probas=tb["probas"], alias=tb["alias"],
                                                                   total_sum=tb["total_sum"]), values)
    for tag, bilinear, rot, intensity in (("near", False, None, 1.0), ("bil", True, ROTATION, 1.7)):
        env = pyoracle.OracleEnv(texels=tb["texels"], cdf=tb["cdf"], probas=tb["probas"], alias=tb["alias"],
                                 intensity=intensity, total_sum=tb["total_sum"], rotation=rot, bilinear=bilinear)
        out[f"{tag}_lookup"] = pyoracle.ref_env_lookup(env, dirs)
        out[f"{tag}_eval_rgb"], out[f"{tag}_eval_pdf"] = pyoracle.ref_env_eval(env, dirs)
        d, c, p, idx, u = pyoracle.ref_env_sample(env, seeds)
        out[f"{tag}_sample_dir"], out[f"{tag}_sample_rgb"], out[f"{tag}_sample_pdf"] = d, c, p
        out[f"{tag}_sample_index"], out[f"{tag}_sample_u"] = idx, u
        out[f"{tag}_intensity"] = np.float32(intensity)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}")

    # principled Cornell box under the sky (sun in through the open -z side)
    mesh, mat_of, raw, eff = P.scene()
    st = P.settings()
    emission = raw[:, 4:7]
    emissive = np.nonzero(np.any(emission[mat_of] != 0, axis=1))[0].astype(np.int32)
    big = scenes.sky_envmap(64, 32, seed=2)
    tb = pyoracle.env_tables(big)
    env = pyoracle.OracleEnv(texels=tb["texels"], cdf=tb["cdf"], probas=tb["probas"], alias=tb["alias"],
                             intensity=1.5, total_sum=tb["total_sum"])
    soup = mesh.triangle_soup()
    mis = pyoracle.pt_render_principled(soup, mat_of, eff, emission, emissive, None, None, 0.0, st,
                                        st.samples_per_launch, env=env)
    st.direct_lighting, st.ris_light_candidates, st.ris_bsdf_candidates = 1, 4, 1
    ris = pyoracle.pt_render_principled(soup, mat_of, eff, emission, emissive, None, None, 0.0, st,
                                        st.samples_per_launch, env=env)
    np.savez_compressed(OUT_PT, sky=big, intensity=np.float32(1.5), texels=tb["texels"], cdf=tb["cdf"],
                        probas=tb["probas"], alias=tb["alias"], total_sum=np.float32(tb["total_sum"]),
                        image_mis=mis, image_ris=ris)
    print(f"wrote {OUT_PT}: mean MIS {mis.mean() / st.samples_per_launch:.4f}, RIS {ris.mean() / st.samples_per_launch:.4f}")


if __name__ == "__main__":
    main()
