"""TEST INFRASTRUCTURE ONLY — the principled-BSDF golden vectors (tests/golden/bsdf_principled.npz; for
the Oren-Nayar diffuse lobe, bsdf_oren_nayar.npz; with thin films, bsdf_thin_film.npz; with dispersion,
bsdf_dispersion.npz; written by the reference's own BSDF through tests/golden/make_bsdf_golden.py)
and the comparison both the CPU test (host build of the BSDF) and the GPU test (CUDA build) apply.

Tolerance on f, pdf and the sampled direction (relative, with an absolute floor of 1e-6 of the
row's largest value): 1e-5 for at least 99.5% of the evaluation queries and 99% of the sampling
queries, and 2e-4 for all of them. The CUDA
build contracts multiply-adds into FMAs and uses CUDA's float math functions, the reference's CPU
build does neither; near the peak of a sharp GGX lobe the lobe's conditioning amplifies those
one-ulp differences past 1e-5 for a fraction of a percent of the queries. A query may also sit on
the other side of a branch threshold (lobe choice u < cdf, total internal reflection, the delta
peak alignment test 0.999999) and then differ completely; those are counted and allowed up to a
small number. The dispersion set, where every material's glass lobe also contributes to the
evaluation of each sampled direction, measured 98.9% of its sampling queries within 1e-5 on the
CUDA build (100% on the host build), all within 2e-4; its sampling bar is 98.5%.
"""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bsdf_principled.npz")
# the same queries' kind against the reference built with its Oren-Nayar diffuse lobe
GOLDEN_OREN_NAYAR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bsdf_oren_nayar.npz")
# every material with a thin film over its metal, specular and glass interfaces
GOLDEN_THIN_FILM = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bsdf_thin_film.npz")
# every material dispersive, each query with the path's wavelength (eval_w, sample_w)
GOLDEN_DISPERSION = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bsdf_dispersion.npz")
SETS = {"lambertian": GOLDEN, "oren_nayar": GOLDEN_OREN_NAYAR, "thin_film": GOLDEN_THIN_FILM,
        "dispersion": GOLDEN_DISPERSION}
RTOL = 1e-5
RTOL_ALL = 2e-4
TIGHT_FRACTION = 0.995
TIGHT_FRACTION_SAMPLE = 0.99
TIGHT_FRACTION_SAMPLE_SET = {"dispersion": 0.985}


def load(which: str = "lambertian"):
    d = np.load(SETS[which])
    out = {k: d[k] for k in d.files}
    out["set"] = which
    return out


def queries(q16: np.ndarray, wavelength=None) -> np.ndarray:
    """Golden query rows (16 floats, inside/lobe as float values) and the path's wavelength per row
    (None: none) -> gbpt_bsdf_query records (20 words)."""
    q16 = np.asarray(q16, np.float32)
    out = np.zeros((len(q16), 20), np.float32)
    out[:, :16] = q16
    out[:, 14] = np.asarray(q16[:, 14] != 0, np.int32).view(np.float32)
    out[:, 15] = np.asarray(q16[:, 15], np.int32).view(np.float32)
    if wavelength is not None:
        out[:, 16] = wavelength
    return out


def close(a, b, rtol=RTOL):
    """Elementwise |a-b| <= rtol*max(|a|,|b|) + tiny, rows must agree on every column."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.maximum(np.abs(a), np.abs(b))
    ok = np.abs(a - b) <= rtol * scale + 1e-30
    # values that are both denormal-small compared with the row's largest magnitude
    row_scale = np.max(scale.reshape(len(scale), -1), axis=1, keepdims=True).reshape(
        (len(scale),) + (1,) * (scale.ndim - 1))
    ok |= np.abs(a - b) <= 1e-6 * row_scale
    return ok.reshape(len(ok), -1).all(axis=1)


def _check(kind, got, want, q, same_path, max_flips, gl=None, wl=None, tight_fraction=TIGHT_FRACTION):
    tight = same_path & close(got, want, RTOL)
    loose = same_path & close(got, want, RTOL_ALL)
    frac = float(tight.mean())
    flips = np.nonzero(~loose)[0]
    assert frac >= tight_fraction, _report(kind, np.nonzero(~tight)[0], got, want, q, gl, wl) + f"\nwithin 1e-5: {frac:.4f}"
    assert len(flips) <= max_flips, _report(kind, flips, got, want, q, gl, wl)
    return frac, len(flips)


def check_eval(got_f4, gold, max_flips=4):
    same = np.ones(len(got_f4), bool)
    return _check("eval", got_f4, gold["eval_out"], gold["eval_q"], same, max_flips)


def _weight(o8):
    """The sampling weight f / pdf per channel (what the path estimator multiplies by)."""
    pdf = o8[:, 6:7].astype(np.float64)
    return np.where(pdf > 0, o8[:, 3:6] / np.where(pdf > 0, pdf, 1.0), 0.0)


def check_sample(got8, got_lobe, got_rng, gold, max_flips=8):
    """Same lobe and same number of random draws; the sampled direction and the weight f/pdf within
    the tolerance above. f and pdf separately are evaluated exactly at the sampled direction, i.e.
    at the peak of the sampled GGX lobe, where a smooth lobe's value (up to 1e6 here) has a
    condition number of order 1/alpha^2; they must agree to 1e-3 for the same fraction of queries.
    The weight f/pdf does not suffer from it (the distribution term cancels)."""
    want = gold["sample_out"]
    tight_fraction = TIGHT_FRACTION_SAMPLE_SET.get(gold.get("set"), TIGHT_FRACTION_SAMPLE)
    same_path = (got_lobe == gold["sample_info"]) & (got_rng == gold["sample_rng"])
    got_dw = np.concatenate([got8[:, :3], _weight(got8)], axis=1)
    want_dw = np.concatenate([want[:, :3], _weight(want)], axis=1)
    res = _check("sample (direction, f/pdf)", got_dw, want_dw, gold["sample_q"], same_path, max_flips, got_lobe,
                 gold["sample_info"], tight_fraction=tight_fraction)
    loose = same_path & close(got8[:, 3:7], want[:, 3:7], 1e-3)
    assert loose.mean() >= tight_fraction, _report("sample (f, pdf)", np.nonzero(~loose)[0], got8, want,
                                                   gold["sample_q"], got_lobe, gold["sample_info"])
    return res


def _report(kind, bad, got, want, q, gl=None, wl=None):
    lines = [f"{kind}: {len(bad)} of {len(got)} queries differ"]
    for i in bad[:8]:
        extra = f" lobe {gl[i]} vs {wl[i]}" if gl is not None else ""
        lines.append(f"  #{i}: got {np.array2string(got[i], precision=6)} want {np.array2string(want[i], precision=6)}"
                     f"{extra} q={np.array2string(q[i], precision=4)}")
    return "\n".join(lines)
