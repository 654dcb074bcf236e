"""TEST INFRASTRUCTURE ONLY — the principled-BSDF golden vectors (tests/golden/bsdf_principled.npz,
written by the reference's own BSDF through tests/golden/make_bsdf_golden.py) and the comparison
both the CPU test (host build of the BSDF) and the GPU test (CUDA build) apply.

Tolerance: 1e-5 relative (with an absolute floor of 1e-6 of the value's scale) on f, pdf and the
sampled direction. The kernels are compiled with FMA contraction while the reference is not, so a
result may sit on the other side of a branch threshold (lobe choice u < cdf, total internal
reflection, the delta-peak alignment test 0.999999) in rare cases; such queries are classified
and allowed up to a small count, everything else must agree.
"""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bsdf_principled.npz")
RTOL = 1e-5


def load():
    d = np.load(GOLDEN)
    return {k: d[k] for k in d.files}


def queries(q16: np.ndarray) -> np.ndarray:
    """Golden query rows (16 floats, inside/lobe as float values) -> gbpt_bsdf_query records."""
    out = np.ascontiguousarray(q16, np.float32).copy()
    out[:, 14] = np.asarray(q16[:, 14] != 0, np.int32).view(np.float32)
    out[:, 15] = np.asarray(q16[:, 15], np.int32).view(np.float32)
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


def check_eval(got_f4, gold, max_flips=4):
    ok = close(got_f4, gold["eval_out"])
    bad = np.nonzero(~ok)[0]
    assert len(bad) <= max_flips, _report("eval", bad, got_f4, gold["eval_out"], gold["eval_q"])
    return len(bad)


def check_sample(got8, got_lobe, got_rng, gold, max_flips=8):
    same_path = (got_lobe == gold["sample_info"]) & (got_rng == gold["sample_rng"])
    ok = same_path & close(got8[:, :7], gold["sample_out"][:, :7])
    bad = np.nonzero(~ok)[0]
    assert len(bad) <= max_flips, _report("sample", bad, got8, gold["sample_out"], gold["sample_q"],
                                          got_lobe, gold["sample_info"])
    return len(bad)


def _report(kind, bad, got, want, q, gl=None, wl=None):
    lines = [f"{kind}: {len(bad)} of {len(got)} queries differ beyond rtol {RTOL}"]
    for i in bad[:8]:
        extra = f" lobe {gl[i]} vs {wl[i]}" if gl is not None else ""
        lines.append(f"  #{i}: got {np.array2string(got[i], precision=6)} want {np.array2string(want[i], precision=6)}"
                     f"{extra} q={np.array2string(q[i], precision=4)}")
    return "\n".join(lines)
