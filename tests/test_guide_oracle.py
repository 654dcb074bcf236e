"""CPU: the guiding-network oracle pinned by mathematics (no reference counterpart exists):
analytic gradients against FP64 central differences, vMF normalisation, orthonormal spherical
harmonics, the level-resolution schedule, BF16 rounding."""
import numpy as np

import guide_oracle as G


def _setup(n=64, seed=3):
    weights, grid = G.random_params(seed, grid_scale=0.2)
    P, N, V, D, w, pb = G.random_batch(n, seed + 1)
    lo, inv = G.domain((0, 0, 0), (1, 1, 1))
    return weights, grid, lo, inv, P, N, V, D, w, pb


def _loss(weights, grid, s):
    """The batch loss with q held fixed at the unperturbed parameters in the alpha term: the
    function whose gradient the analytic backward pass computes."""
    w0, g0, lo, inv, P, N, V, D, w, p = s
    q0 = G.mixture_pdf_of(w0, g0, lo, inv, P, N, V, D)
    return G.batch_loss(weights, grid, lo, inv, P, N, V, D, w, p, q_fixed=q0)


def test_weight_gradients_match_central_differences():
    s = _setup()
    weights, grid, lo, inv, P, N, V, D, w, pb = s
    _, gw, _ = G.gradients(weights, grid, lo, inv, P, N, V, D, w, pb, bf16_ops=False)
    rng = np.random.default_rng(0)
    idx = np.concatenate([rng.choice(np.arange(o, o + a * b), 12, replace=False) for o, (a, b) in zip(G.OFF_W, G.SHAPES)])
    idx = np.concatenate([idx, G.OFF_W[3] + np.arange(G.ALPHA_OUT, 64 * 48, 48)[:8]])  # the alpha column of W4
    h = 1e-6
    for i in idx:
        wp, wm = weights.copy(), weights.copy()
        wp[i] += h
        wm[i] -= h
        fd = (_loss(wp, grid, s) - _loss(wm, grid, s)) / (2 * h)
        assert abs(fd - gw[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, gw[i])


def test_grid_gradients_match_central_differences():
    s = _setup()
    weights, grid, lo, inv, P, N, V, D, w, pb = s
    _, _, gg = G.gradients(weights, grid, lo, inv, P, N, V, D, w, pb, bf16_ops=False)
    touched = np.nonzero(gg)[0]
    assert touched.size > 1000
    rng = np.random.default_rng(1)
    h = 1e-6
    for i in rng.choice(touched, 24, replace=False):
        gp, gm = grid.copy(), grid.copy()
        gp[i] += h
        gm[i] -= h
        fd = (_loss(weights, gp, s) - _loss(weights, gm, s)) / (2 * h)
        assert abs(fd - gg[i]) <= 1e-7 + 1e-4 * abs(fd), (i, fd, gg[i])


def test_head_gradients_cover_clamped_concentration_and_alpha():
    """Lobes whose concentration sits at the 500 clamp get no concentration gradient; the
    selection logit's gradient matches the mixture term of the loss."""
    rng = np.random.default_rng(2)
    raw = rng.normal(size=(5, G.OUT))
    raw[:, 3] = 600.0
    D = rng.normal(size=(5, 3))
    D /= np.linalg.norm(D, axis=1, keepdims=True)
    pb = rng.uniform(0.0, 1.0, 5)
    _, draw, _ = G.loss_and_draw(raw, D, np.ones(5), pb)
    assert np.all(draw[:, 3] == 0.0)
    assert np.all(draw[:, G.ALPHA_OUT + 1:] == 0.0)
    h = 1e-6
    for j in (0, 4, 8, 9, 13, G.ALPHA_OUT):
        rp, rm = raw.copy(), raw.copy()
        rp[2, j] += h
        rm[2, j] -= h
        if j == G.ALPHA_OUT:  # q is held fixed in the alpha term: differentiate only that term
            fd = (_alpha_term(rp, D, pb) - _alpha_term(rm, D, pb)) / (2 * h)
        else:
            fd = (G.loss_and_draw(rp, D, np.ones(5))[0] - G.loss_and_draw(rm, D, np.ones(5))[0]) / (2 * h)
        assert abs(fd - draw[2, j]) <= 1e-8 + 1e-5 * abs(fd), (j, fd, draw[2, j])


def _alpha_term(raw, D, pb):
    q0 = np.exp(G.loss_and_draw(raw, D, np.ones(5))[2])
    full = G.loss_and_draw(raw, D, np.ones(5), pb, q_fixed=q0)[0]
    return full - G.loss_and_draw(raw, D, np.ones(5))[0]


def test_vmf_lobes_integrate_to_one():
    """Midpoint quadrature over the sphere of the vMF density, low and high concentration."""
    nt, nphi = 1200, 600
    t = (np.arange(nt) + 0.5) / nt * np.pi
    ph = (np.arange(nphi) + 0.5) / nphi * 2 * np.pi
    T, PH = np.meshgrid(t, ph, indexing="ij")
    d = np.stack([np.sin(T) * np.cos(PH), np.sin(T) * np.sin(PH), np.cos(T)], -1).reshape(-1, 3)
    dA = (np.sin(T) * (np.pi / nt) * (2 * np.pi / nphi)).reshape(-1)
    for kappa in (0.1, 3.0, 60.0):
        mu = np.array([[0.3, -0.5, 0.81]])
        mu /= np.linalg.norm(mu)
        c = d @ mu[0]
        integral = (np.exp(G.log_vmf(kappa, c)) * dA).sum()
        assert abs(integral - 1.0) < 2e-3, (kappa, integral)


def test_spherical_harmonics_are_orthonormal_and_match_device_constants():
    nt, nphi = 400, 800
    t = (np.arange(nt) + 0.5) / nt * np.pi
    ph = (np.arange(nphi) + 0.5) / nphi * 2 * np.pi
    T, PH = np.meshgrid(t, ph, indexing="ij")
    d = np.stack([np.sin(T) * np.cos(PH), np.sin(T) * np.sin(PH), np.cos(T)], -1).reshape(-1, 3)
    dA = (np.sin(T) * (np.pi / nt) * (2 * np.pi / nphi)).reshape(-1)
    Y = G.sh16(d)
    gram = (Y * dA[:, None]).T @ Y
    np.testing.assert_allclose(gram, np.eye(16), atol=2e-4)
    # the literal constants of sh16 in csrc/guide_device.h
    import os
    import re
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "hiprt-path-tracer_gb300",
                            "csrc", "guide_device.h")).read()
    body = src[src.index("void sh16("):]
    body = body[:body.index("}")]
    consts = [float(c) for c in re.findall(r"o\[\d+\] = ([0-9.]+)f", body)]
    assert len(consts) == 16  # each device constant is the basis function's leading coefficient
    probe = np.array([[0.6, 0.0, 0.8], [0.0, 0.6, 0.8], [0.48, 0.6, 0.64]])
    x, y, z = probe[:, 0], probe[:, 1], probe[:, 2]
    c = consts
    dev = np.stack([np.full(3, c[0]), c[1] * y, c[2] * z, c[3] * x, c[4] * x * y, c[5] * y * z, c[6] * (3 * z * z - 1),
                    c[7] * x * z, c[8] * (x * x - y * y), c[9] * y * (3 * x * x - y * y), c[10] * x * y * z,
                    c[11] * y * (5 * z * z - 1), c[12] * z * (5 * z * z - 3), c[13] * x * (5 * z * z - 1),
                    c[14] * z * (x * x - y * y), c[15] * x * (x * x - 3 * y * y)], 1)
    np.testing.assert_allclose(dev, G.sh16(probe), rtol=1e-12, atol=1e-15)


def test_level_resolutions_follow_the_geometric_schedule():
    import os
    import re
    assert G.RES == (16, 23, 33, 48, 70, 101, 147, 212, 307, 445, 645, 933, 1351, 1955, 2830, 4096)
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "hiprt-path-tracer_gb300",
                            "csrc", "guide_device.h")).read()
    table = re.search(r"const int r\[16\] = \{([^}]*)\}", src).group(1)
    assert tuple(int(v) for v in table.split(",")) == G.RES
    dense = [(r + 1) ** 3 <= G.TABLE for r in G.RES]
    assert dense == [True] * 5 + [False] * 11


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -9, -2.5, 0.0, 3.0e38], np.float32)
    got = G.bf16(x)
    assert got[0] == 1.0
    assert got[1] == 1.0  # a tie: rounds to the even mantissa
    assert got[2] == 1.0 + 2 ** -7
    assert got[3] == 1.0
    assert got[4] == -2.5 and got[5] == 0.0


def test_bf16_loss_is_close_to_fp64_loss():
    s = _setup(256)
    weights, grid, lo, inv, P, N, V, D, w, pb = s
    l64 = G.batch_loss(weights, grid, lo, inv, P, N, V, D, w, pb, bf16_ops=False)
    l16 = G.batch_loss(weights, grid, lo, inv, P, N, V, D, w, pb, bf16_ops=True)
    assert abs(l64 - l16) < 2e-2 * abs(l64)
