"""CPU: the guiding-network oracle pinned by mathematics (no reference counterpart exists):
analytic gradients against FP64 central differences, vMF normalisation, BF16 rounding."""
import numpy as np

import guide_oracle as G


def _setup(n=96, seed=3):
    weights, grid = G.random_params(seed, grid_scale=0.2)
    P, N, V, D, w = G.random_batch(n, seed + 1)
    lo, inv = G.domain((0, 0, 0), (1, 1, 1))
    return weights, grid, lo, inv, P, N, V, D, w


def test_weight_gradients_match_central_differences():
    weights, grid, lo, inv, P, N, V, D, w = _setup()
    _, gw, _ = G.gradients(weights, grid, lo, inv, P, N, V, D, w, bf16_ops=False)
    rng = np.random.default_rng(0)
    idx = np.concatenate([rng.choice(np.arange(G.OFF_W1, G.OFF_W2), 12, replace=False),
                          rng.choice(np.arange(G.OFF_W2, G.OFF_W3), 12, replace=False),
                          rng.choice(np.arange(G.OFF_W3, G.WEIGHTS), 24, replace=False)])
    h = 1e-6
    for i in idx:
        wp, wm = weights.copy(), weights.copy()
        wp[i] += h
        wm[i] -= h
        fd = (G.batch_loss(wp, grid, lo, inv, P, N, V, D, w) - G.batch_loss(wm, grid, lo, inv, P, N, V, D, w)) / (2 * h)
        assert abs(fd - gw[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, gw[i])


def test_grid_gradients_match_central_differences():
    weights, grid, lo, inv, P, N, V, D, w = _setup()
    _, _, gg = G.gradients(weights, grid, lo, inv, P, N, V, D, w, bf16_ops=False)
    touched = np.nonzero(gg)[0]
    assert touched.size > 100
    rng = np.random.default_rng(1)
    h = 1e-6
    for i in rng.choice(touched, 32, replace=False):
        gp, gm = grid.copy(), grid.copy()
        gp[i] += h
        gm[i] -= h
        fd = (G.batch_loss(weights, gp, lo, inv, P, N, V, D, w) - G.batch_loss(weights, gm, lo, inv, P, N, V, D, w)) / (2 * h)
        assert abs(fd - gg[i]) <= 1e-7 + 1e-4 * abs(fd), (i, fd, gg[i])


def test_head_gradients_cover_clamped_concentration():
    """Lobes whose concentration sits at the 500 clamp get no concentration gradient."""
    rng = np.random.default_rng(2)
    raw = rng.normal(size=(5, G.OUT))
    raw[:, 3] = 600.0
    D = rng.normal(size=(5, 3))
    D /= np.linalg.norm(D, axis=1, keepdims=True)
    _, draw, _ = G.loss_and_draw(raw, D, np.ones(5))
    assert np.all(draw[:, 3] == 0.0)
    h = 1e-6
    for j in (0, 4, 8, 9, 13):
        rp, rm = raw.copy(), raw.copy()
        rp[2, j] += h
        rm[2, j] -= h
        fd = (G.loss_and_draw(rp, D, np.ones(5))[0] - G.loss_and_draw(rm, D, np.ones(5))[0]) / (2 * h)
        assert abs(fd - draw[2, j]) <= 1e-8 + 1e-5 * abs(fd)


def test_vmf_lobes_integrate_to_one():
    """Midpoint quadrature over the sphere of the mixture density, low and high concentration."""
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


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -9, -2.5, 0.0, 3.0e38], np.float32)
    got = G.bf16(x)
    assert got[0] == 1.0
    assert got[1] == 1.0  # a tie: rounds to the even mantissa
    assert got[2] == 1.0 + 2 ** -7
    assert got[3] == 1.0
    assert got[4] == -2.5 and got[5] == 0.0


def test_bf16_loss_is_close_to_fp64_loss():
    weights, grid, lo, inv, P, N, V, D, w = _setup(256)
    l64 = G.batch_loss(weights, grid, lo, inv, P, N, V, D, w, bf16_ops=False)
    l16 = G.batch_loss(weights, grid, lo, inv, P, N, V, D, w, bf16_ops=True)
    assert abs(l64 - l16) < 2e-2 * abs(l64)
