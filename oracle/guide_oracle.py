"""CPU oracle of the guiding network (test infrastructure only: imported by tests/, never by the
product path).

The reference renderer has no learned path guiding (its closest relatives are the NEE++ visibility
cache and ReGIR light grids), so there is no reference output to pin this oracle to. It is pinned
instead by mathematics: its analytic gradients are checked against FP64 central differences of its
own loss, its vMF lobes integrate to one, its spherical harmonics are orthonormal, and the CUDA
kernels are checked against it.

Everything runs in float64 numpy. With bf16_ops=True the oracle rounds exactly where the CUDA
kernels hand BF16 values on: the grid features (read through a BF16 copy), the MLP input X, the
weights, the hidden activations, the output gradient dY and the hidden gradients, so the remaining
GPU/oracle difference is FP32 accumulation order and transcendental rounding.

Network: hash-grid features (16 levels x 2, trilinear, 2^19 entries per level) ++ normal ++
SH16(view) ++ zeros (64 inputs) -> ReLU(X W1) -> ReLU(H1 W2) -> ReLU(H2 W3) (64 each) -> H3 W4
(48 raw outputs) -> 8 vMF lobes (raw[5i:5i+3] direction, softplus(raw[5i+3]) + 0.1 clamped to 500
concentration, softmax(raw[5i+4]) weights) and alpha = 0.05 + 0.9 sigmoid(raw[40]).
Loss per sample with s = w / sum(w): -s log q(d) and, when the BSDF pdf p_b is given,
-s log(alpha q(d) + (1 - alpha) p_b) with q held fixed (its gradient reaches raw[40] only).
"""
from __future__ import annotations

import numpy as np

LEVELS, TABLE, FEATURES = 16, 1 << 19, 2
GRID_PARAMS = LEVELS * TABLE * FEATURES
IN, HIDDEN, OUT, LOBES, ROW = 64, 64, 48, 8, 44
OFF_W = (0, 4096, 8192, 12288)
WEIGHTS = 12288 + 64 * 48
SHAPES = ((IN, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, OUT))
RES = tuple(int(np.floor(16 * 256 ** (l / 15))) for l in range(LEVELS))
KAPPA_MIN, KAPPA_MAX, ALPHA_MIN = 0.1, 500.0, 0.05
LOG_2PI = np.log(2.0 * np.pi)
N_GRID_FEATURES, NORMAL_IN, SH_IN, ALPHA_OUT = 32, 32, 35, 40


def bf16(a) -> np.ndarray:
    """Round to the nearest BF16 (ties to even) through float32, returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    out = r.view(np.float32).astype(np.float64)
    nan = np.isnan(f)
    out[nan] = np.nan
    return out


def split_weights(weights):
    w = np.asarray(weights, np.float64)
    return tuple(w[o:o + a * b].reshape(a, b) for o, (a, b) in zip(OFF_W, SHAPES))


def grid_slot(res: int, x, y, z):
    """Table slot of grid vertices at a level: dense index when (res+1)^3 fits, else the XOR hash."""
    side = res + 1
    x = x.astype(np.uint64)
    y = y.astype(np.uint64)
    z = z.astype(np.uint64)
    if side ** 3 <= TABLE:
        return (x + side * (y + side * z)).astype(np.int64)
    h = (x * np.uint64(1)) ^ (y * np.uint64(2654435761)) ^ (z * np.uint64(805459861))
    return (h & np.uint64(TABLE - 1)).astype(np.int64)


def domain(scene_min, scene_max):
    lo = np.asarray(scene_min, np.float32)
    ext = np.asarray(scene_max, np.float32) - lo
    inv = np.where(ext > 0, np.float32(1.0) / np.where(ext > 0, ext, 1), 0).astype(np.float32)
    return lo.astype(np.float64), inv.astype(np.float64)


def corners(lo, inv_ext, P):
    """Per level: (slots (n, 8), trilinear weights (n, 8))."""
    u = np.clip((np.asarray(P, np.float64) - lo) * inv_ext, 0.0, 1.0)
    out = []
    for res in RES:
        x = u * res
        xi = np.clip(np.floor(x), 0, res - 1)
        f = x - xi
        xi = xi.astype(np.int64)
        slots, ws = [], []
        for c in range(8):
            bx, by, bz = c & 1, (c >> 1) & 1, (c >> 2) & 1
            w = ((f[:, 0] if bx else 1 - f[:, 0]) * (f[:, 1] if by else 1 - f[:, 1]) *
                 (f[:, 2] if bz else 1 - f[:, 2]))
            slots.append(grid_slot(res, xi[:, 0] + bx, xi[:, 1] + by, xi[:, 2] + bz))
            ws.append(w)
        out.append((np.stack(slots, 1), np.stack(ws, 1)))
    return out


def encode(grid, cor):
    g = np.asarray(grid, np.float64).reshape(LEVELS, TABLE, FEATURES)
    feats = []
    for l, (slots, ws) in enumerate(cor):
        feats.append(np.einsum("nc,ncf->nf", ws, g[l][slots]))
    return np.concatenate(feats, 1)


def sh16(d):
    """Real spherical harmonics of bands 0..3 of unit vectors (n, 3) -> (n, 16), orthonormal."""
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    pi = np.pi
    c1 = np.sqrt(3 / (4 * pi))
    c2a, c2b, c2c = np.sqrt(15 / (4 * pi)), np.sqrt(5 / (16 * pi)), np.sqrt(15 / (16 * pi))
    c3a, c3b, c3c = np.sqrt(35 / (32 * pi)), np.sqrt(105 / (4 * pi)), np.sqrt(21 / (32 * pi))
    c3d, c3e = np.sqrt(7 / (16 * pi)), np.sqrt(105 / (16 * pi))
    return np.stack([
        np.full_like(x, np.sqrt(1 / (4 * pi))),
        c1 * y, c1 * z, c1 * x,
        c2a * x * y, c2a * y * z, c2b * (3 * z * z - 1), c2a * x * z, c2c * (x * x - y * y),
        c3a * y * (3 * x * x - y * y), c3b * x * y * z, c3c * y * (5 * z * z - 1), c3d * z * (5 * z * z - 3),
        c3c * x * (5 * z * z - 1), c3e * z * (x * x - y * y), c3a * x * (x * x - 3 * y * y)], 1)


def input_rows(feat, N, V):
    n = feat.shape[0]
    x = np.zeros((n, IN))
    x[:, :N_GRID_FEATURES] = feat
    x[:, NORMAL_IN:NORMAL_IN + 3] = N
    x[:, SH_IN:SH_IN + 16] = sh16(np.asarray(V, np.float64))
    return x


def softplus(x):
    return np.where(x > 20.0, x, np.log1p(np.exp(np.minimum(x, 20.0))))


def sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def head(raw):
    """-> mu (n, 8, 3), kappa (n, 8), weight (n, 8), raw direction norms (n, 8), alpha (n,)."""
    r = raw[:, :LOBES * 5].reshape(-1, LOBES, 5)
    a = r[:, :, :3]
    ln = np.sqrt((a * a).sum(-1) + 1e-12)
    mu = a / ln[..., None]
    kappa = np.minimum(softplus(r[:, :, 3]) + KAPPA_MIN, KAPPA_MAX)
    lg = r[:, :, 4]
    e = np.exp(lg - lg.max(1, keepdims=True))
    alpha = ALPHA_MIN + (1 - 2 * ALPHA_MIN) * sigmoid(raw[:, ALPHA_OUT])
    return mu, kappa, e / e.sum(1, keepdims=True), ln, alpha


def log_vmf(kappa, c):
    return np.log(kappa) - LOG_2PI - np.log1p(-np.exp(-2.0 * kappa)) + kappa * (c - 1.0)


def mixture_pdf(mu, kappa, weight, d):
    c = np.einsum("nlk,nk->nl", mu, d)
    return (weight * np.exp(log_vmf(kappa, c))).sum(1)


def forward(weights, grid, lo, inv_ext, P, N, V, bf16_ops=True):
    """-> dict with the input X, pre-activations D1..D3, activations H1..H3, raw outputs."""
    rnd = bf16 if bf16_ops else (lambda a: np.asarray(a, np.float64))
    W = tuple(rnd(w) for w in split_weights(weights))
    cor = corners(lo, inv_ext, P)
    g = rnd(grid)
    X = rnd(input_rows(encode(g, cor), np.asarray(N, np.float64), np.asarray(V, np.float64)))
    acts, pre = [X], []
    for l in range(3):
        D = acts[-1] @ W[l]
        pre.append(D)
        acts.append(rnd(np.maximum(D, 0.0)))
    raw = acts[-1] @ W[3]
    return dict(cor=cor, acts=acts, pre=pre, raw=raw, W=W)


def loss_and_draw(raw, d, w, p_bsdf=None, q_fixed=None):
    """Batch loss and its gradient with respect to the raw outputs (n, 48). q_fixed (n,) replaces q
    in the alpha term (the value that term holds fixed), for finite-difference checks."""
    w = np.maximum(np.asarray(w, np.float64), 0.0)
    total = w.sum()
    scale = w / total if total > 0 else np.zeros_like(w)
    mu, kappa, pi, ln, alpha = head(raw)
    c = np.einsum("nlk,nk->nl", mu, d)
    lv = np.log(np.maximum(pi, 1e-30)) + log_vmf(kappa, c)
    m = lv.max(1, keepdims=True)
    logq = (m + np.log(np.exp(lv - m).sum(1, keepdims=True)))[:, 0]
    resp = np.exp(lv - logq[:, None])
    r = raw[:, :LOBES * 5].reshape(-1, LOBES, 5)
    draw = np.zeros((raw.shape[0], OUT))
    dl = draw[:, :LOBES * 5].reshape(-1, LOBES, 5)
    s = scale[:, None]
    dl[:, :, 4] = -s * (resp - pi)
    e2 = np.exp(-2.0 * kappa)
    dlogv = 1.0 / kappa - 2.0 * e2 / (1.0 - e2) + c - 1.0
    clamped = softplus(r[:, :, 3]) + KAPPA_MIN >= KAPPA_MAX
    dl[:, :, 3] = np.where(clamped, 0.0, -s * resp * dlogv * sigmoid(r[:, :, 3]))
    gm = (d[:, None, :] - c[..., None] * mu) * (resp * kappa / ln)[..., None]
    dl[:, :, :3] = -s[..., None] * gm
    loss = float((scale * -logq).sum())
    if p_bsdf is not None:
        pb = np.maximum(np.asarray(p_bsdf, np.float64), 0.0)
        q = np.exp(logq) if q_fixed is None else np.asarray(q_fixed, np.float64)
        mix = alpha * q + (1 - alpha) * pb
        ok = (mix > 0) & (scale > 0)
        sg = sigmoid(raw[:, ALPHA_OUT])
        safe = np.where(ok, mix, 1.0)
        draw[:, ALPHA_OUT] = np.where(ok, -scale * (q - pb) / safe * (1 - 2 * ALPHA_MIN) * sg * (1 - sg), 0.0)
        loss += float(np.where(ok, -scale * np.log(safe), 0.0).sum())
    return loss, draw, logq


def gradients(weights, grid, lo, inv_ext, P, N, V, D, w, p_bsdf=None, bf16_ops=True):
    """-> (loss, grad_weights (WEIGHTS,), grad_grid (GRID_PARAMS,)) of the batch loss."""
    rnd = bf16 if bf16_ops else (lambda a: np.asarray(a, np.float64))
    f = forward(weights, grid, lo, inv_ext, P, N, V, bf16_ops)
    W = f["W"]
    loss, draw, _ = loss_and_draw(f["raw"], np.asarray(D, np.float64), w, p_bsdf)
    dH = rnd(draw)
    gW = [None] * 4
    for l in range(3, -1, -1):
        gW[l] = f["acts"][l].T @ dH
        g = dH @ W[l].T
        if l > 0:
            dH = rnd(g * (f["pre"][l - 1] > 0))
        else:
            dX = g
    gg = np.zeros((LEVELS, TABLE, FEATURES))
    for l, (slots, ws) in enumerate(f["cor"]):
        contrib = ws[:, :, None] * dX[:, None, 2 * l:2 * l + 2]
        np.add.at(gg[l], slots.reshape(-1), contrib.reshape(-1, 2))
    return loss, np.concatenate([g.reshape(-1) for g in gW]), gg.reshape(-1)


def batch_loss(weights, grid, lo, inv_ext, P, N, V, D, w, p_bsdf=None, bf16_ops=False, q_fixed=None):
    f = forward(weights, grid, lo, inv_ext, P, N, V, bf16_ops)
    return loss_and_draw(f["raw"], np.asarray(D, np.float64), w, p_bsdf, q_fixed)[0]


def mixture_pdf_of(weights, grid, lo, inv_ext, P, N, V, D, bf16_ops=False):
    """q(D) per sample under the given parameters (what the alpha term holds fixed)."""
    f = forward(weights, grid, lo, inv_ext, P, N, V, bf16_ops)
    mu, kappa, pi, _, _ = head(f["raw"])
    return mixture_pdf(mu, kappa, pi, np.asarray(D, np.float64))


def infer(weights, grid, lo, inv_ext, P, N, V, bf16_ops=True):
    """-> (n, 44) rows in the layout of gbpt_guide_infer: 8 x (mu xyz, kappa, weight), alpha, 0, 0, 0."""
    f = forward(weights, grid, lo, inv_ext, P, N, V, bf16_ops)
    mu, kappa, pi, _, alpha = head(f["raw"])
    lobes = np.concatenate([mu, kappa[..., None], pi[..., None]], -1).reshape(-1, LOBES * 5)
    out = np.zeros((lobes.shape[0], ROW))
    out[:, :LOBES * 5] = lobes
    out[:, ALPHA_OUT] = alpha
    return out


def adam(params, grads, m, v, step, lr, b1, b2, eps):
    """One Adam step in float32, the update rule of gbpt_guide_train."""
    p = np.asarray(params, np.float32).copy()
    g = np.asarray(grads, np.float32)
    m = np.float32(b1) * m + np.float32(1 - b1) * g
    v = np.float32(b2) * v + np.float32(1 - b2) * g * g
    c1 = np.float32(1 - b1 ** step)
    c2 = np.float32(1 - b2 ** step)
    p -= np.float32(lr) * (m / c1) / (np.sqrt(v / c2) + np.float32(eps))
    return p, m, v


def random_params(seed=0, grid_scale=1e-2):
    """Glorot-uniform weights and uniform grid features (for CPU-only checks)."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out in SHAPES:
        s = np.sqrt(6.0 / (fan_in + fan_out))
        parts.append(rng.uniform(-s, s, fan_in * fan_out))
    grid = rng.uniform(-grid_scale, grid_scale, GRID_PARAMS)
    return np.concatenate(parts), grid


def random_batch(n, seed=0, lo=(0, 0, 0), hi=(1, 1, 1)):
    """Seeded training samples: positions in the box, unit normals, view and incident directions,
    weights >= 0 (a fifth of them zero) and BSDF pdfs (cosine lobes around the normal)."""
    rng = np.random.default_rng(seed)
    P = rng.uniform(lo, hi, (n, 3))
    N, V, D = (rng.normal(size=(n, 3)) for _ in range(3))
    for a in (N, V, D):
        a /= np.linalg.norm(a, axis=1, keepdims=True)
    w = rng.exponential(1.0, n) * (rng.random(n) < 0.8)
    pb = np.maximum((N * D).sum(1), 0.0) / np.pi
    f = np.float32
    return P.astype(f), N.astype(f), V.astype(f), D.astype(f), w.astype(f), pb.astype(f)
