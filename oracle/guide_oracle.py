"""CPU oracle of the guiding network (test infrastructure only: imported by tests/, never by the
product path).

The reference renderer has no learned path guiding (its closest relatives are the NEE++ visibility
cache and ReGIR light grids), so there is no reference output to pin this oracle to. It is pinned
instead by mathematics: its analytic gradients are checked against FP64 central differences of its
own loss, its vMF lobes integrate to one, and the CUDA kernels are checked against it.

Everything runs in float64 numpy. With bf16=True the oracle rounds exactly where the CUDA kernels
hand BF16 operands to the tensor cores (the MLP input X, the weights, the hidden activations H1 and
H2, the output gradient dY and the hidden gradients dH2 and dH1), so the remaining GPU/oracle
difference is FP32 accumulation order and transcendental rounding.

Network: hash-grid features (8 levels x 2, trilinear) ++ normal ++ [1] ++ view ++ zeros (32 inputs) ->
ReLU(X W1) (64) -> ReLU(H1 W2) (64) -> H2 W3 (48 raw outputs) -> 8 vMF lobes (raw[5i:5i+3]
direction, softplus(raw[5i+3]) + 0.1 clamped to 500 concentration, softmax(raw[5i+4]) weights).
Outputs 40..47 are unused. Loss: sum_i w_i / sum(w) * -log q(d_i).
"""
from __future__ import annotations

import numpy as np

LEVELS, TABLE, FEATURES = 8, 32768, 2
GRID_PARAMS = LEVELS * TABLE * FEATURES
IN, HIDDEN, OUT, LOBES = 32, 64, 48, 8
OFF_W1, OFF_W2 = 0, IN * HIDDEN
OFF_W3 = OFF_W2 + HIDDEN * HIDDEN
WEIGHTS = OFF_W3 + HIDDEN * OUT
RES = (4, 6, 9, 13, 20, 30, 45, 68)
KAPPA_MIN, KAPPA_MAX = 0.1, 500.0
LOG_2PI = np.log(2.0 * np.pi)


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
    return (w[OFF_W1:OFF_W2].reshape(IN, HIDDEN), w[OFF_W2:OFF_W3].reshape(HIDDEN, HIDDEN),
            w[OFF_W3:WEIGHTS].reshape(HIDDEN, OUT))


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


def input_rows(feat, N, V):
    n = feat.shape[0]
    x = np.zeros((n, IN))
    x[:, :16] = feat
    x[:, 16:19] = N
    x[:, 19] = 1.0
    x[:, 20:23] = V
    return x


def softplus(x):
    return np.where(x > 20.0, x, np.log1p(np.exp(np.minimum(x, 20.0))))


def sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def head(raw):
    """-> mu (n, 8, 3), kappa (n, 8), weight (n, 8), raw direction norms (n, 8)."""
    r = raw[:, :LOBES * 5].reshape(-1, LOBES, 5)
    a = r[:, :, :3]
    ln = np.sqrt((a * a).sum(-1) + 1e-12)
    mu = a / ln[..., None]
    kappa = np.minimum(softplus(r[:, :, 3]) + KAPPA_MIN, KAPPA_MAX)
    lg = r[:, :, 4]
    e = np.exp(lg - lg.max(1, keepdims=True))
    return mu, kappa, e / e.sum(1, keepdims=True), ln


def log_vmf(kappa, c):
    return np.log(kappa) - LOG_2PI - np.log1p(-np.exp(-2.0 * kappa)) + kappa * (c - 1.0)


def mixture_pdf(mu, kappa, weight, d):
    c = np.einsum("nlk,nk->nl", mu, d)
    return (weight * np.exp(log_vmf(kappa, c))).sum(1)


def forward(weights, grid, lo, inv_ext, P, N, V, bf16_ops=True):
    """-> dict with the input X, pre-activations D1, D2, activations H1, H2, raw outputs."""
    rnd = bf16 if bf16_ops else (lambda a: np.asarray(a, np.float64))
    W1, W2, W3 = (rnd(w) for w in split_weights(weights))
    cor = corners(lo, inv_ext, P)
    X = rnd(input_rows(encode(grid, cor), np.asarray(N, np.float64), np.asarray(V, np.float64)))
    D1 = X @ W1
    H1 = rnd(np.maximum(D1, 0.0))
    D2 = H1 @ W2
    H2 = rnd(np.maximum(D2, 0.0))
    raw = H2 @ W3
    return dict(cor=cor, X=X, D1=D1, H1=H1, D2=D2, H2=H2, raw=raw, W=(W1, W2, W3))


def loss_and_draw(raw, d, w):
    """Batch loss and its gradient with respect to the raw outputs (n, 48)."""
    w = np.maximum(np.asarray(w, np.float64), 0.0)
    total = w.sum()
    scale = w / total if total > 0 else np.zeros_like(w)
    mu, kappa, pi, ln = head(raw)
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
    return float((scale * -logq).sum()), draw, logq


def gradients(weights, grid, lo, inv_ext, P, N, V, D, w, bf16_ops=True):
    """-> (loss, grad_weights (WEIGHTS,), grad_grid (GRID_PARAMS,)) of the batch loss."""
    rnd = bf16 if bf16_ops else (lambda a: np.asarray(a, np.float64))
    f = forward(weights, grid, lo, inv_ext, P, N, V, bf16_ops)
    W1, W2, W3 = f["W"]
    loss, draw, _ = loss_and_draw(f["raw"], np.asarray(D, np.float64), w)
    dY = rnd(draw)
    gW3 = f["H2"].T @ dY
    dH2 = rnd((dY @ W3.T) * (f["D2"] > 0))
    gW2 = f["H1"].T @ dH2
    dH1 = rnd((dH2 @ W2.T) * (f["D1"] > 0))
    gW1 = f["X"].T @ dH1
    dX = dH1 @ W1.T
    gg = np.zeros((LEVELS, TABLE, FEATURES))
    for l, (slots, ws) in enumerate(f["cor"]):
        contrib = ws[:, :, None] * dX[:, None, 2 * l:2 * l + 2]
        np.add.at(gg[l], slots.reshape(-1), contrib.reshape(-1, 2))
    gw = np.concatenate([gW1.reshape(-1), gW2.reshape(-1), gW3.reshape(-1)])
    return loss, gw, gg.reshape(-1)


def batch_loss(weights, grid, lo, inv_ext, P, N, V, D, w, bf16_ops=False):
    f = forward(weights, grid, lo, inv_ext, P, N, V, bf16_ops)
    return loss_and_draw(f["raw"], np.asarray(D, np.float64), w)[0]


def infer(weights, grid, lo, inv_ext, P, N, V, bf16_ops=True):
    """-> (n, 8, 5): per lobe (mu xyz, kappa, weight), the layout of gbpt_guide_infer."""
    f = forward(weights, grid, lo, inv_ext, P, N, V, bf16_ops)
    mu, kappa, pi, _ = head(f["raw"])
    return np.concatenate([mu, kappa[..., None], pi[..., None]], -1)


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
    for fan_in, fan_out in ((IN, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, OUT)):
        s = np.sqrt(6.0 / (fan_in + fan_out))
        parts.append(rng.uniform(-s, s, fan_in * fan_out))
    grid = rng.uniform(-grid_scale, grid_scale, GRID_PARAMS)
    return np.concatenate(parts), grid


def random_batch(n, seed=0, lo=(0, 0, 0), hi=(1, 1, 1)):
    """Seeded training samples: positions in the box, unit normals, view and incident directions,
    weights >= 0 (a fifth of them zero)."""
    rng = np.random.default_rng(seed)
    P = rng.uniform(lo, hi, (n, 3))
    N, V, D = (rng.normal(size=(n, 3)) for _ in range(3))
    for a in (N, V, D):
        a /= np.linalg.norm(a, axis=1, keepdims=True)
    w = rng.exponential(1.0, n) * (rng.random(n) < 0.8)
    f = np.float32
    return P.astype(f), N.astype(f), V.astype(f), D.astype(f), w.astype(f)
