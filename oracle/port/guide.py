"""CPU oracle of the learned guide: a multiresolution hash-grid encoding of
the position, a 48-64-64-64-48 ReLU network, and its 40 outputs read as a
mixture of eight von Mises-Fisher lobes over the sphere of directions.

Test infrastructure only (the checker of kodanuki_gb300/csrc/guide.cu): the
product never imports it.

The reference has no learned guide (its guides are the highlight guide,
plugins/sampler/highlight_guide/mixture.cpp:113 mixtureDirection, a
one-sample mixture of lumps and the BSDF); the learned form is the added
form of this backend, so this oracle restates published methods, not
reference code:

* the encoding is the multiresolution hash grid of Mueller et al. 2022
  ("Instant neural graphics primitives"): L levels of resolution
  floor(Nmin * b^l), b = exp(ln(Nmax / Nmin) / (L - 1)); a level whose
  (N + 1)^3 vertices fit its table is indexed densely, the others by the
  spatial hash (x * 1) ^ (y * 2654435761) ^ (z * 805459861) mod T;
  features trilinearly interpolated;
* the loss is the radiance-weighted negative log-likelihood of neural
  importance sampling (Mueller et al. 2019, "Neural importance sampling";
  Dong et al. 2023, "Neural parametric mixtures for path guiding"):
  mean over samples of -w * log q(direction), w the sample's estimate of the
  integrand over the density it was drawn with;
* the vMF density k / (2 pi (1 - exp(-2k))) exp(k (mu . w - 1)) and its
  sampling (Jakob 2012, "Numerically stable sampling of the von
  Mises-Fisher distribution on S2");
* Adam (Kingma and Ba 2015).

Parity is pinned by finite differences of this oracle's own loss (the
float64 path) and, for the device, by the bf16 roundings restated here at
the same points as the device kernels round (inputs and activations of each
layer and the output gradients, fp32 sums).
"""
from __future__ import annotations

import numpy as np

LEVELS = 16
FEATURES = 2
NMIN = 16
NMAX = 2048
LOBES = 8
IN = 48        # 32 grid features, the normal, a constant 1, zeros
HIDDEN = 64
OUT = 48       # 40 used: per lobe a logit, the log concentration, a mean direction
SHAPES = [(HIDDEN, IN), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (OUT, HIDDEN)]
KAPPA_LO, KAPPA_HI = -2.0, 8.0   # log concentration clamp
PRIMES = (1, 2654435761, 805459861)


def weight_count() -> int:
    return sum(a * b for a, b in SHAPES)


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), kept as float32."""
    x = np.ascontiguousarray(x, np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


# floor(Nmin * b^l), b = exp(ln(Nmax / Nmin) / (L - 1)), written out so the
# last level is 2048 and not the 2047 a rounding of b^15 below 128 would give
RESOLUTIONS = [16, 22, 30, 42, 58, 80, 111, 153, 212, 294, 406, 561, 776, 1072, 1482, 2048]


def resolutions() -> list[int]:
    return RESOLUTIONS


def initial(seed: int, table_log2: int):
    """Seeded start: Xavier-uniform weights (the output layer's unused rows
    zero) and a table uniform in +-1e-4, as the device's kdn_guide_open."""
    rng = np.random.default_rng(seed)
    ws = []
    for (n, k) in SHAPES:
        a = np.sqrt(6.0 / (n + k))
        w = rng.uniform(-a, a, size=(n, k)).astype(np.float32)
        ws.append(w)
    ws[3][LOBES * 5:] = 0.0
    table = rng.uniform(-1e-4, 1e-4, size=(LEVELS, 1 << table_log2, FEATURES)).astype(np.float32)
    return ws, table


def corners(pos: np.ndarray, lo, hi, table_log2: int):
    """Per sample and level, the 8 corner indices and trilinear weights."""
    T = 1 << table_log2
    u = np.clip((pos.astype(np.float32) - np.float32(lo)) / (np.float32(hi) - np.float32(lo)), 0.0, 1.0).astype(np.float32)
    n = len(pos)
    idx = np.zeros((n, LEVELS, 8), np.int64)
    wts = np.zeros((n, LEVELS, 8), np.float32)
    for l, N in enumerate(resolutions()):
        x = u * np.float32(N)
        c0 = np.minimum(np.floor(x), N - 1).astype(np.int64)
        f = (x - c0.astype(np.float32)).astype(np.float32)
        dense = (N + 1) ** 3 <= T
        for c in range(8):
            o = np.array([(c >> 0) & 1, (c >> 1) & 1, (c >> 2) & 1])
            g = c0 + o
            if dense:
                i = g[:, 0] + (N + 1) * (g[:, 1] + (N + 1) * g[:, 2])
            else:
                i = ((g[:, 0] * PRIMES[0]) ^ (g[:, 1] * PRIMES[1]) ^ (g[:, 2] * PRIMES[2])) & (T - 1)
            w = np.ones(n, np.float32)
            for a in range(3):
                w = w * (f[:, a] if o[a] else (np.float32(1) - f[:, a]))
            idx[:, l, c] = i
            wts[:, l, c] = w
    return idx, wts


def encode(pos, normal, table, lo, hi, table_log2):
    """The network's input row (float32, before the bf16 rounding)."""
    idx, wts = corners(pos, lo, hi, table_log2)
    t16 = table.astype(np.float16).astype(np.float32)
    n = len(pos)
    x = np.zeros((n, IN), np.float32)
    for l in range(LEVELS):
        feats = t16[l][idx[:, l, :]]                    # n, 8, 2
        x[:, 2 * l:2 * l + 2] = np.einsum("nc,ncf->nf", wts[:, l, :], feats).astype(np.float32)
    x[:, 32:35] = normal
    x[:, 35] = 1.0
    return x, idx, wts


def forward(x0, ws):
    """bf16 operands, fp32 sums: the activations each layer reads and the outputs."""
    acts = [bf16(x0)]
    for l in range(3):
        h = np.maximum(acts[-1] @ bf16(ws[l]).T, 0.0).astype(np.float32)
        acts.append(bf16(h))
    out = (acts[-1] @ bf16(ws[3]).T).astype(np.float32)
    return acts, out


def mixture(out):
    """(pi, kappa, mu, |m|, kappa_live) of each lobe from the outputs."""
    o = out[:, :LOBES * 5].reshape(-1, LOBES, 5).astype(np.float64)
    a = o[:, :, 0]
    a = a - a.max(axis=1, keepdims=True)
    e = np.exp(a)
    pi = e / e.sum(axis=1, keepdims=True)
    c = o[:, :, 1]
    live = (c > KAPPA_LO) & (c < KAPPA_HI)
    kappa = np.exp(np.clip(c, KAPPA_LO, KAPPA_HI))
    m = o[:, :, 2:5]
    norm = np.sqrt((m * m).sum(axis=2))
    # a mean of length under 1e-6 is read as +z, and passes no gradient
    flat = norm <= 1e-6
    safe = np.where(flat, np.inf, norm)
    mu = np.where(flat[:, :, None], np.array([0.0, 0.0, 1.0]), m / np.maximum(norm, 1e-6)[:, :, None])
    return pi, kappa, mu, safe, live


def log_vmf(kappa, cosine):
    return np.log(kappa) - np.log(2 * np.pi) - np.log1p(-np.exp(-2 * kappa)) + kappa * (cosine - 1.0)


def density(out, dirs):
    pi, kappa, mu, _, _ = mixture(out)
    cos = (mu * dirs[:, None, :]).sum(axis=2)
    return (pi * np.exp(log_vmf(kappa, cos))).sum(axis=1)


def loss_and_grad(out, dirs, weights):
    """mean(-w log q(d)) and its gradient with respect to the 48 outputs."""
    n = len(out)
    pi, kappa, mu, norm, live = mixture(out)
    cos = (mu * dirs[:, None, :]).sum(axis=2)
    lv = log_vmf(kappa, cos)
    pv = pi * np.exp(lv)
    q = pv.sum(axis=1)
    w = weights.astype(np.float64)
    loss = float(np.mean(-w * np.log(np.maximum(q, 1e-30))))
    gamma = pv / np.maximum(q, 1e-30)[:, None]           # responsibility of each lobe
    s = (-w / n)[:, None]                                  # d loss / d log v_j = s * gamma_j
    g = np.zeros((n, OUT), np.float64)
    g5 = g[:, :LOBES * 5].reshape(n, LOBES, 5)
    g5[:, :, 0] = s * (gamma - pi)
    e2 = np.exp(-2 * kappa)
    dlog_dk = 1.0 / kappa - 2 * e2 / (1 - e2) + (cos - 1.0)
    g5[:, :, 1] = np.where(live, s * gamma * dlog_dk * kappa, 0.0)
    gmu = (s * gamma)[:, :, None] * kappa[:, :, None] * dirs[:, None, :]
    proj = (gmu * mu).sum(axis=2, keepdims=True)
    g5[:, :, 2:5] = (gmu - proj * mu) / norm[:, :, None]
    g[:, :LOBES * 5] = g5.reshape(n, LOBES * 5)
    return loss, g.astype(np.float32)


def backward(acts, dout, ws, idx, wts, table_shape):
    """Weight gradients, and the table gradient, with the device's roundings."""
    dws = [None] * 4
    dy = bf16(dout)
    for l in (3, 2, 1, 0):
        dws[l] = (dy.T @ acts[l]).astype(np.float32)
        dx = (dy @ bf16(ws[l])).astype(np.float32)
        if l > 0:
            dy = bf16(np.where(acts[l] > 0, dx, 0.0).astype(np.float32))
    dtable = np.zeros(table_shape, np.float32)
    for l in range(LEVELS):
        for f in range(FEATURES):
            np.add.at(dtable[l, :, f], idx[:, l, :].ravel(), (wts[:, l, :] * dx[:, 2 * l + f][:, None]).ravel())
    return dws, dtable


def gradients(pos, normal, dirs, weights, ws, table, lo, hi, table_log2):
    x0, idx, wts = encode(pos, normal, table, lo, hi, table_log2)
    acts, out = forward(x0, ws)
    loss, dout = loss_and_grad(out, dirs, weights)
    dws, dtable = backward(acts, dout, ws, idx, wts, table.shape)
    return loss, dws, dtable, out


class Adam:
    """Adam over float32 parameters, as the device's kernels step it."""

    def __init__(self, lr=1e-2, b1=0.9, b2=0.99, eps=1e-8):
        self.lr, self.b1, self.b2, self.eps = lr, b1, b2, eps
        self.t = 0
        self.m = None
        self.v = None

    def step(self, params: list[np.ndarray], grads: list[np.ndarray]):
        if self.m is None:
            self.m = [np.zeros_like(p) for p in params]
            self.v = [np.zeros_like(p) for p in params]
        self.t += 1
        c1 = 1 - self.b1 ** self.t
        c2 = 1 - self.b2 ** self.t
        for p, g, m, v in zip(params, grads, self.m, self.v):
            m[...] = self.b1 * m + (1 - self.b1) * g
            v[...] = self.b2 * v + (1 - self.b2) * g * g
            p[...] = p - self.lr * (m / c1) / (np.sqrt(v / c2) + self.eps)


def sample(out, u_lobe, u, v):
    """Directions drawn from the mixture: a lobe by its weight, then the
    vMF by Jakob's stable inversion."""
    pi, kappa, mu, _, _ = mixture(out)
    cdf = np.cumsum(pi, axis=1)
    j = np.minimum((u_lobe[:, None] >= cdf).sum(axis=1), LOBES - 1)
    r = np.arange(len(out))
    k = kappa[r, j]
    m = mu[r, j]
    w = 1.0 + np.log(u + (1.0 - u) * np.exp(-2 * k)) / k
    s = np.sqrt(np.maximum(0.0, 1.0 - w * w))
    phi = 2 * np.pi * v
    t = np.where(np.abs(m[:, 0:1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    a = np.cross(m, t)
    a /= np.linalg.norm(a, axis=1, keepdims=True)
    b = np.cross(m, a)
    return w[:, None] * m + s[:, None] * (np.cos(phi)[:, None] * a + np.sin(phi)[:, None] * b)
