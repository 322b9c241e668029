"""The learned guide's tensor-core kernels against the CPU oracle
(oracle/port/guide.py) on the same parameters and samples: the lobes of the
inference kernel, the loss and the gradients of every weight and table
entry from the training kernel, and a training run that fits a known field
of directions."""
import numpy as np
import pytest

from oracle.port import guide as G

pytestmark = pytest.mark.gpu

LOG2 = 12
LO, HI = -1.0, 1.0


def _guide(**kw):
    import kodanuki_gb300 as K
    return K.Guide(0, table_log2=LOG2, seed=kw.pop("seed", 3), region=((LO,) * 3, (HI,) * 3), **kw)


def _weights(flat):
    ws, o = [], 0
    for (n, k) in G.SHAPES:
        ws.append(flat[o:o + n * k].reshape(n, k))
        o += n * k
    return ws


def _rows(rng, n):
    p = rng.uniform(-1.1, 1.1, size=(n, 3)).astype(np.float32)
    nv = rng.normal(size=(n, 3))
    nv = (nv / np.linalg.norm(nv, axis=1, keepdims=True)).astype(np.float32)
    return p, nv


def _livelier(g, rng):
    """Weights and a table scaled up from the start, so every layer and the
    grid carry signal through the ReLUs."""
    w, t = g.params()
    w = w * 2.0
    t = rng.uniform(-0.5, 0.5, size=t.shape).astype(np.float32)
    g.set_params(w, t)
    return _weights(w), t.reshape(G.LEVELS, 1 << LOG2, 2)


def test_query_matches_oracle():
    rng = np.random.default_rng(11)
    with _guide() as g:
        ws, table = _livelier(g, rng)
        p, nv = _rows(rng, 3000)
        lobes = g.query(np.concatenate([p, nv], axis=1))
        x0, _, _ = G.encode(p, nv, table, LO, HI, LOG2)
        _, out = G.forward(x0, ws)
        pi, kappa, mu, _, _ = G.mixture(out)
        L = lobes.reshape(-1, 8, 5)
        err_pi = np.abs(L[:, :, 0] - pi)
        err_k = np.abs(np.log(L[:, :, 1]) - np.log(kappa))
        cos = (L[:, :, 2:5] * mu).sum(axis=2)
        assert np.quantile(err_pi, 0.99) < 5e-3 and err_pi.max() < 3e-2, err_pi.max()
        assert np.quantile(err_k, 0.99) < 1e-2, np.quantile(err_k, 0.99)
        assert np.quantile(1 - cos, 0.99) < 1e-4, np.quantile(1 - cos, 0.99)


def test_gradients_match_oracle():
    rng = np.random.default_rng(13)
    with _guide() as g:
        ws, table = _livelier(g, rng)
        n = 1000  # not a multiple of the 128-sample tile
        p, nv = _rows(rng, n)
        d = rng.normal(size=(n, 3))
        d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
        w = rng.uniform(0.0, 3.0, n).astype(np.float32)
        samples = np.concatenate([p, nv, d, w[:, None]], axis=1)
        loss, dw, dt = g.gradients(samples)
        want_loss, want_dws, want_dt, _ = G.gradients(p, nv, d, w, ws, table, LO, HI, LOG2)
        assert abs(loss - want_loss) <= 2e-3 * abs(want_loss), (loss, want_loss)
        got = _weights(dw)
        for l in range(4):
            a, b = got[l].ravel(), want_dws[l].ravel()
            rel = np.linalg.norm(a - b) / np.linalg.norm(b)
            assert rel < 2e-2, (l, rel)
            assert np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b)) > 0.999, l
        a, b = dt.ravel(), want_dt.ravel()
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 2e-2
        # the output layer's unused rows get no gradient
        assert np.all(got[3][40:] == 0)


def test_training_fits_a_field_of_directions():
    """Directions drawn around normalize(p) (vMF, k = 20) at uniform points:
    after training, held-out samples are far likelier under the guide than
    under a uniform sphere."""
    rng = np.random.default_rng(17)

    def draw(n):
        p, nv = _rows(rng, n)
        axis = p / np.linalg.norm(p, axis=1, keepdims=True)
        lo = np.zeros((n, G.OUT), np.float32)
        lo[:, 0] = 10.0
        lo[:, 1] = np.log(20.0)
        lo[:, 2:5] = axis
        d = G.sample(lo, rng.random(n), rng.random(n), rng.random(n)).astype(np.float32)
        return np.concatenate([p, nv, d, np.ones((n, 1), np.float32)], axis=1)

    with _guide(seed=5) as g:
        # online, as the renderer trains: ~2 passes over many samples, not
        # many passes over few (the fine levels would learn the samples
        # themselves and lose the held-out ones)
        train = draw(1 << 20)
        first = g.train(train, batch=8192, steps=1)
        last = g.train(train, batch=8192, steps=300)
        held = draw(4096)
        lobes = g.query(held[:, 0:6])
        q = G.density(_lobes_as_outputs(lobes), held[:, 6:9].astype(np.float64))
        gain = np.mean(np.log(q)) + np.log(4 * np.pi)
        assert last < first - 1.0, (first, last)
        # a perfect fit gains log(20 / 2pi) + 20 (coth 20 - 1/20 - 1) + log 4pi
        # = 2.69 nats; the weight-gradient sums run in atomics' order, so
        # runs differ a little: ask for a third of it
        assert gain > 0.9, gain


def _lobes_as_outputs(lobes):
    """Outputs whose mixture is these lobes (log weights, log concentration, mean)."""
    L = lobes.reshape(-1, 8, 5).astype(np.float64)
    out = np.zeros((len(L), G.OUT))
    o = out[:, :40].reshape(-1, 8, 5)
    o[:, :, 0] = np.log(np.maximum(L[:, :, 0], 1e-30))
    o[:, :, 1] = np.log(L[:, :, 1])
    o[:, :, 2:5] = L[:, :, 2:5]
    return out
