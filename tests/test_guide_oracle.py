"""The learned guide's oracle checked against the mathematics it restates:
the loss gradient by finite differences (float64, no roundings), the vMF
mixture integrating to one and its sampling by the known mean cosine
coth(k) - 1/k (Jakob 2012), the hash-grid corners' weights summing to one."""
import numpy as np

from oracle.port import guide as G


def _outputs(rng, n):
    out = rng.normal(size=(n, G.OUT)).astype(np.float32)
    out[:, G.LOBES * 5:] = 0.0
    return out


def test_loss_gradient_by_finite_differences():
    rng = np.random.default_rng(3)
    n = 6
    out = _outputs(rng, n).astype(np.float64)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = rng.uniform(0.1, 2.0, n)
    _, g = G.loss_and_grad(out, d, w)
    eps = 1e-6
    for i in range(n):
        for k in range(G.LOBES * 5):
            a = out.copy()
            b = out.copy()
            a[i, k] += eps
            b[i, k] -= eps
            fd = (G.loss_and_grad(a, d, w)[0] - G.loss_and_grad(b, d, w)[0]) / (2 * eps)
            assert abs(fd - g[i, k]) <= 1e-4 * max(1.0, abs(fd)), (i, k, fd, g[i, k])


def test_mixture_is_a_density_and_samples_follow_it():
    rng = np.random.default_rng(5)
    out = _outputs(rng, 1)
    m = 200000
    d = rng.normal(size=(m, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    q = G.density(np.repeat(out, m, axis=0), d)
    assert abs(q.mean() * 4 * np.pi - 1.0) < 0.03
    # one lobe: the mean cosine to its axis is coth(k) - 1/k
    one = np.zeros((m, G.OUT), np.float32)
    one[:, 0] = 10.0
    one[:, 1] = np.log(3.0)
    one[:, 2:5] = [0.0, 0.6, 0.8]
    s = G.sample(one, rng.random(m), rng.random(m), rng.random(m))
    assert np.allclose(np.linalg.norm(s, axis=1), 1.0, atol=1e-6)
    cos = s @ np.array([0.0, 0.6, 0.8])
    assert abs(cos.mean() - (1 / np.tanh(3.0) - 1 / 3.0)) < 5e-3


def test_corner_weights_sum_to_one_and_stay_in_table():
    rng = np.random.default_rng(7)
    pos = rng.uniform(-1.2, 1.2, size=(500, 3)).astype(np.float32)
    idx, w = G.corners(pos, -1.0, 1.0, 12)
    assert np.allclose(w.sum(axis=2), 1.0, atol=1e-5)
    assert idx.min() >= 0 and idx.max() < (1 << 12)


def test_set_guide_checks_its_arguments_without_a_device():
    """kdn_set_guide on a host-only context: no guide detaches (OK), unknown
    flags and a share outside (0, 1) with a guide are refused; the guide
    entry points refuse null handles."""
    import ctypes

    import kodanuki_gb300 as K
    from helpers import host_backend

    b = host_backend()
    L = b.lib
    assert L.kdn_set_guide(b.handle, None, ctypes.c_float(0.5), 0) == K.KDN_OK
    assert L.kdn_set_guide(b.handle, None, ctypes.c_float(0.5), 8) == K.KDN_BAD_ARG
    fake = ctypes.c_void_p(1)  # never dereferenced: the share is refused first
    assert L.kdn_set_guide(b.handle, fake, ctypes.c_float(1.5), K.GUIDE_SAMPLE) == K.KDN_BAD_ARG
    assert L.kdn_guide_close(None) == K.KDN_BAD_ARG
    assert L.kdn_guide_ready(None) == 0
    o = K.GuideOptions()
    o.table_log2 = 30  # past the limit: refused before any device call
    h = ctypes.c_void_p()
    assert L.kdn_guide_open(0, ctypes.byref(o), ctypes.byref(h)) == K.KDN_BAD_ARG
    # pilot frames of no or of too many pixels, samples or surfaces are refused
    # before any host buffer is sized for them
    g, pc, gc = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
    for w, h_, spp, surf in [(-1, 64, 4, 6), (64, 0, 4, 6), (1 << 20, 1 << 20, 4, 6), (64, 64, 0, 6), (64, 64, 1 << 21, 6), (64, 64, 4, 0), (64, 64, 4, 256)]:
        f = K.Frame(w, h_, spp, surf, 1, 0, 0, 0)
        assert L.kdn_guide_select(b.handle, ctypes.byref(f), ctypes.byref(g), ctypes.byref(pc), ctypes.byref(gc)) == K.KDN_BAD_ARG, (w, h_, spp, surf)
