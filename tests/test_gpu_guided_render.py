"""Frames drawn with the learned guide: trained online on the tracer's own
paths, then mixed with the BSDF by one-sample MIS.  The guided frame must
keep the plain frame's expectation (the estimator stays unbiased) and gain
over plain BSDF sampling at equal samples, in relative MSE against a
high-sample plain frame (relMSE = mean((img - ref)^2 / (ref^2 + 0.01)))."""
import numpy as np
import pytest

from helpers import scene

pytestmark = pytest.mark.gpu

W, H, SURFACES = 96, 64, 6


def rel_mse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 0.01)))


@pytest.fixture(scope="module")
def room():
    import kodanuki_gb300 as K
    sc = scene("room_small")
    with K.Backend(0) as b:
        b.load(sc)
        b.build(5, 10, 64)
        ref = b.render(W, H, 4096, surfaces=SURFACES, seed=101)
        yield b, sc, ref


def trained_guide(b, sc, frames=8, spp=16):
    import kodanuki_gb300 as K
    lo = np.asarray(sc.region_lower, np.float64)
    hi = lo + np.asarray(sc.region_size, np.float64)
    g = K.Guide(0, table_log2=16, seed=2, region=(lo, hi), batch=4096, max_steps=64)
    b.set_guide(g, 0.5, K.GUIDE_TRAIN)
    for k in range(frames):
        b.render(W, H, spp, surfaces=SURFACES, seed=1000 + k)
    return g


def test_guided_frame_is_unbiased_and_gains(room):
    import kodanuki_gb300 as K
    b, sc, ref = room
    plain = b.render(W, H, 32, surfaces=SURFACES, seed=7)
    g = trained_guide(b, sc)
    try:
        b.set_guide(g, 0.5, K.GUIDE_SAMPLE)
        guided = b.render(W, H, 32, surfaces=SURFACES, seed=7)
        many = b.render(W, H, 1024, surfaces=SURFACES, seed=8)
    finally:
        b.set_guide(None)
        g.close()
    assert np.isfinite(guided).all()
    # the same expectation: the guided frame at 1024 spp against the plain 4096-spp frame
    for c in range(3):
        assert abs(many[..., c].mean() / ref[..., c].mean() - 1) < 0.01, (c, many[..., c].mean(), ref[..., c].mean())
    rp, rg = rel_mse(plain, ref), rel_mse(guided, ref)
    assert rg < rp / 1.2, (rp, rg)


def test_training_while_guided_and_plain_frames_unchanged(room):
    """A frame both guided and training runs; a context without a guide
    draws the same frame as before the guide was attached."""
    import kodanuki_gb300 as K
    b, sc, _ = room
    before = b.render(32, 24, 4, surfaces=SURFACES, seed=5)
    g = trained_guide(b, sc, frames=2, spp=4)
    try:
        b.set_guide(g, 0.5, K.GUIDE_SAMPLE | K.GUIDE_TRAIN)
        img = b.render(32, 24, 4, surfaces=SURFACES, seed=5)
        assert np.isfinite(img).all()
    finally:
        b.set_guide(None)
        g.close()
    after = b.render(32, 24, 4, surfaces=SURFACES, seed=5)
    assert np.array_equal(before, after)


def test_select_keeps_a_useful_guide_and_drops_a_harmful_one(room):
    """kdn_guide_select's pilots keep the trained guide on the room (it
    gains there) and turn off a guide trained to point into the surfaces."""
    import kodanuki_gb300 as K
    b, sc, _ = room
    g = trained_guide(b, sc)
    try:
        b.set_guide(g, 0.5, K.GUIDE_SAMPLE)
        keep, pc, gc = b.guide_select(W, H, 16, surfaces=SURFACES, seed=21)
        assert keep and gc < pc, (pc, gc)
    finally:
        b.set_guide(None)
        g.close()
    lo = np.asarray(sc.region_lower, np.float64)
    hi = lo + np.asarray(sc.region_size, np.float64)
    with K.Guide(0, table_log2=16, seed=4, region=(lo, hi)) as bad:
        rng = np.random.default_rng(1)
        n = 1 << 15
        p = rng.uniform(lo, hi, size=(n, 3))
        nv = np.tile([0.0, 0.0, 1.0], (n, 1))
        d = np.tile([0.0, 0.0, -1.0], (n, 1))  # straight into the surface
        bad.train(np.concatenate([p, nv, d, np.ones((n, 1))], axis=1).astype(np.float32), batch=4096, steps=200)
        b.set_guide(bad, 0.9, K.GUIDE_SAMPLE)
        keep, pc, gc = b.guide_select(W, H, 16, surfaces=SURFACES, seed=21)
        assert not keep and gc > pc, (pc, gc)
        b.set_guide(None)
