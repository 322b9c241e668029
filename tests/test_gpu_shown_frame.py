"""The denoised frame of kdn_render (KDN_FRAME_DENOISE), through the C ABI.

It is three pieces, each checked against the oracle:

1. the first surfaces through the pixel centres (core/surfaces.cpp:133
   tracedSurfaces): leaves agree for all but 1% of pixels (FP32 against
   double camera rays part ways at silhouettes), and where they agree the
   FP16 distance, normal and albedo are within FP16 rounding of the
   oracle's;
2. the temporal state of a still camera (temporal.cpp:797 freshBlend, :835
   heldBlend): colour the running mean, moment the blended squared
   luminance of each frame, length the frames drawn;
3. the a-trous denoiser over them: the frame kdn_render returns is within
   1e-3 of the oracle's denoiser (itself pinned to the reference's
   denoisedFrame) run on the same pixel means and surfaces.
"""
import os

import numpy as np
import pytest

from helpers import scene

pytestmark = pytest.mark.gpu

BUILD = dict(min_depth=5, max_depth=10, split_steps=64)


@pytest.fixture(scope="module")
def backend():
    import kodanuki_gb300 as K
    b = K.Backend(0)
    yield b
    b.close()


def luminance(rgb):
    rgb = np.asarray(rgb, np.float64)
    return 0.2126 * rgb[..., 0] + 0.7152 * rgb[..., 1] + 0.0722 * rgb[..., 2]


def oracle_denoised(sc, w, h, colour, moment, length, surf):
    import oracle.port as op
    n = w * h
    return op.denoise(w, h, 0, op.lens_of(sc, w, h), colour.reshape(n, 3), moment.reshape(n), np.full(n, length, np.float32),
                      surf["distance"].reshape(n).astype(np.float32), surf["normal"].reshape(n, 3).astype(np.float64),
                      surf["leaf"].reshape(n), surf["albedo"].reshape(n, 3).astype(np.float64)).reshape(h, w, 3)


@pytest.mark.parametrize("name", ["c2_small", "room_small"])
def test_surfaces_match_oracle(backend, name):
    import oracle.port as op
    sc = scene(name)
    h, w = sc.render["height"], sc.render["width"]
    backend.load(sc)
    backend.build(**BUILD)
    backend.render(w, h, 1, seed=1, denoise=True)
    got = backend.frame_surfaces(w, h)
    want = op.traced_surfaces(sc, w, h, BUILD)
    leaf = got["leaf"].reshape(-1)
    same = leaf == want["leaf"]
    print(f"{name}: leaves agree on {same.mean():.4f} of pixels")
    assert same.mean() >= 0.99
    hit = same & (leaf != 0xFFFFFFFF)
    assert hit.any()
    d_got = got["distance"].reshape(-1).astype(np.float64)[hit]
    d_want = want["distance"][hit].astype(np.float64)
    assert np.all(np.abs(d_got - d_want) <= 2e-3 * d_want + 1e-4)
    n_err = np.abs(got["normal"].reshape(-1, 3).astype(np.float64)[hit] - want["normal"][hit])
    a_err = np.abs(got["albedo"].reshape(-1, 3).astype(np.float64)[hit] - want["albedo"][hit])
    assert np.quantile(n_err.max(1), 0.99) <= 2e-3
    assert np.quantile(a_err.max(1), 0.99) <= 2e-3
    missed = (leaf == 0xFFFFFFFF) & same
    assert np.all(np.isinf(got["distance"].reshape(-1)[missed].astype(np.float32)))
    assert np.all(got["albedo"].reshape(-1, 3)[missed] == 0)


@pytest.mark.parametrize("name", ["c2_small", "room_small"])
def test_denoised_frame_is_the_denoiser_over_the_frame(backend, name):
    sc = scene(name)
    h, w = sc.render["height"], sc.render["width"]
    spp = 8
    backend.load(sc)
    backend.build(**BUILD)
    means = backend.render(w, h, spp, seed=4)
    shown = backend.render(w, h, spp, seed=4, denoise=True)
    surf = backend.frame_surfaces(w, h)
    want = oracle_denoised(sc, w, h, means.astype(np.float64), luminance(means) ** 2, 1.0, surf)
    err = np.abs(shown.astype(np.float64) - want)
    print(f"{name}: denoised max |gpu - oracle| {err.max():.3e}; noise {np.abs(means - shown).mean():.3e}")
    assert np.isfinite(shown).all()
    assert err.max() <= 1e-3
    assert not np.allclose(shown, means)


def test_denoised_history_of_two_frames(backend):
    """Two accumulated calls: colour the mean of both, moment the two frames'
    squared luminance blended half and half, history length 2."""
    sc = scene("c2_small")
    h, w = sc.render["height"], sc.render["width"]
    spp = 4
    backend.load(sc)
    backend.build(**BUILD)
    one = backend.render(w, h, spp, seed=9, first=0).astype(np.float64)
    two = backend.render(w, h, spp, seed=9, first=spp).astype(np.float64)
    backend.render(w, h, spp, seed=9, first=0, denoise=True)
    shown = backend.render(w, h, spp, seed=9, first=spp, accumulate=True, denoise=True)
    surf = backend.frame_surfaces(w, h)
    moment = 0.5 * luminance(one) ** 2 + 0.5 * luminance(two) ** 2
    want = oracle_denoised(sc, w, h, (one + two) / 2, moment, 2.0, surf)
    err = np.abs(shown.astype(np.float64) - want)
    print(f"two frames: denoised max |gpu - oracle| {err.max():.3e}")
    assert err.max() <= 1e-3


def test_surfaces_need_a_denoised_frame(backend):
    import kodanuki_gb300 as K
    sc = scene("room_small")
    backend.load(sc)
    backend.build(**BUILD)
    backend.render(16, 16, 1, seed=1)
    with pytest.raises(K.KdnError) as e:
        backend.frame_surfaces(16, 16)
    assert e.value.status == K.KDN_NOT_READY
