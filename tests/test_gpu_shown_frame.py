"""The shown frame of kdn_render (KDN_FRAME_DENOISE), through the C ABI.

It is the reference's reconstruction chain temporal + a-trous over the
frame, in three pieces, each checked against the oracle:

1. the G-buffer through the pixel centres (core/surfaces.cpp:133
   tracedSurfaces): leaves agree for all but 1% of pixels (FP32 against
   double camera rays part ways at silhouettes), and where they agree the
   FP16 distance, normal and albedo are within FP16 rounding of the
   oracle's;
2. the record: each pixel's light of the call equals the pixel means of the
   same call drawn without the flag;
3. the temporal member and the a-trous denoiser over the record and the
   G-buffer: the frame kdn_render returns is within 1e-4 relative of the
   oracle's temporal member (pinned to the reference's temporalFrame) and denoiser
   (pinned to its denoisedFrame) run on the frame's own record and
   G-buffer, for a first frame, a still second frame and a moved one.
"""
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


def flat(d: dict) -> dict:
    return {k: np.asarray(v).reshape(-1, *np.asarray(v).shape[2:]) for k, v in d.items()}


def oracle_step(sc, w, h, record, gbuffer, before, lens_now, lens_before, kept, moved):
    """The oracle's temporal member, then its denoiser on the state."""
    import oracle.port as op
    rec = flat(record)
    g = flat(gbuffer)
    first = {k: rec[k].astype(np.float32) for k in ("distance", "normal", "albedo")}
    first["leaf"] = rec["leaf"]
    centre = {k: g[k].astype(np.float32) for k in ("distance", "normal", "albedo")}
    centre["leaf"] = g["leaf"]
    state, _ = op.temporal(w, h, moved, False, kept, lens_now, lens_before, rec["light"].astype(np.float64), first, centre, before)
    shown = op.denoise(w, h, 1, lens_now, state["colour"], state["moment"], state["length"], state["distance"], state["normal"], state["leaf"],
                       state["albedo"]).reshape(h, w, 3)
    return state, shown


def check(name, shown, want):
    err = np.abs(shown.astype(np.float64) - want)
    rel = err / (np.abs(want) + 1e-2)
    print(f"{name}: denoised max |gpu - oracle| {err.max():.3e}, within 1e-3 relative {np.mean(rel <= 1e-3):.4f}")
    assert np.isfinite(shown).all()
    assert np.mean(rel.max(axis=2) <= 1e-4) >= 0.999
    assert np.all(rel <= 1e-3)
    assert np.median(err) <= 1e-6


@pytest.mark.parametrize("name", ["c2_small", "room_small", "patterns_small"])
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
def test_shown_frame_is_temporal_and_denoiser(backend, name):
    import oracle.port as op
    sc = scene(name)
    h, w = sc.render["height"], sc.render["width"]
    spp = 8
    backend.load(sc)
    backend.build(**BUILD)
    means = backend.render(w, h, spp, seed=4)
    shown = backend.render(w, h, spp, seed=4, denoise=True)
    record = backend.frame_record(w, h)
    gbuffer = backend.frame_surfaces(w, h)
    assert np.allclose(record["light"], means, rtol=1e-6, atol=1e-7)
    lens = op.lens_of(sc, w, h)
    _, want = oracle_step(sc, w, h, record, gbuffer, None, lens, lens, False, False)
    check(name, shown, want)
    assert not np.allclose(shown, means)


def test_shown_frames_still_then_moved(backend):
    """Three denoised frames: a first, a still second (its history the
    first's), then the camera moved (the history reprojected)."""
    import kodanuki_gb300 as K
    import oracle.port as op
    sc = scene("c2_small")
    h, w = sc.render["height"], sc.render["width"]
    spp = 4
    backend.load(sc)
    backend.build(**BUILD)
    lens = op.lens_of(sc, w, h)
    shown0 = backend.render(w, h, spp, seed=9, first=0, denoise=True, restart=True)
    rec0, g0 = backend.frame_record(w, h), backend.frame_surfaces(w, h)
    state0, want0 = oracle_step(sc, w, h, rec0, g0, None, lens, lens, False, False)
    check("first", shown0, want0)
    shown1 = backend.render(w, h, spp, seed=9, first=spp, accumulate=True, denoise=True)
    rec1, g1 = backend.frame_record(w, h), backend.frame_surfaces(w, h)
    state1, want1 = oracle_step(sc, w, h, rec1, g1, state0, lens, lens, True, False)
    check("still", shown1, want1)
    # move the camera a little sideways
    blocks = K.scene_blocks(sc)
    cam = blocks["shot.camera"].copy()
    cam["eye"][0][0] += 0.05
    cam["target"][0][0] += 0.05
    backend.upload("shot.camera", cam)
    moved_scene = sc
    eye = np.asarray(cam["eye"][0], np.float64)
    fw = np.asarray(cam["target"][0], np.float64) - eye
    fw /= np.linalg.norm(fw)
    rt = np.cross(fw, np.asarray(cam["up"][0], np.float64))
    rt /= np.linalg.norm(rt)
    lens2 = np.concatenate([eye, fw, rt, np.cross(rt, fw), lens[12:14]])
    try:
        shown2 = backend.render(w, h, spp, seed=9, first=2 * spp, denoise=True)
        rec2, g2 = backend.frame_record(w, h), backend.frame_surfaces(w, h)
        _, want2 = oracle_step(moved_scene, w, h, rec2, g2, state1, lens2, lens, True, True)
        check("moved", shown2, want2)
    finally:
        backend.upload("shot.camera", blocks["shot.camera"])


def test_surfaces_need_a_denoised_frame(backend):
    import kodanuki_gb300 as K
    sc = scene("room_small")
    backend.load(sc)
    backend.build(**BUILD)
    backend.render(16, 16, 1, seed=1)
    with pytest.raises(K.KdnError) as e:
        backend.frame_surfaces(16, 16)
    assert e.value.status == K.KDN_NOT_READY
    with pytest.raises(K.KdnError) as e:
        backend.frame_record(16, 16)
    assert e.value.status == K.KDN_NOT_READY
