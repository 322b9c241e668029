"""Frames at a film factor above 1 (kdn_frame.factor / .phase), through the
C ABI.

1. The phased draws: at factor 2 each drawn pixel's samples aim at the
   shown pixel of the phase (plugins/transport/paths/trace.cpp:93
   phasedDraw).  The record's light of a factor-2 frame (the drawn frame's
   pixel means) against the oracle renderer drawing the same phase, 12 seeds
   each, to the bar of the frame tests (per-pixel z beyond 3 for at most 1%
   of pixel channels, every channel's image mean within 3 standard errors);
   and the phases differ from one another where the frame has detail.
2. The shown frame: a sequence of factor-2 frames in Bayer order (a first
   frame, still frames, a moved camera) is the reference's chain temporal +
   a-trous + upscale run by the oracle (each member pinned to the
   reference's own) on the frame's own record and G-buffer, within 1e-4
   relative for 99.9% of shown pixels and 1e-3 for all.
3. The other chains: mean + upsample, temporal + a-trous + upsample, and
   the temporal member alone.
4. Refusals: a factor above 1 with no chain to the shown size, a size that
   is not a multiple of the factor, a phase past the factor's square, a
   factor above 4.
"""
import os

import numpy as np
import pytest

from helpers import scene

pytestmark = pytest.mark.gpu

BUILD = dict(min_depth=5, max_depth=10, split_steps=64)
SEEDS = list(range(1, 13))
THREADS = os.cpu_count() or 4


@pytest.fixture(scope="module")
def backend():
    import kodanuki_gb300 as K
    b = K.Backend(0)
    yield b
    b.close()


def zscores(a, b):
    z = (a.mean(0) - b.mean(0)) / np.sqrt(a.var(0, ddof=1) / len(a) + b.var(0, ddof=1) / len(b) + 1e-12)
    ca, cb = a.mean(axis=(1, 2)), b.mean(axis=(1, 2))
    cz = (ca.mean(0) - cb.mean(0)) / np.sqrt(ca.var(0, ddof=1) / len(ca) + cb.var(0, ddof=1) / len(cb))
    return z, cz


@pytest.mark.parametrize("phase", [0, 3])
def test_phased_record_matches_oracle(backend, phase):
    import oracle.port as op
    sc = scene("c1_small")
    w, h, surfaces = int(sc.render["width"]), int(sc.render["height"]), int(sc.render["surfaces"])
    factor, spp = 2, 16
    dw, dh = w // factor, h // factor
    backend.load(sc)
    backend.build(**BUILD)
    gpu = []
    for s in SEEDS:
        backend.render(w, h, spp, surfaces=surfaces, seed=s, denoise=True, restart=True, factor=factor, phase=phase)
        gpu.append(backend.frame_record(dw, dh)["light"].astype(np.float64))
    gpu = np.stack(gpu)
    oracle = np.stack([op.render_band(sc, dw, dh, spp, surfaces, s, 0, dh, THREADS, BUILD, factor=factor, phase=phase) / spp for s in SEEDS])
    z, cz = zscores(gpu, oracle)
    far = float((np.abs(z) > 3).mean())
    other = np.stack([op.render_band(sc, dw, dh, spp, surfaces, s, 0, dh, THREADS, BUILD, factor=factor, phase=3 - phase) / spp for s in SEEDS])
    z_other, _ = zscores(gpu, other)
    far_other = float((np.abs(z_other) > 3).mean())
    print(f"phase {phase}: channel z {cz}, far px {far:.4f}; against the other phase's draws far px {far_other:.4f}")
    assert far <= 0.01, far
    assert np.all(np.abs(cz) < 3), cz
    assert far_other > 3 * max(far, 0.005), far_other


def oracle_chain(w, h, factor, phase, before_phase, record, gbuffer, t_state, u_state, lens_now, lens_before, kept, moved):
    """The oracle's temporal member on the drawn grid, its denoiser, then its
    upscale member to the shown size; the states after and the shown frame."""
    import oracle.port as op
    dw, dh = w // factor, h // factor
    rec = {k: np.asarray(v).reshape(-1, *np.asarray(v).shape[2:]) for k, v in record.items()}
    g = {k: np.asarray(v).reshape(-1, *np.asarray(v).shape[2:]) for k, v in gbuffer.items()}
    first = {k: rec[k].astype(np.float32) for k in ("distance", "normal", "albedo")}
    first["leaf"] = rec["leaf"]
    centre = {k: g[k].astype(np.float32) for k in ("distance", "normal", "albedo")}
    centre["leaf"] = g["leaf"]
    drawn_lens = np.array(lens_now, np.float64)
    state, _ = op.temporal(dw, dh, moved, False, kept, drawn_lens, lens_before, rec["light"].astype(np.float64), first, centre, t_state,
                           (factor, phase, factor, before_phase))
    internal = op.denoise(dw, dh, 1, drawn_lens, state["colour"], state["moment"], state["length"], state["distance"], state["normal"],
                          state["leaf"], state["albedo"]).reshape(-1, 3)
    up_kept = u_state is not None
    settling, count = op.upscale_settling(up_kept, moved, u_state[2] if up_kept else False, u_state[3] if up_kept else 0)
    colour, depth, image = op.upscale(w, h, factor, phase, moved, up_kept, settling, lens_now, lens_before, internal, centre["distance"],
                                      u_state[0] if up_kept else None, u_state[1] if up_kept else None)
    return state, (colour, depth, moved, count), image.reshape(h, w, 3)


def check(name, shown, want):
    err = np.abs(shown.astype(np.float64) - want)
    rel = err / (np.abs(want) + 1e-2)
    print(f"{name}: shown max |gpu - oracle| {err.max():.3e}, within 1e-3 relative {np.mean(rel.max(axis=2) <= 1e-3):.4f}, "
          f"relative p50 {np.median(rel):.1e} p99 {np.quantile(rel, 0.99):.1e}")
    assert np.isfinite(shown).all()
    assert np.mean(rel.max(axis=2) <= 1e-4) >= 0.999
    assert np.all(rel <= 1e-3)
    assert np.median(err) <= 1e-6


def test_shown_frames_at_factor_2(backend):
    import kodanuki_gb300 as K
    import oracle.port as op
    sc = scene("c2_small")
    factor, spp = 2, 4
    # drawn at the scene's own size (64 x 36, the grid of the factor-1
    # shown-frame test), shown at twice it
    dw, dh = int(sc.render["width"]), int(sc.render["height"])
    w, h = dw * factor, dh * factor
    backend.load(sc)
    backend.build(**BUILD)
    lens = op.lens_of(sc, dw, dh)
    blocks = K.scene_blocks(sc)
    cam = blocks["shot.camera"].copy()
    moved_cam = cam.copy()
    moved_cam["eye"][0][0] += 0.05
    moved_cam["target"][0][0] += 0.05
    eye = np.asarray(moved_cam["eye"][0], np.float64)
    fw = np.asarray(moved_cam["target"][0], np.float64) - eye
    fw /= np.linalg.norm(fw)
    rt = np.cross(fw, np.asarray(moved_cam["up"][0], np.float64))
    rt /= np.linalg.norm(rt)
    lens2 = np.concatenate([eye, fw, rt, np.cross(rt, fw), lens[12:14]])
    # (camera, lens, kept, moved) a frame; the phases in Bayer order
    plan = [(cam, lens, False, False), (cam, lens, True, False), (cam, lens, True, False), (moved_cam, lens2, True, True),
            (moved_cam, lens2, True, False)]
    t_state, u_state, before_lens, before_phase = None, None, lens, 0
    # a frame without the chain first: the sequence starts with no history
    # (else the lens of the module's frames before would count as a move)
    backend.render(dw, dh, 1, seed=1)
    try:
        for k, (camera, lens_now, kept, moved) in enumerate(plan):
            phase = K.BAYER[factor][k % 4]
            backend.upload("shot.camera", camera)
            shown = backend.render(w, h, spp, seed=7, first=k * spp, denoise=True, restart=k == 0, factor=factor, phase=phase)
            assert shown.shape == (h, w, 3)
            record, gbuffer = backend.frame_record(dw, dh), backend.frame_surfaces(dw, dh)
            t_state, u_state, want = oracle_chain(w, h, factor, phase, before_phase, record, gbuffer, t_state if kept else None,
                                                  u_state if kept else None, lens_now, before_lens, kept, moved)
            check(f"frame {k} phase {phase} kept {kept} moved {moved}", shown, want)
            before_lens, before_phase = lens_now, phase
    finally:
        backend.upload("shot.camera", blocks["shot.camera"])


def test_other_chains(backend):
    """The chain mean + upsample at factor 2 (KDN_FRAME_UPSAMPLE without
    KDN_FRAME_DENOISE) shows the drawn frame's pixel means blown up by the
    oracle's upsample member (pinned to the reference's upsampledImage);
    temporal + a-trous + upsample shows the chain's drawn frame blown up; the
    chain `temporal` alone (KDN_FRAME_TEMPORAL) shows the temporal member's
    light, the oracle's on the frame's own record and G-buffer."""
    import oracle.port as op
    sc = scene("c2_small")
    factor, spp = 2, 4
    dw, dh = int(sc.render["width"]), int(sc.render["height"])
    w, h = dw * factor, dh * factor
    backend.load(sc)
    backend.build(**BUILD)
    shown = backend.render(w, h, spp, seed=3, factor=factor, phase=2, upsample=True)
    backend.render(w, h, spp, seed=3, factor=factor, phase=2, denoise=True, restart=True)
    means = backend.frame_record(dw, dh)["light"].reshape(-1, 3)
    want = op.upsample(w, h, factor, means).reshape(h, w, 3)
    assert np.allclose(shown, want, rtol=1e-6, atol=1e-7)
    # temporal + a-trous + upsample: a first frame, so the chain's drawn frame
    # is the oracle's temporal and denoiser on the record (as the shown-frame tests)
    up = backend.render(w, h, spp, seed=3, factor=factor, phase=2, denoise=True, restart=True, upsample=True)
    record, gbuffer = backend.frame_record(dw, dh), backend.frame_surfaces(dw, dh)
    lens = op.lens_of(sc, dw, dh)
    rec = {k: np.asarray(v).reshape(-1, *np.asarray(v).shape[2:]) for k, v in record.items()}
    g = {k: np.asarray(v).reshape(-1, *np.asarray(v).shape[2:]) for k, v in gbuffer.items()}
    first = {k: rec[k].astype(np.float32) for k in ("distance", "normal", "albedo")}
    first["leaf"] = rec["leaf"]
    centre = {k: g[k].astype(np.float32) for k in ("distance", "normal", "albedo")}
    centre["leaf"] = g["leaf"]
    state, _ = op.temporal(dw, dh, False, False, False, lens, lens, rec["light"].astype(np.float64), first, centre, None, (factor, 2, factor, 2))
    internal = op.denoise(dw, dh, 1, lens, state["colour"], state["moment"], state["length"], state["distance"], state["normal"], state["leaf"],
                          state["albedo"]).reshape(-1, 3)
    check("temporal + a-trous + upsample", up, op.upsample(w, h, factor, internal).reshape(h, w, 3))
    # the temporal member alone, at factor 1
    alone = backend.render(dw, dh, spp, seed=5, denoise=True, restart=True, temporal_only=True)
    record, gbuffer = backend.frame_record(dw, dh), backend.frame_surfaces(dw, dh)
    rec = {k: np.asarray(v).reshape(-1, *np.asarray(v).shape[2:]) for k, v in record.items()}
    g = {k: np.asarray(v).reshape(-1, *np.asarray(v).shape[2:]) for k, v in gbuffer.items()}
    first = {k: rec[k].astype(np.float32) for k in ("distance", "normal", "albedo")}
    first["leaf"] = rec["leaf"]
    centre = {k: g[k].astype(np.float32) for k in ("distance", "normal", "albedo")}
    centre["leaf"] = g["leaf"]
    _, image = op.temporal(dw, dh, False, False, False, lens, lens, rec["light"].astype(np.float64), first, centre, None)
    check("temporal alone", alone, image.reshape(dh, dw, 3).astype(np.float64))


def test_film_factor_refusals(backend):
    import kodanuki_gb300 as K
    sc = scene("room_small")
    backend.load(sc)
    backend.build(**BUILD)
    for kwargs in (dict(factor=2, denoise=False), dict(factor=2, denoise=True, width=33), dict(factor=2, denoise=True, phase=4),
                   dict(factor=5, denoise=True, width=40, height=40)):
        args = dict(width=32, height=32, phase=0)
        args.update(kwargs)
        with pytest.raises(K.KdnError) as e:
            backend.render(args.pop("width"), args.pop("height"), 1, **args)
        assert e.value.status == K.KDN_BAD_ARG, kwargs
