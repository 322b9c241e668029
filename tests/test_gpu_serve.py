"""The serving loop on the device (include/kdn.h kdn_serve_*).

1. Requests of three scenes, four sizes, several spp, some interactive and
   some denoised, submitted together and drawn side by side on four slots:
   each result is bit-for-bit the same request drawn alone (kdn_render on
   a context of the scene).
2. A progressive session (1 spp a frame, denoised, its accumulation and
   history resident in the server) equals the same frames accumulated on a
   plain context, frame by frame.
"""
import numpy as np
import pytest

from helpers import scene

pytestmark = pytest.mark.gpu

BUILD = dict(min_depth=5, max_depth=10, split_steps=64)
NAMES = ("c1_small", "room_small", "glow_small")


@pytest.fixture(scope="module")
def scenes():
    import kodanuki_gb300 as K
    out = {}
    for name in NAMES:
        b = K.Backend(0)
        b.load(scene(name))
        b.build(**BUILD)
        out[name] = b
    yield out
    for b in out.values():
        b.close()


def test_mixed_requests_equal_alone(scenes):
    import kodanuki_gb300 as K
    rng = np.random.default_rng(5)
    sizes = [(64, 48), (96, 64), (160, 90), (48, 48)]
    requests = []
    for k in range(14):
        name = NAMES[k % 3]
        w, h = sizes[k % 4]
        requests.append(dict(name=name, w=w, h=h, spp=int(rng.choice([1, 2, 4, 8])), seed=100 + k, interactive=k % 4 == 1, denoise=k % 5 == 2))
    alone = [scenes[r["name"]].render(r["w"], r["h"], r["spp"], surfaces=8, seed=r["seed"], denoise=r["denoise"], restart=True) for r in requests]
    with K.Server(0, slots=4) as srv:
        ids = {name: srv.add_scene(b) for name, b in scenes.items()}
        tickets = [srv.submit(ids[r["name"]], r["w"], r["h"], r["spp"], surfaces=8, seed=r["seed"], denoise=r["denoise"], interactive=r["interactive"])
                   for r in requests]
        results = [srv.wait(t) for t in tickets]
        lat = srv.latency()
        print(f"latency p50 {lat['p50_ms']:.2f} ms p99 {lat['p99_ms']:.2f} ms over {lat['count']}")
    for r, want, (status, served, got) in zip(requests, alone, results):
        assert status == K.KDN_OK
        assert served["latency_ms"] >= served["render_ms"] > 0
        assert np.array_equal(got, want), r
    assert lat["count"] == len(requests)


def test_session_equals_accumulated_frames(scenes):
    import kodanuki_gb300 as K
    b = scenes["room_small"]
    w, h = 64, 48
    want = [b.render(w, h, 1, surfaces=8, seed=9, first=k, accumulate=k > 0, denoise=True, restart=k == 0) for k in range(4)]
    with K.Server(0, slots=3) as srv:
        sid = srv.add_scene(b)
        # a background request of another scene alongside the session
        other = srv.add_scene(scenes["c1_small"])
        bg = srv.submit(other, 160, 90, 8, surfaces=8, seed=3)
        tickets = [srv.submit(sid, w, h, 1, surfaces=8, seed=9, denoise=True, interactive=True, session=42) for _ in range(4)]
        got = [srv.wait(t) for t in tickets]
        assert srv.wait(bg)[0] == K.KDN_OK
        srv.end_session(42)
    for k, (status, served, img) in enumerate(got):
        assert status == K.KDN_OK
        assert served["frame"] == k
        assert np.array_equal(img, want[k]), k
