"""The serving loop's host logic (include/kdn.h kdn_serve_*) on contexts
without a device: every request ends in KDN_NO_DEVICE, which is enough to
check tickets, sessions (their frames in order, one at a time), admission,
cancelling and the latency counts; and the rules of contexts that share a
scene's world (kdn_open_sharing)."""
import ctypes

import pytest

import kodanuki_gb300 as K
from helpers import host_backend, scene

BUILD = dict(min_depth=3, max_depth=6, split_steps=64)


@pytest.fixture(scope="module")
def built():
    b = host_backend()
    b.load(scene("c1_small"))
    b.build(**BUILD)
    yield b
    b.close()


def test_sharing_context_rules(built):
    L = K.library()
    shared = built.share()
    # the scene can be neither rebuilt nor closed while it is shared
    assert L.kdn_build(built.handle, None) == K.KDN_BAD_ARG
    assert L.kdn_close(built.handle) == K.KDN_BAD_ARG
    # a sharing context cannot build or be shared itself
    assert L.kdn_build(shared.handle, None) == K.KDN_BAD_ARG
    h = ctypes.c_void_p()
    assert L.kdn_open_sharing(shared.handle, 0, ctypes.byref(h)) == K.KDN_BAD_ARG
    # it has the scene's world
    assert shared.world_stats() == built.world_stats()
    shared.set_frame_budget(1 << 26)
    shared.close()
    # once closed, the scene may be rebuilt
    built.build(**BUILD)


def test_unbuilt_scene_cannot_be_shared():
    b = host_backend()
    b.load(scene("c1_small"))
    h = ctypes.c_void_p()
    assert K.library().kdn_open_sharing(b.handle, 0, ctypes.byref(h)) == K.KDN_NOT_READY
    b.close()


def test_requests_and_sessions_without_a_device(built):
    with K.Server(device=-1, slots=3) as srv:
        sid = srv.add_scene(built)
        tickets = [srv.submit(sid, 32, 24, 4, seed=k) for k in range(6)]
        session = [srv.submit(sid, 16, 16, 1, session=7, interactive=True) for _ in range(4)]
        results = [srv.wait(t) for t in tickets + session]
        assert all(st == K.KDN_NO_DEVICE for st, _, _ in results)
        # a session's frames are admitted one at a time, in order
        assert [r[1]["frame"] for r in results[6:]] == [0, 1, 2, 3]
        assert all(r[1]["latency_ms"] >= r[1]["render_ms"] >= 0 for r in results)
        # latency counts only completed requests
        assert srv.latency()["count"] == 0
        srv.end_session(7)
        with pytest.raises(K.KdnError):
            srv.end_session(7)


def test_bad_requests_are_refused(built):
    with K.Server(device=-1, slots=2) as srv:
        sid = srv.add_scene(built)
        with pytest.raises(K.KdnError) as e:
            srv.submit(sid + 1, 8, 8, 1)
        assert e.value.status == K.KDN_BAD_ARG
        with pytest.raises(K.KdnError) as e:
            srv.submit(sid, 8, 8, 0)
        assert e.value.status == K.KDN_BAD_ARG
        srv.wait(srv.submit(sid, 8, 8, 1, session=3))
        other = host_backend()
        other.load(scene("room_small"))
        other.build(**BUILD)
        sid2 = srv.add_scene(other)
        with pytest.raises(K.KdnError) as e:  # a session draws one scene
            srv.submit(sid2, 8, 8, 1, session=3)
        assert e.value.status == K.KDN_BAD_ARG
        srv.end_session(3)
    other.close()


def test_cancel_queued(built):
    with K.Server(device=-1, slots=1) as srv:
        sid = srv.add_scene(built)
        tickets = [srv.submit(sid, 64, 64, 8, seed=k) for k in range(40)]
        cancelled = srv.cancel_queued()
        statuses = [srv.wait(t)[0] for t in tickets]
        assert statuses.count(K.KDN_NOT_READY) == cancelled
        assert all(s in (K.KDN_NOT_READY, K.KDN_NO_DEVICE) for s in statuses)


def test_server_options():
    L = K.library()
    h = ctypes.c_void_p()
    assert L.kdn_serve_open(ctypes.byref(K.ServeOptions(-1, 0, 0)), ctypes.byref(h)) == K.KDN_BAD_ARG
    assert L.kdn_serve_open(ctypes.byref(K.ServeOptions(-1, 65, 0)), ctypes.byref(h)) == K.KDN_BAD_ARG
