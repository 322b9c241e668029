"""The march budget (kdn_set_march_budget): a ray that has taken its budget
of march steps in one trace launch stops with its march state and goes on in
the next launch, and a path whose shadow line is still marching waits for it.
The march is deterministic and each path's radiance takes its terms in the
same order, so a frame drawn with any budget is the frame drawn without one,
to the bit.  Tiny budgets carry nearly every ray through many launches (and
so exercise the rounds that finish the paths that waited)."""
import numpy as np
import pytest

from helpers import scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name, sampler", [("c2_small", None), ("room_small", None), ("glass_small", None), ("rough_small", None),
                                           ("lamps_small", "each_lamp_first"), ("scatter_small", None)])
def test_frames_with_a_budget_equal_frames_without(name, sampler):
    """With --use sampler=each_lamp_first a path holds up to five lines at
    its first vertex, each carried on its own; in scatter_small paths stand
    on collisions inside scattering bodies between their surfaces."""
    import kodanuki_gb300 as K
    sc = scene(name)
    extra = {sampler: True} if sampler else {}
    w, h = int(sc.render["width"]), int(sc.render["height"])
    surfaces = int(sc.render["surfaces"])
    with K.Backend(0) as b:
        b.load(sc)
        b.build(5, 10, 64)
        b.set_march_budget(0)
        plain = b.render(w, h, 8, surfaces=surfaces, seed=3, **extra)
        st0 = b.frame_stats()
        assert st0.carried_rays == 0
        for budget in (1, 5, 64):
            b.set_march_budget(budget)
            img = b.render(w, h, 8, surfaces=surfaces, seed=3, **extra)
            st = b.frame_stats()
            assert np.array_equal(img, plain), (budget, np.abs(img - plain).max())
            assert st.carried_rays > 0, budget
            assert st.segments == st0.segments, (budget, st.segments, st0.segments)
            assert st.capped_rays == st0.capped_rays and st.longest_march == st0.longest_march


def test_denoised_and_accumulated_frames_with_a_budget():
    """The shown frame (its surfaces pass, temporal member and denoiser) and
    frames accumulated over calls are the same with a budget."""
    import kodanuki_gb300 as K
    sc = scene("c2_small")
    w, h = int(sc.render["width"]), int(sc.render["height"])
    surfaces = int(sc.render["surfaces"])
    out = {}
    for budget in (0, 3):
        with K.Backend(0) as b:
            b.load(sc)
            b.build(5, 10, 64)
            b.set_march_budget(budget)
            frames = [b.render(w, h, 4, surfaces=surfaces, seed=11 + k, first=4 * k, accumulate=k > 0, denoise=True) for k in range(3)]
            frames.append(b.render(w, h, 4, surfaces=surfaces, seed=20, first=12, accumulate=True))
            out[budget] = np.stack(frames)
    assert np.array_equal(out[0], out[3]), np.abs(out[0] - out[3]).max()


def test_budget_above_the_march_cap_is_no_budget():
    import kodanuki_gb300 as K
    sc = scene("c1_small")
    with K.Backend(0) as b:
        b.load(sc)
        b.build(5, 10, 64)
        b.set_march_budget(1 << 16)
        b.render(24, 24, 2, surfaces=4, seed=1)
        assert b.frame_stats().carried_rays == 0
