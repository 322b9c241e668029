"""The oracle's temporal member against the reference's temporalFrame.

tests/golden/temporal.npz holds a seeded sequence of frames over config 2's
small scene (a still camera, then a moving one, then still again), each
run through the reference's own temporalFrame with the state the frame
before left (plugins/reconstruction/temporal/temporal.cpp:1001, with a
G-buffer, as before the a-trous denoiser); tests/golden/temporal_factor2.npz
the same at a film factor of 2, the phases in Bayer order (each frame's
draws and G-buffer aim at one of the four shown pixels a drawn pixel
covers, and the history is read through the phase the state before was
drawn at).  The oracle (oracle/port/temporal.c) is fed the same inputs and
the same state before.
"""
import os

import numpy as np
import pytest

from helpers import GOLDEN

FIELDS = ("colour", "moment", "length", "distance", "normal", "leaf", "albedo")


def golden(name="temporal"):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    return {k: z[k] for k in z.files}


def surfaces(g, f, part):
    return {key: g[f"{f}.{part}.{key}"] for key in ("distance", "normal", "leaf", "albedo")}


def state_of(g, f):
    import oracle.port as op
    n = int(g["width"]) * int(g["height"])
    s = np.zeros(n, op.TPIXEL_DTYPE)
    for key in FIELDS:
        s[key] = g[f"{f}.state.{key}"]
    return s


@pytest.mark.parametrize("name", ["temporal", "temporal_factor2"])
@pytest.mark.parametrize("frame", range(5))
def test_temporal_oracle_matches_reference(name, frame):
    import oracle.port as op
    g = golden(name)
    w, h = int(g["width"]), int(g["height"])
    factor = int(g["factor"])
    film = (factor, int(g[f"{frame}.phase"]), factor, int(g[f"{frame}.before_phase"]))
    before = state_of(g, frame - 1) if frame > 0 else None
    after, image = op.temporal(w, h, bool(g[f"{frame}.moved"]), False, bool(g[f"{frame}.kept"]), g[f"{frame}.lens"], g[f"{frame}.before"],
                               g[f"{frame}.light"], surfaces(g, frame, "first"), surfaces(g, frame, "gbuffer"), before, film)
    want = state_of(g, frame)
    for key in ("colour", "moment", "albedo", "normal"):
        assert np.allclose(after[key], want[key], rtol=1e-12, atol=1e-12), key
    for key in ("length", "distance", "leaf"):
        assert np.array_equal(after[key], want[key]), key
    assert np.array_equal(image, g[f"{frame}.image"])
