"""The oracle's upscale member against the reference's upscaledFrame.

tests/golden/upscale.npz holds a sequence of frames run through the
reference's own upscaledFrame (plugins/reconstruction/upscale/upscale.cpp)
with the state the frame before left: the drawn frames of the temporal
fixture at a film factor of 2 (still, moving, still), three still frames
that settle after the movement, a restart, and two frames at a film factor
of 4 with no G-buffer.  The oracle (oracle/port/upscale.c) is fed the same
inputs and the same state before, and must answer to the bit; the settling
count it keeps (upscale.cpp:557 settlingFrames) must follow the
reference's.
"""
import os

import numpy as np
import pytest

from helpers import GOLDEN


def golden():
    z = np.load(os.path.join(GOLDEN, "upscale.npz"))
    return {k: z[k] for k in z.files}


@pytest.mark.parametrize("frame", range(11))
def test_upscale_oracle_matches_reference(frame):
    import oracle.port as op
    g = golden()
    assert int(g["frames"]) == 11
    factor = int(g[f"{frame}.factor"])
    internal = g[f"{frame}.internal"]
    shown = len(g[f"{frame}.image"])
    drawn = len(internal)
    dw = int(round(np.sqrt(drawn * 1.5)))  # the drawn grids are 3:2
    dh = drawn // dw
    assert dw * dh == drawn and dw * dh * factor * factor == shown
    w, h = dw * factor, dh * factor
    kept = bool(g[f"{frame}.kept"])
    settling, count = op.upscale_settling(kept, bool(g[f"{frame}.moved"]), bool(g[f"{frame}.before_moved"]), int(g[f"{frame}.before_settling"]))
    assert count == int(g[f"{frame}.settling_after"])
    before = (g[f"{frame - 1}.colour"], g[f"{frame - 1}.depth"]) if kept else (None, None)
    distance = g.get(f"{frame}.distance")
    colour, depth, image = op.upscale(w, h, factor, int(g[f"{frame}.phase"]), bool(g[f"{frame}.moved"]), kept, settling, g[f"{frame}.lens"],
                                      g[f"{frame}.before"], internal, distance, *before)
    assert np.array_equal(depth, g[f"{frame}.depth"])
    assert np.array_equal(colour, g[f"{frame}.colour"])
    assert np.array_equal(image, g[f"{frame}.image"])


@pytest.mark.parametrize("factor", [2, 3, 4])
def test_upsample_oracle_matches_reference(factor):
    """The oracle's upsample member (oracle/port/upscale.c kp_upsample)
    against the reference's upsampledImage (tests/golden/upsample.npz), to
    the bit."""
    import oracle.port as op
    z = np.load(os.path.join(GOLDEN, "upsample.npz"))
    w, h = (int(v) for v in z[f"{factor}.size"])
    shown = op.upsample(w, h, factor, z[f"{factor}.drawn"])
    assert np.array_equal(shown, z[f"{factor}.shown"])
