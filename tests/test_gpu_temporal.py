"""The device's temporal member (kdn_temporal_device) against the
reference's temporalFrame, frame by frame over the golden still / moving /
still sequences (tests/golden/temporal.npz at a film factor of 1,
temporal_factor2.npz at 2, each frame at its Bayer phase), each frame fed
the state the reference left after the frame before.

The device computes the geometry (headings, planes, where a point was seen
before, the bilinear weights) in double as the reference does, and the
light in FP32; the bar: the state's colour, moment and the shown light
within 1e-5 relative for at least 99.5% of pixels and within 1e-4 for all,
1e-6 at the median; the length equal within 1e-6 on every pixel.
"""
import ctypes
import os

import numpy as np
import pytest

from helpers import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    import kodanuki_gb300 as K
    b = K.Backend(0)
    yield b
    b.close()


def fp16_bits(a):
    return np.ascontiguousarray(np.asarray(a, np.float32).astype(np.float16)).view(np.int16)


@pytest.mark.parametrize("name", ["temporal", "temporal_factor2"])
@pytest.mark.parametrize("frame", range(5))
def test_temporal_matches_reference(backend, name, frame):
    import torch
    import kodanuki_gb300 as K
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    g = {k: z[k] for k in z.files}
    w, h = int(g["width"]), int(g["height"])
    n = w * h
    dev = torch.device("cuda:0")

    def put(a, dtype):
        return torch.from_numpy(np.ascontiguousarray(a, dtype)).to(dev)

    def half(a):
        return torch.from_numpy(fp16_bits(a)).to(dev)

    keep = []
    bufs = K.TemporalBuffers()

    def bind(name, t):
        keep.append(t)
        setattr(bufs, name, t.data_ptr())

    bind("light", put(g[f"{frame}.light"], np.float32))
    for part, prefix in (("first", "first"), ("gbuffer", "centre")):
        bind(f"{prefix}_distance", half(g[f"{frame}.{part}.distance"]))
        bind(f"{prefix}_normal", half(g[f"{frame}.{part}.normal"]))
        bind(f"{prefix}_albedo", half(g[f"{frame}.{part}.albedo"]))
        bind(f"{prefix}_leaf", put(g[f"{frame}.{part}.leaf"], np.uint32).view(torch.int32))
    if frame > 0:
        bind("before_colour", put(g[f"{frame - 1}.state.colour"], np.float32))
        bind("before_moment", put(g[f"{frame - 1}.state.moment"], np.float32))
        bind("before_length", put(g[f"{frame - 1}.state.length"], np.float32))
        bind("before_distance", half(g[f"{frame - 1}.gbuffer.distance"]))
        bind("before_normal", half(g[f"{frame - 1}.gbuffer.normal"]))
        bind("before_leaf", put(g[f"{frame - 1}.gbuffer.leaf"], np.uint32).view(torch.int32))
    colour = torch.zeros(n * 3, dtype=torch.float32, device=dev)
    moment = torch.zeros(n, dtype=torch.float32, device=dev)
    length = torch.zeros(n, dtype=torch.float32, device=dev)
    image = torch.zeros(n * 3, dtype=torch.float32, device=dev)
    for name, t in (("colour", colour), ("moment", moment), ("length", length), ("image", image)):
        bind(name, t)
    factor = int(g["factor"])
    fr = K.TemporalFrame(w, h, int(g[f"{frame}.moved"]), 0, int(g[f"{frame}.kept"]), factor, int(g[f"{frame}.phase"]), factor,
                         int(g[f"{frame}.before_phase"]))
    for k in range(14):
        fr.now[k] = float(g[f"{frame}.lens"][k])
        fr.before[k] = float(g[f"{frame}.before"][k])
    stream = torch.cuda.current_stream()
    backend._check(backend.lib.kdn_temporal_device(backend.handle, ctypes.byref(fr), ctypes.byref(bufs), ctypes.c_void_p(stream.cuda_stream)))
    torch.cuda.synchronize()

    def rel(got, want):
        got = got.cpu().numpy().astype(np.float64).reshape(want.shape)
        return np.abs(got - want) / (np.abs(want) + 1e-3)

    # a reprojected history's length is a bilinear blend: FP32 against double
    want_length = g[f"{frame}.state.length"].astype(np.float64)
    length_same = (np.abs(length.cpu().numpy().astype(np.float64) - want_length) <= 1e-6 * np.maximum(want_length, 1.0)).mean()
    errs = {"colour": rel(colour, g[f"{frame}.state.colour"]).max(axis=1), "moment": rel(moment, g[f"{frame}.state.moment"]),
            "image": rel(image, g[f"{frame}.image"].astype(np.float64)).max(axis=1)}
    print(f"frame {frame}: length equal {length_same:.4f}; " + "; ".join(f"{k} p50 {np.median(e):.1e} max {e.max():.1e} within 1e-5 {np.mean(e <= 1e-5):.4f}"
                                                                        for k, e in errs.items()))
    assert length_same == 1.0
    for e in errs.values():
        assert np.mean(e <= 1e-5) >= 0.995
        assert np.all(e <= 1e-4)
        assert np.median(e) <= 1e-6
