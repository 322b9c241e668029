"""The device's upscale member (kdn_upscale_device) against the reference's
upscaledFrame, frame by frame over tests/golden/upscale.npz (factor-2
frames still, moving, settling and restarted, then factor-4 frames without
a G-buffer), each frame fed the state the reference left after the frame
before.  The device keeps the reference's number types and order of
operations (tones in float, positions and history colours in double, no
FMA contraction, the axes' weights from the host's exp), so the bar is the
bit: the shown frame and the state's colour and depth equal the
reference's.
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


@pytest.mark.parametrize("frame", range(11))
def test_upscale_matches_reference(backend, frame):
    import torch
    import kodanuki_gb300 as K
    import oracle.port as op
    z = np.load(os.path.join(GOLDEN, "upscale.npz"))
    g = {k: z[k] for k in z.files}
    factor = int(g[f"{frame}.factor"])
    internal = g[f"{frame}.internal"]
    n = len(g[f"{frame}.image"])
    dw = int(round(np.sqrt(len(internal) * 1.5)))  # the drawn grids are 3:2
    dh = len(internal) // dw
    w, h = dw * factor, dh * factor
    assert w * h == n
    dev = torch.device("cuda:0")
    kept = bool(g[f"{frame}.kept"])
    settling, _ = op.upscale_settling(kept, bool(g[f"{frame}.moved"]), bool(g[f"{frame}.before_moved"]), int(g[f"{frame}.before_settling"]))
    keep = []
    bufs = K.UpscaleBuffers()

    def bind(name, t):
        keep.append(t)
        setattr(bufs, name, t.data_ptr())

    bind("internal", torch.from_numpy(np.ascontiguousarray(internal, np.float32)).to(dev))
    if f"{frame}.distance" in g:
        bits = np.ascontiguousarray(g[f"{frame}.distance"].astype(np.float16)).view(np.int16)
        bind("distance", torch.from_numpy(bits).to(dev))
    if kept:
        before = np.zeros((n, 4), np.float32)
        before[:, :3] = g[f"{frame - 1}.colour"].astype(np.float32)
        before[:, 3] = g[f"{frame - 1}.depth"]
        assert np.array_equal(before[:, :3].astype(np.float64), g[f"{frame - 1}.colour"])  # the state's colours are float values
        bind("before", torch.from_numpy(before).to(dev))
    after = torch.zeros(n * 4, dtype=torch.float32, device=dev)
    image = torch.zeros(n * 3, dtype=torch.float32, device=dev)
    bind("after", after)
    bind("image", image)
    fr = K.UpscaleFrame(w, h, factor, int(g[f"{frame}.phase"]), int(kept), int(settling))
    for k in range(14):
        fr.now[k] = float(g[f"{frame}.lens"][k])
        fr.before[k] = float(g[f"{frame}.before"][k])
    stream = torch.cuda.current_stream()
    backend._check(backend.lib.kdn_upscale_device(backend.handle, ctypes.byref(fr), ctypes.byref(bufs), ctypes.c_void_p(stream.cuda_stream)))
    torch.cuda.synchronize()
    got_image = image.cpu().numpy().reshape(n, 3)
    got_state = after.cpu().numpy().reshape(n, 4)
    same = (got_image == g[f"{frame}.image"]).all(1)
    print(f"frame {frame} factor {factor} kept {kept} settling {settling}: image equal on {same.mean():.6f}, "
          f"max |diff| {np.abs(got_image - g[f'{frame}.image']).max():.3e}")
    assert np.array_equal(got_image, g[f"{frame}.image"])
    assert np.array_equal(got_state[:, :3].astype(np.float64), g[f"{frame}.colour"])
    assert np.array_equal(got_state[:, 3], g[f"{frame}.depth"])


def test_upscale_refuses_bad_frames(backend):
    import kodanuki_gb300 as K
    bufs = K.UpscaleBuffers()
    for factor, phase, w, h in ((1, 0, 64, 64), (5, 0, 60, 60), (2, 4, 64, 64), (2, 0, 63, 64), (3, 0, 0, 0)):
        fr = K.UpscaleFrame(w, h, factor, phase, 0, 0)
        status = backend.lib.kdn_upscale_device(backend.handle, ctypes.byref(fr), ctypes.byref(bufs), None)
        assert status == K.KDN_BAD_ARG, (factor, phase, w, h)


@pytest.mark.parametrize("factor", [2, 3, 4])
def test_upsample_matches_reference(backend, factor):
    """kdn_upsample_device against the reference's upsampledImage
    (tests/golden/upsample.npz), to the bit."""
    import torch
    z = np.load(os.path.join(GOLDEN, "upsample.npz"))
    w, h = (int(v) for v in z[f"{factor}.size"])
    drawn = torch.from_numpy(np.ascontiguousarray(z[f"{factor}.drawn"], np.float32)).cuda()
    shown = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    backend._check(backend.lib.kdn_upsample_device(backend.handle, w, h, factor, drawn.data_ptr(), shown.data_ptr(), ctypes.c_void_p(stream.cuda_stream)))
    torch.cuda.synchronize()
    assert np.array_equal(shown.cpu().numpy().reshape(-1, 3), z[f"{factor}.shown"])
