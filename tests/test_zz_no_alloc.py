"""kdn_denoise_static, the denoiser entry point that allocates nothing, for
callers that may not allocate device memory once running (a frame loop with
a device-memory budget fixed at start-up, or one that must not stall other
streams on cudaMalloc).  Its output must equal the context entry point's
(kdn_denoise_device) within the denoiser tests' tolerance (1e-3), on two
calls in a row through the C ABI, and it must refuse a frame past its
512x512 static scratch.  Collected last: tests/test_zz_*.
"""
import ctypes
import os

import numpy as np
import pytest

from helpers import GOLDEN

pytestmark = pytest.mark.gpu


def test_static_denoiser_matches_context_denoiser():
    torch = pytest.importorskip("torch")
    import kodanuki_gb300 as K

    z = np.load(os.path.join(GOLDEN, "denoise.npz"))
    d = {k: z[k] for k in z.files}
    w, h = int(d["width"]), int(d["height"])
    lens = d["lens"]
    frame = K.DenoiseFrame(w, h, 0, 0)
    for k in range(3):
        frame.eye[k], frame.forward[k], frame.right[k], frame.up[k] = lens[k], lens[3 + k], lens[6 + k], lens[9 + k]
    frame.reach, frame.aspect = float(lens[12]), float(lens[13])
    L = K.library()
    dev = torch.device("cuda:0")
    with K.Backend(0) as b:
        for call, name in enumerate(["mixed", "checker"]):  # two calls in a row
            f = {k.split(".", 1)[1]: v for k, v in d.items() if k.startswith(name + ".")}
            frame.demodulated = int(f["demodulated"])
            ins = [torch.from_numpy(np.ascontiguousarray(f["colour"], np.float32)).to(dev),
                   torch.from_numpy(np.ascontiguousarray(f["moment"], np.float32)).to(dev),
                   torch.from_numpy(np.ascontiguousarray(f["length"], np.float32)).to(dev),
                   torch.from_numpy(np.ascontiguousarray(f["distance"], np.float16).view(np.int16)).to(dev),
                   torch.from_numpy(np.ascontiguousarray(f["normal"], np.float16).view(np.int16)).to(dev),
                   torch.from_numpy(np.ascontiguousarray(f["albedo"], np.float16).view(np.int16)).to(dev),
                   torch.from_numpy(np.ascontiguousarray(f["leaf"], np.uint32).view(np.int32)).to(dev)]
            ptrs = [ctypes.c_void_p(t.data_ptr()) for t in ins]
            ref = torch.zeros(w * h * 3, dtype=torch.float32, device=dev)
            got = torch.full((w * h * 3,), -1.0, dtype=torch.float32, device=dev)
            torch.cuda.synchronize()
            assert L.kdn_denoise_device(b.handle, ctypes.byref(frame), *ptrs, ctypes.c_void_p(ref.data_ptr()), None) == K.KDN_OK
            torch.cuda.synchronize()  # the context's stream
            assert L.kdn_denoise_static(ctypes.byref(frame), *ptrs, ctypes.c_void_p(got.data_ptr()), None) == K.KDN_OK, L.kdn_last_error(None)
            torch.cuda.synchronize()
            diff = (got - ref).abs().max().item()
            print(f"call {call} ({name}): max |static - context| {diff:.3e}")
            assert diff <= 1e-3
            assert np.abs(got.cpu().numpy().reshape(-1, 3) - f["out"]).max() <= 1e-3
        big = K.DenoiseFrame(513, 512, 0, 0)
        big.reach, big.aspect = 0.5, 1.0
        assert L.kdn_denoise_static(ctypes.byref(big), *ptrs, ctypes.c_void_p(got.data_ptr()), None) == K.KDN_BAD_ARG
        assert b"512x512" in L.kdn_last_error(None)
