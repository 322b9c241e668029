"""GPU denoiser parity against the reference's own denoisedFrame on
identical feature buffers (tests/golden/denoise.npz, FP16-rounded distance,
normal and albedo, as the GPU stores them).  Bar: every output value within
1e-3 of the reference's (the device keeps the reference's float order and
computes the guides in double, so most values match to the bit)."""
import os

import numpy as np
import pytest

from helpers import GOLDEN

pytestmark = pytest.mark.gpu


def test_denoiser_matches_reference():
    import kodanuki_gb300 as K
    z = np.load(os.path.join(GOLDEN, "denoise.npz"))
    d = {k: z[k] for k in z.files}
    names = sorted({k.split(".", 1)[0] for k in d if "." in k})
    with K.Backend(0) as b:
        for name in names:
            f = {k.split(".", 1)[1]: v for k, v in d.items() if k.startswith(name + ".")}
            out = b.denoise(int(d["width"]), int(d["height"]), bool(f["demodulated"]), d["lens"], f["colour"], f["moment"], f["length"],
                            f["distance"], f["normal"], f["albedo"], f["leaf"])
            diff = np.abs(out - f["out"])
            print(f"{name}: max |gpu - reference| {diff.max():.3e}, exact {np.mean(out == f['out']):.4f}")
            assert diff.max() <= 1e-3, name
