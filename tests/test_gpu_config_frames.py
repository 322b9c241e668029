"""Frame parity on the benchmark configurations, through the C ABI.

* Config 1 at its stated size (64 primitives, 256 x 256, 16 spp, 8
  surfaces): the GPU's frames against the oracle's (oracle/port, double
  precision) on the same 12 seeds, and against the reference renderer's
  own frames (tests/golden/image_c1.npz, written by the reference built from
  its sources: 8 seeds of 16 spp on its sphere-traced geometry over the
  world's region, the geometry the oracle and the device restate).
* Config 2 (4096 primitives, 1920 x 1080, 64 spp, 16 surfaces) on the
  octree the benchmark builds (7, 11, 32): a band of rows through the middle
  of the frame against the oracle's render_band on the same seeds.
* Convergence: relative MSE (mean((img - ref)^2 / (ref^2 + 0.01)), the
  reference's target/tools/realtime.py relative_mse) against a 65536-spp
  frame falls as spp^-1 for the GPU and the oracle alike, at the same rate
  and level.

Bars: the per-pixel difference of the seeds' means within 3 combined
standard errors for all but 1.5% of pixel channels (the t-distribution of
a 12 + 12 seed comparison puts ~0.7% past 3 by chance; path-traced noise has
heavier tails) and every channel's image mean within 3 standard errors;
against the reference's own frames (fewer seeds, written once) the image
mean is held to 0.5% and at most 2% of pixel channels past 3."""
import os

import numpy as np
import pytest

from helpers import GOLDEN, scene

pytestmark = pytest.mark.gpu

SEEDS = list(range(1, 13))
THREADS = os.cpu_count() or 4


def rel_mse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 0.01)))


def zscores(a, b):
    """Per pixel channel and per channel image-mean z of two stacks of
    independent frames (seeds first)."""
    ka, kb = len(a), len(b)
    z = (a.mean(0) - b.mean(0)) / np.sqrt(a.var(0, ddof=1) / ka + b.var(0, ddof=1) / kb + 1e-12)
    ca, cb = a.mean(axis=(1, 2)), b.mean(axis=(1, 2))
    cz = (ca.mean(0) - cb.mean(0)) / np.sqrt(ca.var(0, ddof=1) / ka + cb.var(0, ddof=1) / kb)
    return z, cz, ca.mean(0), cb.mean(0)


@pytest.fixture(scope="module")
def backend():
    import kodanuki_gb300 as K
    b = K.Backend(0)
    yield b
    b.close()


def test_config1_frame_matches_oracle_and_reference(backend):
    import oracle.port as op
    sc = scene("c1")
    w, h, spp, surfaces = int(sc.render["width"]), int(sc.render["height"]), int(sc.render["samples"]), int(sc.render["surfaces"])
    assert (w, h, spp, surfaces) == (256, 256, 16, 8)
    build = dict(min_depth=6, max_depth=11, split_steps=64)
    backend.load(sc)
    backend.build(**build)
    gpu = np.stack([backend.render(w, h, spp, surfaces=surfaces, seed=s) for s in SEEDS]).astype(np.float64)
    oracle = np.stack([op.render_band(sc, w, h, spp, surfaces, s, 0, h, THREADS, build) / spp for s in SEEDS])
    z, cz, g_mean, o_mean = zscores(gpu, oracle)
    far = float((np.abs(z) > 3).mean())
    ref = np.load(os.path.join(GOLDEN, "image_c1.npz"))
    rk = int(ref["seeds"])
    rz = (gpu.mean(0) - ref["mean"]) / np.sqrt(gpu.var(0, ddof=1) / len(gpu) + ref["var"] / rk + 1e-12)
    r_mean = ref["mean"].mean(axis=(0, 1))
    far_r = float((np.abs(rz) > 3).mean())
    print(f"config 1: gpu {g_mean} oracle {o_mean} reference {r_mean}; vs oracle z {cz} px {far:.4f}; vs reference rel {g_mean / r_mean - 1} px {far_r:.4f}")
    assert far <= 0.015, far
    assert np.all(np.abs(cz) < 3), cz
    assert np.all(np.abs(g_mean / r_mean - 1) < 0.005), (g_mean, r_mean)
    assert far_r <= 0.02, far_r


def test_config2_band_matches_oracle(backend):
    """Rows 536..543 of the 1920 x 1080 frame at 64 spp and 16 surfaces: the
    benchmark's frame, checked where it crosses the scene's middle."""
    import oracle.port as op
    sc = scene("c2")
    w, h, spp, surfaces = int(sc.render["width"]), int(sc.render["height"]), int(sc.render["samples"]), int(sc.render["surfaces"])
    assert (w, h, spp, surfaces) == (1920, 1080, 64, 16)
    build = dict(min_depth=7, max_depth=11, split_steps=32)
    row0, rows = 536, 8
    seeds = SEEDS[:8]
    backend.load(sc)
    backend.build(**build)
    gpu = np.stack([backend.render(w, h, spp, surfaces=surfaces, seed=s)[row0:row0 + rows] for s in seeds]).astype(np.float64)
    oracle = np.stack([op.render_band(sc, w, h, spp, surfaces, s, row0, rows, THREADS, build) / spp for s in seeds])
    z, cz, g_mean, o_mean = zscores(gpu, oracle)
    far = float((np.abs(z) > 3).mean())
    print(f"config 2 band: gpu {g_mean} oracle {o_mean}; z {cz} px {far:.4f}")
    assert far <= 0.02, far
    assert np.all(np.abs(cz) < 3), cz


def test_relmse_converges_at_the_oracle_rate(backend):
    """relMSE against a 65536-spp GPU frame at 4, 16 and 64 spp (4 seeds
    each): the GPU's and the oracle's fall as spp^-1, with slopes within
    0.05 of each other and levels within 10% (they draw the same numbers, so
    they follow the same paths where FP32 and double agree)."""
    import oracle.port as op
    sc = scene("c1_small")
    w, h, surfaces = int(sc.render["width"]), int(sc.render["height"]), int(sc.render["surfaces"])
    build = dict(min_depth=5, max_depth=10, split_steps=64)
    backend.load(sc)
    backend.build(**build)
    ref = np.zeros((h, w, 3), np.float64)
    for k in range(16):
        ref += backend.render(w, h, 4096, surfaces=surfaces, seed=50_000 + k)
    ref /= 16
    counts = [4, 16, 64]
    g, o = [], []
    for spp in counts:
        g.append(np.mean([rel_mse(backend.render(w, h, spp, surfaces=surfaces, seed=s), ref) for s in range(1, 5)]))
        o.append(np.mean([rel_mse(op.render_band(sc, w, h, spp, surfaces, s, 0, h, THREADS, build) / spp, ref) for s in range(1, 5)]))
    sg = np.polyfit(np.log(counts), np.log(g), 1)[0]
    so = np.polyfit(np.log(counts), np.log(o), 1)[0]
    print(f"relMSE gpu {np.round(g, 5)} slope {sg:.3f}; oracle {np.round(o, 5)} slope {so:.3f}")
    assert abs(sg + 1) < 0.15 and abs(so + 1) < 0.15, (sg, so)
    assert abs(sg - so) < 0.05, (sg, so)
    assert np.all(np.abs(np.array(g) / np.array(o) - 1) < 0.1), (g, o)
