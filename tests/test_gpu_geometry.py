"""GPU geometry parity: hits of kdn_extend (through the C ABI) against the
reference's own sphereTraced hits on the same seeded rays
(tests/golden/trace_*.npz), and the device world against the host build.

Tolerances: the reference marches in double to 1e-6; the device marches in
FP32 to 1e-5 (relative to the point's magnitude past 16).  Hit leaves
(primitive ids, hence materials) must agree on every ray both call a hit
except where the hit point sits within the tie band of a seam; distances
agree to 1e-5 relative for 95% of hits and 1e-4 for 99% (a grazing ray
stops up to tolerance / cos(angle) short of the surface in either
precision); normals to within 1e-3 in 99% of hits."""
import numpy as np
import pytest

from helpers import golden_rays, scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    import kodanuki_gb300 as K
    b = K.Backend(0)
    yield b
    b.close()


@pytest.mark.parametrize("name,build", [("c1", (6, 11, 64)), ("c2", (7, 10, 96))])
def test_hits_match_reference(backend, name, build):
    sc = scene(name)
    backend.load(sc)
    backend.build(*build)
    rays, tr = golden_rays(name)
    h = backend.extend(rays)
    ref_hit = tr["kind"] == 1
    got_hit = h["kind"] == 1
    agree = (ref_hit == got_hit).mean()
    both = ref_hit & got_hit
    leaf_agree = (h["leaf"][both] == tr["leaf"][both]).mean()
    rel = np.abs(h["distance"][both] - tr["distance"][both]) / np.maximum(tr["distance"][both], 1e-6)
    cosang = np.clip((h["normal"][both] * tr["normal"][both]).sum(1), -1, 1)
    print(f"{name}: kind agree {agree:.4f} leaf agree {leaf_agree:.4f} rel p50 {np.median(rel):.2e} p99 {np.quantile(rel, 0.99):.2e} max {rel.max():.2e} normal p99 {np.quantile(1 - cosang, 0.99):.2e}")
    assert agree >= 0.99
    assert leaf_agree >= 0.99
    assert np.quantile(rel, 0.95) <= 1e-5
    assert np.quantile(rel, 0.99) <= 1e-4
    assert np.quantile(1 - cosang, 0.99) <= 1e-3


def test_extend_empty_and_missing(backend):
    import kodanuki_gb300 as K
    sc = scene("c1")
    backend.load(sc)
    backend.build(6, 11, 64)
    assert len(backend.extend(np.zeros(0, K.RAY_DTYPE))) == 0
    # rays pointing away from everything miss
    r = np.zeros(64, K.RAY_DTYPE)
    r["origin"] = [0.0, 0.0, 50.0]
    r["direction"] = [0.0, 0.0, 1.0]
    r["far"] = np.inf
    r["within"] = 0xFFFFFFFF
    h = backend.extend(r)
    assert (h["kind"] == 0).all()
