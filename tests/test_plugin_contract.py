"""The reference-side binding (kodanuki_gb300/reference_plugin/backend_gb300.cpp)
compiled against the reference renderer built from its own sources
(oracle/ref), linked with libkdn_gb300, and driven through the reference's
frame loop (tests/plugin_contract.cpp).  On a machine without a GPU the
binding opens a host-only context (KDN_GB300_HOST_ONLY=1): it maps the
scene into this library's blocks and builds the world, then, owning no
kernel there, hands every step to the fallback.  That is the reference's own
Backend contract (target/tests/generic.cpp:268-285 checkBackendPoint): the
frame keeps backend/cpu's mean within 4.5 standard errors, the backend is
asked for every step of its workers, and it finds the transport's finishes,
lamps and sky as blocks of the frame (three with the reference set) and the
tree's arrays too with geometry/tree (five more).

Runs only where the reference checkout and its build are present (the
machine that writes the golden fixtures)."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("KDN_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
LIBREF = os.path.join(ROOT, "oracle", "_ref", "libkodanuki_ref.a")
KDN = os.path.join(ROOT, "kodanuki_gb300", "_build")

pytestmark = pytest.mark.skipif(not (os.path.isdir(os.path.join(REF, "source")) and os.path.exists(LIBREF)),
                                reason="needs the reference checkout and its build (oracle/ref)")

REFERENCE_USES = ["geometry=sphere_trace", "execution=single", "stopping=fixed_count", "detail=none", "build=none", "strategy=none",
                  "sampler=none", "observer=none"]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    import kodanuki_gb300 as K
    K.library()
    out = str(tmp_path_factory.mktemp("contract") / "plugin_contract")
    cmd = ["g++", "-std=c++23", "-O1", "-include", "algorithm", "-ffp-contract=off", "-w", "-I", os.path.join(REF, "source"), "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "plugin_contract.cpp"), os.path.join(ROOT, "kodanuki_gb300", "reference_plugin", "backend_gb300.cpp"),
           LIBREF, "-L", KDN, "-lkdn_gb300", f"-Wl,-rpath,{KDN}", "-lpthread", "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def read_pfm(path):
    data = open(path, "rb").read()
    head, dims, scale, rest = data.split(b"\n", 3)
    w, h = map(int, dims.split())
    return np.frombuffer(rest[: w * h * 12], "<f4" if float(scale) < 0 else ">f4").reshape(h, w, 3).astype(np.float64)


def frame(driver, sdf, backend, seed, tmp, uses=REFERENCE_USES):
    pfm = os.path.join(tmp, f"{backend}_{seed}_{len(uses)}.pfm")
    words = [driver, sdf, backend, "--seed", str(seed), "--threads", "4", "--samples", "4", "--out", pfm[:-4] + ".ppm", "--pfm", pfm]
    for u in uses:
        words += ["--use", u]
    env = dict(os.environ, KDN_GB300_HOST_ONLY="1")
    r = subprocess.run(words, check=True, capture_output=True, text=True, env=env)
    seen = dict(zip(r.stdout.split()[::2], map(int, r.stdout.split()[1::2])))
    return read_pfm(pfm), seen


def spread(a, b):
    """target/tests/generic.cpp:165 spreadOf: the mean of two frames and the
    variance of that mean, per channel."""
    px = a.shape[0] * a.shape[1]
    mean = ((a + b) / 2).reshape(-1, 3).sum(0) / px
    var = ((a - b) ** 2).reshape(-1, 3).sum(0) / (4 * px * px)
    return mean, var


def test_binding_keeps_the_backend_contract(driver, tmp_path):
    sys.path.insert(0, ROOT)
    from kodanuki_gb300 import scenegen
    sdf = str(tmp_path / "scene.sdf")
    open(sdf, "w").write(scenegen.scene_config1(seed=2, width=48, height=48, samples=4, count=12))
    cpu = [frame(driver, sdf, "cpu", s, str(tmp_path))[0] for s in (3, 4)]
    runs = [frame(driver, sdf, "gb300", s, str(tmp_path)) for s in (3, 4)]
    gb = [r[0] for r in runs]
    seen = runs[-1][1]
    m0, v0 = spread(*cpu)
    m1, v1 = spread(*gb)
    errors = np.max(np.abs(m1 - m0) / (np.sqrt(v0 + v1) + 1e-9))
    print(f"binding: means {m1} against backend/cpu {m0}, {errors:.2f} standard errors apart; seen {seen}")
    assert errors <= 4.5
    assert seen["device"] == 0 and seen["steps"] > 0
    assert seen["cells"] > 1, "the binding built the world from the scene's object programs"
    assert seen["blocks"] == 3, "the transport's finishes, lamps and sky as blocks of the frame"
    _, tree = frame(driver, sdf, "gb300", 3, str(tmp_path), uses=["geometry=tree"] + REFERENCE_USES[1:])
    assert tree["blocks"] >= 3 + 5, tree
