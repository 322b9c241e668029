"""Write tests/golden/bsdf_<scene>.npz: the reference's own respondBsdf and
sampleBsdf (plugins/transport/paths/material/material.cpp:1076, :1366) at
seeded vertices of every material of a scene, through oracle/_ref's
``kdn_ref_dump bsdf`` (the reference library built from its sources).

Each material gets 200 vertices: a unit normal, an outgoing direction on
its side (one in eight below it), an incoming direction anywhere, a
wavelength share, the four draw numbers, and for a glass the inside or the
outside of its body.  Albedos and normals are float-representable (the
reference's Bsdf holds them as floats).  The oracle (oracle/port
bsdf_answers) is held to these answers by tests/test_oracle.py.  Run here,
where the reference builds:

    python tests/golden/make_bsdf.py [--only films_small]
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_golden import SCENES  # noqa: E402

NAMES = ["films_small", "glass_small", "rough_small", "c2_small"]
PER_MATERIAL = 200
NO_MATERIAL = 0xFFFFFFFF


def unit(v: np.ndarray) -> np.ndarray:
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def vertices(scene, rng: np.random.Generator):
    kinds = np.asarray(scene.materials["kind"])
    albedo = np.asarray(scene.materials["albedo"], np.float64)
    ids, recs = [], []
    for m, kind in enumerate(kinds):
        n = PER_MATERIAL
        normal = unit(rng.normal(size=(n, 3))).astype(np.float32).astype(np.float64)
        out = unit(rng.normal(size=(n, 3)))
        flip = (out * normal).sum(1) < 0
        below = rng.random(n) < 0.125
        out[flip != below] *= -1
        incoming = unit(rng.normal(size=(n, 3)))
        inside = (rng.random(n) < 0.5) if kind == 3 else np.zeros(n, bool)
        medium = np.where(inside, m, NO_MATERIAL).astype(np.uint32)
        rgb = np.repeat(albedo[m:m + 1].astype(np.float32).astype(np.float64), n, 0)
        share = rng.random(n)
        numbers = rng.random((n, 4))
        ids.append(np.stack([np.full(n, m, np.uint32), medium], 1))
        recs.append(np.concatenate([rgb, normal, out, incoming, share[:, None], numbers], 1))
    return np.concatenate(ids), np.ascontiguousarray(np.concatenate(recs))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-bin", default=os.path.join(ROOT, "oracle", "_ref"))
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    from kodanuki_gb300.scene import Scene
    dump = os.path.join(args.ref_bin, "kdn_ref_dump")
    tmp = tempfile.mkdtemp()
    for k, name in enumerate(NAMES):
        if args.only and name != args.only:
            continue
        gen, kw, _, _ = SCENES[name]
        sdf = os.path.join(tmp, name + ".sdf")
        open(sdf, "w").write(gen(**kw))
        scene = Scene.load(os.path.join(HERE, "scenes", name + ".npz"))
        ids, recs = vertices(scene, np.random.default_rng(4200 + k))
        inp, outp = os.path.join(tmp, name + ".in"), os.path.join(tmp, name + ".out")
        with open(inp, "wb") as f:
            for i in range(len(ids)):
                f.write(ids[i].tobytes())
                f.write(recs[i].tobytes())
        subprocess.run([dump, "bsdf", sdf, inp, outp], check=True)
        raw = np.fromfile(outp, np.uint8).reshape(len(ids), 112)
        value = raw[:, 0:32].copy().view("<f8")
        density = raw[:, 32:40].copy().view("<f8")[:, 0]
        seen = raw[:, 40:48].copy().view("<u4")
        incoming = raw[:, 48:72].copy().view("<f8")
        weight = raw[:, 72:104].copy().view("<f8")
        drawn = raw[:, 104:112].copy().view("<f8")[:, 0]
        np.savez_compressed(os.path.join(HERE, f"bsdf_{name}.npz"), ids=ids, records=recs, value=value, density=density, seen=seen,
                            incoming=incoming, weight=weight, drawn_density=drawn)
        print(f"{name}: {len(ids)} vertices, found {int(seen[:, 0].sum())}, through {int(seen[:, 1].sum())}, "
              f"value > 0 {int((value.max(1) > 0).sum())}")


if __name__ == "__main__":
    main()
