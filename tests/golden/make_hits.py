"""Write tests/golden/hits_<name>.npz: 10^5 seeded rays of configs 1 and 2
traced by the oracle's restatement of the reference's sphereTraced
(plugins/geometry/sphere_trace/sphere_trace.cpp:216; oracle/port/geometry.c,
pinned bit for bit to the reference's own hits in tests/golden/trace_*.npz),
once under the reference's stopping tolerance (1e-6) and once under the FP32
device march's (2e-6 max(1, |p|_inf / 4)).  The first is the answer the
device is held to; the difference between the two is the reference's own
sensitivity to its stopping tolerance.  For each hit the fixture also keeps
how far its distance and normal can move over the stretch of the ray either
march may stop in (from the device's tolerance before the reference's stop
to the reference's after it, over |gradient| cos(angle)), the normal read
off the reference's own sphereNormal at both ends (oracle kp_normal_at).
From these the GPU test marks the rays whose answer the reference itself
does not fix to the bar (the tie band).

The rays are not stored: tests/golden/hit_rays.py regenerates them from the
seed, and the fixture keeps their SHA-256 so a test can tell that it holds
the same rays.  Run here, where the oracle builds:

    python tests/golden/make_hits.py [--rays 100000] [--workers 8]
"""
from __future__ import annotations

import argparse
import hashlib
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from hit_rays import REACH, hit_rays  # noqa: E402

CONFIGS = {"c1": 11, "c2": 12}  # scene -> ray seed


def _trace(job):
    name, lo, hi, n, seed = job
    import oracle.port as op
    from kodanuki_gb300.scene import Scene
    sc = Scene.load(os.path.join(HERE, "scenes", name + ".npz"))
    rays = hit_rays(sc, n, seed)[lo:hi]
    r = np.zeros(len(rays), op.RAY_DTYPE)
    for k in ("origin", "direction", "far", "within"):
        r[k] = rays[k]
    r["inside"] = rays["inside"]
    lower, size = REACH(sc)
    h0 = op.sphere_trace(sc, r, lower, size, 0)
    h1 = op.sphere_trace(sc, r, lower, size, 1)
    # the stretch of the ray either march may stop in: the reference stops
    # up to 1e-6 / (|grad| cos) before the surface, the device up to its own
    # tolerance / (|grad| cos); the hit's distance and normal anywhere on it
    hit = np.nonzero((h0["kind"] != 0) & (h0["distance"] > 0))[0]
    t = h0["distance"][hit].astype(np.float64)
    n_at, grad = op.normal_at(sc, r[hit], h0["object"][hit], t)
    p = r["origin"][hit].astype(np.float64) + r["direction"][hit].astype(np.float64) * t[:, None]
    tol_dev = 2e-6 * np.maximum(1.0, np.abs(p).max(1) / 4)
    cos = np.maximum(np.abs((r["direction"][hit].astype(np.float64) * n_at).sum(1)), 1e-3)
    g = np.maximum(grad, 1e-3)
    before, after = tol_dev / (g * cos), 1e-6 / (g * cos)
    n_before, _ = op.normal_at(sc, r[hit], h0["object"][hit], t - before)
    n_after, _ = op.normal_at(sc, r[hit], h0["object"][hit], t + after)
    dspread = np.zeros(len(r), np.float32)
    nspread = np.zeros(len(r), np.float32)
    dspread[hit] = (before + after) / t
    nspread[hit] = np.maximum(np.linalg.norm(n_before - n_at, axis=1), np.linalg.norm(n_after - n_at, axis=1))
    return lo, h0, h1, dspread, nspread


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--rays", type=int, default=100_000)
    ap.add_argument("--workers", type=int, default=os.cpu_count() or 8)
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    import oracle.port as op
    from kodanuki_gb300.scene import Scene
    op.build()
    ctx = mp.get_context("spawn")
    for name, seed in CONFIGS.items():
        if args.only and name != args.only:
            continue
        t0 = time.time()
        sc = Scene.load(os.path.join(HERE, "scenes", name + ".npz"))
        rays = hit_rays(sc, args.rays, seed)
        chunk = 500
        jobs = [(name, lo, min(lo + chunk, args.rays), args.rays, seed) for lo in range(0, args.rays, chunk)]
        h0 = np.zeros(args.rays, op.HIT_DTYPE)
        h1 = np.zeros(args.rays, op.HIT_DTYPE)
        dspread = np.zeros(args.rays, np.float32)
        nspread = np.zeros(args.rays, np.float32)
        with ctx.Pool(args.workers) as pool:
            for lo, a, b, ds, ns in pool.imap_unordered(_trace, jobs):
                h0[lo:lo + len(a)] = a
                h1[lo:lo + len(b)] = b
                dspread[lo:lo + len(a)] = ds
                nspread[lo:lo + len(a)] = ns
        both = (h0["kind"] != 0) & (h1["kind"] != 0)
        moved = np.zeros(args.rays, np.float32)
        moved[both] = np.abs(h0["distance"][both].astype(np.float64) - h1["distance"][both]) / np.maximum(h0["distance"][both].astype(np.float64), 1e-6)
        turned = np.zeros(args.rays, np.float32)
        turned[both] = np.linalg.norm(h0["normal"][both].astype(np.float64) - h1["normal"][both], axis=1)
        lower, size = REACH(sc)
        np.savez_compressed(os.path.join(HERE, f"hits_{name}.npz"), seed=seed, n=args.rays,
                            rays_sha256=hashlib.sha256(rays.tobytes()).hexdigest(), reach_lower=lower, reach_size=size,
                            kind=h0["kind"].astype(np.uint8), leaf=h0["leaf"], distance=h0["distance"], normal=h0["normal"],
                            kind_fp32_rule=h1["kind"].astype(np.uint8), leaf_fp32_rule=h1["leaf"], distance_moved=moved, normal_moved=turned,
                            distance_spread=dspread, normal_spread=nspread)
        print(f"{name}: {args.rays} rays, {int((h0['kind'] != 0).sum())} hits, {time.time() - t0:.0f} s; "
              f"kind moved {int((h0['kind'] != h1['kind']).sum())}, leaf moved {int((h0['leaf'] != h1['leaf'])[both].sum())}, "
              f"distance moved > 5e-6 {int((moved > 5e-6).sum())}, normal moved > 5e-6 {int((turned > 5e-6).sum())}; "
              f"distance spread > 5e-6 {int((dspread > 5e-6).sum())}, normal spread > 5e-6 {int((nspread > 5e-6).sum())}", flush=True)


if __name__ == "__main__":
    main()
