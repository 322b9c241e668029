"""Seeded rays for the geometry parity fixtures (tests/golden/hits_*.npz):
half from the eye through random film points (core/camera.cpp:34
filmDirection), half from random points around the objects in random
directions.  Generated with numpy's PCG64 and plain float64 arithmetic
rounded once to float32, so every machine draws the same rays (the fixture
keeps their SHA-256 to check that)."""
from __future__ import annotations

import numpy as np

RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("direction", "<f4", 3), ("far", "<f4"), ("inside", "u1"), ("pad", "u1", 3), ("within", "<u4")])


def REACH(scene):
    """The box rays are clipped to: the region the reference's tree (and the
    device's octree) is built over (plugins/geometry/tree/build.cpp:405
    sceneRegion), handed to the reference's sphere tracer as its region, as
    the reference's golden frames are drawn (--region); its own default,
    the cube of the render's reach about the target (sphere_trace.h
    reachRegion), would let a ground plane reach past the world."""
    return np.asarray(scene.region_lower, np.float64), np.asarray(scene.region_size, np.float64)


def hit_rays(scene, n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    cam = scene.camera
    eye = np.asarray(cam["eye"], np.float64)
    target = np.asarray(cam["target"], np.float64)
    up = np.asarray(cam["up"], np.float64)
    fwd = (target - eye) / np.sqrt(np.sum((target - eye) ** 2))
    right = np.cross(fwd, up)
    right = right / np.sqrt(np.sum(right ** 2))
    upv = np.cross(right, fwd)
    reach = np.tan(float(cam["fov"]) / 2)
    w, h = int(scene.render["width"]), int(scene.render["height"])
    m = n // 2
    x = rng.uniform(0, w, m)
    y = rng.uniform(0, h, m)
    u = 2 * x / w - 1
    v = 1 - 2 * y / h
    d = fwd[None] + right[None] * (u * reach * w / h)[:, None] + upv[None] * (v * reach)[:, None]
    o2 = rng.uniform(-3, 3, (n - m, 3))
    d2 = rng.normal(size=(n - m, 3))
    dirs = np.concatenate([d, d2])
    dirs = dirs / np.sqrt(dirs[:, 0] ** 2 + dirs[:, 1] ** 2 + dirs[:, 2] ** 2)[:, None]
    rays = np.zeros(n, RAY_DTYPE)
    rays["origin"] = np.concatenate([np.broadcast_to(eye, (m, 3)), o2]).astype(np.float32)
    rays["direction"] = dirs.astype(np.float32)
    rays["far"] = np.inf
    rays["within"] = 0xFFFFFFFF
    return rays
