"""Regenerate the golden fixtures from the reference renderer itself.

Run only where the reference checkout and its oracle build exist:

    make -C oracle/ref REF=<the reference checkout> -j8
    python tests/golden/make_golden.py [--ref-bin oracle/_ref] [--only NAME]

It writes, under tests/golden/:
  scenes/<name>.npz      the compiled scene (kodanuki_gb300.scene.Scene)
  trace_<name>.npz       seeded rays and the reference's sphereTraced hits
  cut_<name>.npz         cutCell results down a fixed-depth octree
  cutdeep_c2.npz         cutCell of a sample of the benchmark octree's cells
  image_<name>.npz       reference frames (fixed spp, several seeds; config 1 at
                         its own size as per-pixel mean and variance)
Every input is seeded; rerunning gives the same files.
"""
from __future__ import annotations

import argparse
import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from kodanuki_gb300 import scenegen  # noqa: E402
from kodanuki_gb300.scene import STEP_DTYPE, Scene  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

REFERENCE_FLAGS = ["--threads", "8", "--use", "stopping=fixed_count", "--use", "execution=single", "--use", "detail=none",
                   "--use", "build=none", "--use", "strategy=none", "--use", "sampler=none", "--use", "observer=none"]

# The image fixtures are drawn on the reference's sphere-traced geometry
# (plugins/geometry/sphere_trace, sphereTraced), the geometry the oracle and
# the device restate, over the region the tree would be built over
# (--region, the scene's sceneRegion) rather than the sphere tracer's own
# reach around the target; the reference's default tree geometry
# (face-fitted leaves) lands hits a little differently and its frames
# differ from the sphere-traced ones by up to ~0.7% on scenes with close
# contacts.
IMAGE_FLAGS = REFERENCE_FLAGS + ["--use", "geometry=sphere_trace"]


def region_flags(scene: Scene) -> list[str]:
    lower = np.asarray(scene.region_lower, np.float64)
    upper = lower + np.asarray(scene.region_size, np.float64)
    return ["--region"] + [repr(float(x)) for x in lower] + [repr(float(x)) for x in upper]

# name -> (seeds, spp per seed) of the reference frames kept as image fixtures
IMAGES = {"room_small": (16, 64), "c1_small": (16, 64), "c2_small": (16, 64), "glow_small": (16, 64), "glass_small": (16, 64), "patterns_small": (16, 64), "rough_small": (16, 64),
          "films_small": (16, 64), "skylit_small": (16, 64), "lamps_small": (16, 64),
          "far_small": (16, 64), "scatter_small": (16, 64), "physical_small": (16, 64),
          "lens_small": (16, 64), "split_small": (48, 64),
          "stars_small": (16, 64)}

# the scenes whose reference frames are also drawn with --use sampler=sobol
SOBOL_IMAGES = ("c1_small", "glass_small")
# ... and with --use sampler=sky_map
SKY_MAP_IMAGES = ("skylit_small",)
# ... and with --use sampler=each_lamp_first
EACH_LAMP_IMAGES = ("lamps_small",)

# name -> (generator, kwargs, trace rays, cut depth)
SCENES = {
    "c1": (scenegen.scene_config1, dict(seed=1), 2000, 4),
    "c1_small": (scenegen.scene_config1, dict(seed=2, width=48, height=48, samples=64, count=12), 0, 0),
    "room": (scenegen.scene_room, dict(seed=1), 0, 0),
    "room_small": (scenegen.scene_room, dict(seed=3, width=48, height=48, samples=64, count=8), 0, 0),
    "c2": (scenegen.scene_config2, dict(seed=1), 200, 3),
    "c2_small": (scenegen.scene_config2, dict(seed=3, width=64, height=36, samples=64, groups=24), 0, 0),
    "glow_small": (scenegen.scene_glow, dict(seed=5, width=48, height=48, samples=64), 0, 0),
    "glass_small": (scenegen.scene_glass, dict(seed=6, width=48, height=48, samples=64), 0, 0),
    "patterns_small": (scenegen.scene_patterns, dict(seed=7, width=48, height=48, samples=64), 0, 0),
    "rough_small": (scenegen.scene_glass, dict(seed=8, width=48, height=48, samples=64, rough=True), 0, 0),
    "films_small": (scenegen.scene_films, dict(seed=9, width=48, height=48, samples=64), 0, 0),
    # config 5, the stress scene (the benchmark's --stress run)
    "c5": (scenegen.scene_config5, dict(seed=1), 0, 0),
    "skylit_small": (scenegen.scene_skylit, dict(seed=10, width=48, height=48, samples=64), 0, 0),
    "lamps_small": (scenegen.scene_lamps, dict(seed=11, width=48, height=48, samples=64), 0, 0),
    "far_small": (scenegen.scene_far_lights, dict(seed=12, width=48, height=48, samples=64), 0, 0),
    "scatter_small": (scenegen.scene_scattering, dict(seed=13, width=48, height=48, samples=64), 0, 0),
    "physical_small": (scenegen.scene_physical_sky, dict(seed=14, width=48, height=48, samples=64), 0, 0),
    "lens_small": (scenegen.scene_lens, dict(seed=15, width=48, height=48, samples=64), 0, 0),
    "split_small": (scenegen.scene_split, dict(seed=16, width=48, height=48, samples=64), 0, 0),
    "stars_small": (scenegen.scene_stars, dict(seed=17, width=48, height=48, samples=64), 0, 0),
}
# config 3: the eight resident scenes of the serving run, 256 to 16384
# config-1-style primitives (merge(0.05) groups of 64)
SERVE_COUNTS = [256, 512, 1024, 2048, 4096, 6144, 10240, 16384]
for _k, _n in enumerate(SERVE_COUNTS):
    SCENES[f"serve_{_n}"] = (scenegen.scene_serving, dict(seed=31 + _k, count=_n), 0, 0)


def camera_rays(scene: Scene, n: int, rng: np.random.Generator) -> np.ndarray:
    """Rays from the eye through random film points (core/camera.cpp:34)."""
    cam = scene.camera
    eye = np.array(cam["eye"])
    target = np.array(cam["target"])
    up = np.array(cam["up"])
    fwd = (target - eye) / np.linalg.norm(target - eye)
    right = np.cross(fwd, up)
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    reach = np.tan(cam["fov"] / 2)
    w, h = scene.render["width"], scene.render["height"]
    x = rng.uniform(0, w, n)
    y = rng.uniform(0, h, n)
    u = 2 * x / w - 1
    v = 1 - 2 * y / h
    d = fwd[None] + right[None] * (u * reach * w / h)[:, None] + upv[None] * (v * reach)[:, None]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = eye
    rays[:, 3:6] = d
    rays[:, 6] = np.inf
    return rays


def scattered_rays(scene: Scene, n: int, rng: np.random.Generator) -> np.ndarray:
    """Rays from random points near the objects in random directions."""
    o = rng.uniform(-3, 3, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3:6] = d
    rays[:, 6] = np.inf
    return rays


def step_digest(steps: np.ndarray) -> int:
    """64-bit FNV-1a over each step's opcode, a, b, c, value bits and leaf,
    little-endian: a golden digest of a cut program."""
    h = 0xCBF29CE484222325
    for s in steps:
        rec = struct.pack("<IIIIQI", int(s["opcode"]), int(s["a"]), int(s["b"]), int(s["c"]), int(np.float64(s["value"]).view(np.uint64)), int(s["leaf"]))
        for byte in rec:
            h = ((h ^ byte) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h


def read_cut(path: str):
    data = open(path, "rb").read()
    off = 0
    cells = []
    while off < len(data):
        level, px, py, pz, occ, n = struct.unpack_from("<6I", data, off)
        off += 24
        progs = []
        for _ in range(n):
            obj, result, count = struct.unpack_from("<3I", data, off)
            off += 12
            steps = np.zeros(count, STEP_DTYPE)
            for s in range(count):
                op, a, b, c = struct.unpack_from("<4I", data, off)
                value, = struct.unpack_from("<d", data, off + 16)
                leaf, = struct.unpack_from("<I", data, off + 24)
                off += 28
                steps[s] = (op, a, b, c, value, leaf)
            progs.append((obj, result, steps))
        cells.append((level, (px, py, pz), occ, progs))
    return cells


def read_pfm(path: str) -> np.ndarray:
    data = open(path, "rb").read()
    head, dims, scale, rest = data.split(b"\n", 3)
    w, h = map(int, dims.split())
    a = np.frombuffer(rest[: w * h * 12], "<f4" if float(scale) < 0 else ">f4").reshape(h, w, 3)
    return a[::-1].copy()


def reference_images(render: str, sdf: str, name: str, tmp: str, scene: Scene, sampler: str = "none") -> None:
    """Frames of the reference renderer at fixed spp under independent seeds:
    their per-pixel mean and the standard error of one seed's frame; with
    `sampler` "sobol", drawn with --use sampler=sobol (image_<name>_sobol.npz)."""
    seeds, spp = IMAGES[name]
    flags = [f if f != "sampler=none" else f"sampler={sampler}" for f in IMAGE_FLAGS]
    suffix = "" if sampler == "none" else f"_{sampler}"
    frames = []
    for k in range(seeds):
        pfm = os.path.join(tmp, f"{name}_{k}.pfm")
        subprocess.run([render, sdf, "--out", os.path.join(tmp, f"{name}_{k}.ppm"), "--pfm", pfm, "--seed", str(1000 + k),
                        "--samples", str(spp)] + flags + region_flags(scene), check=True, capture_output=True)
        frames.append(read_pfm(pfm))
    f = np.stack(frames)
    np.savez_compressed(os.path.join(HERE, f"image_{name}{suffix}.npz"), frames=f.astype(np.float32), spp=spp, seeds=np.arange(1000, 1000 + seeds))
    print(" image", suffix, f.shape, "mean", f.mean(axis=(0, 1, 2)))


# name -> (seeds, spp) of reference frames drawn at the scene's own size on
# the reference's sphere-traced geometry over the world's region (as
# IMAGE_FLAGS), kept as the per-pixel mean and variance over the seeds.
# (The reference's tree geometry capped at the config's "--depth 6" is a
# tree too shallow for its face fits: measured on config 1 it draws the
# frame 16% darker than its own sphere-traced frame; at its default depth
# it is within 0.7%.)
SIZED_IMAGES = {"c1": (8, 16)}


def reference_sized_images(render: str, sdf: str, name: str, tmp: str, scene: Scene) -> None:
    """Frames of the reference renderer at the scene's size and spp under
    independent seeds: the per-pixel mean and the variance of one seed's
    frame."""
    seeds, spp = SIZED_IMAGES[name]
    flags = [f if f != "8" else str(os.cpu_count() or 8) for f in IMAGE_FLAGS]
    frames = []
    for k in range(seeds):
        pfm = os.path.join(tmp, f"{name}_sized_{k}.pfm")
        subprocess.run([render, sdf, "--out", os.path.join(tmp, f"{name}_sized_{k}.ppm"), "--pfm", pfm, "--seed", str(2000 + k),
                        "--samples", str(spp)] + flags + region_flags(scene), check=True, capture_output=True)
        frames.append(read_pfm(pfm).astype(np.float64))
    f = np.stack(frames)
    np.savez_compressed(os.path.join(HERE, f"image_{name}.npz"), mean=f.mean(0).astype(np.float32), var=f.var(0, ddof=1).astype(np.float32),
                        seeds=seeds, spp=spp)
    print(" sized image", f.shape, "mean", f.mean(axis=(0, 1, 2)))


def denoise_fields(width: int = 64, height: int = 48):
    """Seeded feature buffers in the manner of the reference's own denoiser
    checks (target/tests/denoise.cpp: a noisy plane, depth and tilt edges, a
    checker albedo, young history) plus a random mix with sky pixels.  The
    distance, normal and albedo are rounded to FP16, the storage the GPU
    keeps them in, so both denoisers read identical features."""
    rng = np.random.default_rng(99)
    aspect = width / height
    reach = 0.5
    lens = np.array([0, 0, 0, 0, 0, -1, 1, 0, 0, 0, 1, 0, reach, aspect], np.float64)
    xs, ys = np.meshgrid(np.arange(width), np.arange(height))
    across = (2 * (xs + 0.5) / width - 1) * reach * aspect
    down = (1 - 2 * (ys + 0.5) / height) * reach
    ray = np.sqrt(1 + across ** 2 + down ** 2)
    fields = {}

    def field(value, length=8.0, depth=10.0, normal=(0, 0, 1), albedo=(0, 0, 0), leaf=1, demodulated=0, extra=0.0):
        n = width * height
        colour = np.broadcast_to(np.asarray(value, np.float64).reshape(height, width, -1), (height, width, 3)).reshape(n, 3).copy()
        lum = 0.2126 * colour[:, 0] + 0.7152 * colour[:, 1] + 0.0722 * colour[:, 2]
        moment = lum * lum + np.broadcast_to(np.asarray(extra, np.float64), (height, width)).reshape(n)
        dist = (np.broadcast_to(np.asarray(depth, np.float64), (height, width)) * ray).reshape(n).astype(np.float16).astype(np.float32)
        nrm = np.broadcast_to(np.asarray(normal, np.float64).reshape(-1, 3) if np.ndim(normal) == 1 else np.asarray(normal), (n, 3)).astype(np.float16).astype(np.float64)
        alb = np.broadcast_to(np.asarray(albedo, np.float64).reshape(-1, 3) if np.ndim(albedo) == 1 else np.asarray(albedo), (n, 3)).astype(np.float16).astype(np.float64)
        return dict(colour=colour, moment=moment, length=np.broadcast_to(np.asarray(length, np.float32), (height, width)).reshape(n).copy(),
                    distance=dist, normal=nrm.copy(), leaf=np.broadcast_to(np.asarray(leaf, np.uint32), (height, width)).reshape(n).copy(),
                    albedo=alb.copy(), demodulated=demodulated)

    noise = rng.uniform(-1, 1, (height, width))
    v = 0.5 + 0.3 * noise
    fields["plane"] = field(np.stack([v, v, v], -1), extra=0.01)
    right = xs >= width // 2
    v = np.where(right, 0.6, 0.4) + 0.3 * rng.uniform(-1, 1, (height, width))
    fields["depth_edge"] = field(np.stack([v, v, v], -1), depth=np.where(right, 12.0, 10.0), extra=0.02)
    tilt = np.where(right[..., None], np.array([0.8, 0, 0.6]), np.array([0, 0, 1.0])).reshape(-1, 3)
    fields["tilt_edge"] = field(np.stack([v, v, v], -1), normal=tilt, extra=0.02)
    checker = np.where(((xs // 4 + ys // 4) % 2) == 0, 0.2, 0.8)
    lit = 0.7 + 0.2 * rng.uniform(-1, 1, (height, width))
    alb = np.stack([checker, checker, checker], -1).reshape(-1, 3)
    fields["checker"] = field(np.stack([lit * checker] * 3, -1), albedo=alb, demodulated=1, extra=0.005)
    young = rng.integers(1, 6, (height, width)).astype(np.float32)
    v = 0.5 + 0.3 * rng.uniform(-1, 1, (height, width))
    fields["young"] = field(np.stack([v, v * 0.9, v * 0.8], -1), length=young, extra=0.01)
    n = width * height
    col = rng.gamma(1.5, 0.3, (n, 3))
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm[:, 2] = np.abs(nrm[:, 2])
    leaf = np.where(rng.random((height, width)) < 0.08, 0xFFFFFFFF, 3).astype(np.uint32)
    f = field(col.reshape(height, width, 3), length=rng.integers(1, 40, (height, width)).astype(np.float32), depth=rng.uniform(2, 30, (height, width)),
              normal=nrm, albedo=rng.uniform(0, 1, (n, 3)), leaf=leaf, demodulated=1, extra=rng.uniform(0, 0.05, (height, width)))
    fields["mixed"] = f
    return lens, fields


def denoise_fixture(dump: str, tmp: str) -> None:
    lens, fields = denoise_fields()
    out = {"lens": lens, "width": 64, "height": 48}
    for name, f in fields.items():
        path = os.path.join(tmp, f"denoise_{name}.bin")
        with open(path, "wb") as fh:
            fh.write(struct.pack("<3i", 64, 48, int(f["demodulated"])))
            fh.write(lens.astype("<f8").tobytes())
            for k in range(64 * 48):
                fh.write(f["colour"][k].astype("<f8").tobytes())
                fh.write(struct.pack("<d", float(f["moment"][k])))
                fh.write(struct.pack("<ff", float(f["length"][k]), float(f["distance"][k])))
                fh.write(f["normal"][k].astype("<f8").tobytes())
                fh.write(struct.pack("<I", int(f["leaf"][k])))
                fh.write(f["albedo"][k].astype("<f8").tobytes())
        res = os.path.join(tmp, f"denoise_{name}.out")
        subprocess.run([dump, "denoise", path, res], check=True)
        rgb = np.fromfile(res, "<f4").reshape(-1, 3)
        for k, v in f.items():
            out[f"{name}.{k}"] = v
        out[f"{name}.out"] = rgb
        print(" denoise", name, "mean in", f["colour"].mean(0), "out", rgb.mean(0))
    np.savez_compressed(os.path.join(HERE, "denoise.npz"), **out)


TEMPORAL_SIZE = (48, 32)


def _surface_record(surf: dict, k: int) -> bytes:
    return struct.pack("<f", float(surf["distance"][k])) + surf["normal"][k].astype("<f4").tobytes() + struct.pack("<I", int(surf["leaf"][k])) + \
        surf["albedo"][k].astype("<f4").tobytes()


def _fp16_surfaces(surf: dict) -> dict:
    """The first surfaces as the GPU stores them: FP16 distance, normal, albedo."""
    return {"distance": surf["distance"].astype(np.float16).astype(np.float32), "normal": surf["normal"].astype(np.float16).astype(np.float32),
            "albedo": surf["albedo"].astype(np.float16).astype(np.float32), "leaf": surf["leaf"].astype(np.uint32)}


# core/shown.cpp bayerPhase: the order a film factor's phases are drawn in
BAYER = {1: [0], 2: [0, 3, 1, 2], 3: [0, 7, 5, 2, 6, 4, 3, 1, 8], 4: [0, 10, 2, 8, 5, 15, 7, 13, 1, 11, 3, 9, 4, 14, 6, 12]}


def temporal_frames(scene: Scene, rng: np.random.Generator, factor: int = 1):
    """A seeded sequence of frames over config 2's small scene, the camera
    still, then moving, then still again: per frame the lens now and before,
    the record's light and first surfaces (each pixel's last sample, jittered
    within the shown pixel its phase aims at) and the G-buffer (through that
    shown pixel's centre, core/camera.cpp:51 filmCentre), on the drawn grid
    of TEMPORAL_SIZE at a film factor of `factor`, the phases in Bayer
    order."""
    import oracle.port as op
    w, h = TEMPORAL_SIZE
    build = dict(min_depth=5, max_depth=9, split_steps=64)
    base = op.lens_of(scene, w, h)

    def moved(lens, shift, turn):
        eye = lens[0:3] + np.asarray(shift)
        fw = lens[3:6] + turn * lens[6:9]
        fw = fw / np.linalg.norm(fw)
        rt = np.cross(fw, np.array([0.0, 0.0, 1.0]))
        rt = rt / np.linalg.norm(rt)
        up = np.cross(rt, fw)
        return np.concatenate([eye, fw, rt, up, lens[12:14]])

    lenses = [base, base, moved(base, [0.15, 0.05, 0.0], 0.01), moved(base, [0.3, 0.1, 0.02], 0.02), moved(base, [0.3, 0.1, 0.02], 0.02)]
    plan = [(0, 0), (1, 0), (1, 1), (1, 1), (1, 0)]  # (kept, moved)
    sun = np.array([0.3, -0.4, 0.87])
    sun = sun / np.linalg.norm(sun)
    frames = []
    for f, (kept, move) in enumerate(plan):
        lens = lenses[f]
        phase = BAYER[factor][f % (factor * factor)]
        column, row = phase % factor, phase // factor
        centre = np.tile([(column + 0.5) / factor, (row + 0.5) / factor], (w * h, 1))
        jitter = (np.array([column, row]) + rng.random((w * h, 2))) / factor
        gbuffer = _fp16_surfaces(op.traced_surfaces(scene, w, h, build, lens=lens, offsets=None if factor == 1 else centre))
        first = _fp16_surfaces(op.traced_surfaces(scene, w, h, build, lens=lens, offsets=jitter))
        hit = first["leaf"] != 0xFFFFFFFF
        shade = 0.3 + 0.7 * np.clip(first["normal"].astype(np.float64) @ sun, 0, None)
        light = np.where(hit[:, None], first["albedo"].astype(np.float64) * shade[:, None], np.array([0.4, 0.5, 0.7]))
        light = light * (1 + 0.3 * rng.normal(size=light.shape))
        light = np.clip(light, 0, None)
        frames.append(dict(lens=lens, before=lenses[max(f - 1, 0)], kept=kept, moved=move, light=light, first=first, gbuffer=gbuffer,
                           factor=factor, phase=phase))
    return frames


def temporal_fixture(dump: str, tmp: str, factor: int = 1) -> None:
    """tests/golden/temporal.npz (a film factor of 1) and
    temporal_factor<k>.npz: the reference's temporalFrame over a sequence of
    frames, each fed the state the one before left."""
    scene = Scene.load(os.path.join(HERE, "scenes", "c2_small.npz"))
    w, h = TEMPORAL_SIZE
    n = w * h
    frames = temporal_frames(scene, np.random.default_rng(2024 + factor - 1), factor)
    state = None
    out = {"width": w, "height": h, "frames": len(frames), "factor": factor}
    pixel = np.dtype([("colour", "<f8", 3), ("moment", "<f8"), ("length", "<f4"), ("distance", "<f4"), ("normal", "<f8", 3), ("leaf", "<u4"),
                      ("albedo", "<f8", 3)])
    for f, fr in enumerate(frames):
        path = os.path.join(tmp, f"temporal_{f}.bin")
        before_phase = frames[f - 1]["phase"] if f else 0
        with open(path, "wb") as fh:
            fh.write(struct.pack("<10i", w, h, fr["moved"], 0, fr["kept"], 1, factor, fr["phase"], factor, before_phase))
            fh.write(fr["lens"].astype("<f8").tobytes())
            fh.write(fr["before"].astype("<f8").tobytes())
            before = state if state is not None else np.zeros(n, pixel)
            for k in range(n):
                fh.write(fr["light"][k].astype("<f8").tobytes())
                fh.write(_surface_record(fr["first"], k))
                fh.write(_surface_record(fr["gbuffer"], k))
                fh.write(before[k].tobytes())
        res = os.path.join(tmp, f"temporal_{f}.out")
        subprocess.run([dump, "temporal", path, res], check=True)
        raw = open(res, "rb").read()
        after = np.frombuffer(raw[: n * pixel.itemsize], pixel).copy()
        image = np.frombuffer(raw[n * pixel.itemsize:], "<f4").reshape(n, 3).copy()
        for key in ("lens", "before", "kept", "moved", "light", "phase"):
            out[f"{f}.{key}"] = fr[key]
        out[f"{f}.before_phase"] = before_phase
        for part in ("first", "gbuffer"):
            for key, v in fr[part].items():
                out[f"{f}.{part}.{key}"] = v
        for key in pixel.names:
            out[f"{f}.state.{key}"] = after[key]
        out[f"{f}.image"] = image
        state = after
        print(" temporal frame", f, "factor", factor, "phase", fr["phase"], "kept", fr["kept"], "moved", fr["moved"], "held",
              float((after["length"] > 1).mean()), "image", image.mean(0))
    np.savez_compressed(os.path.join(HERE, "temporal.npz" if factor == 1 else f"temporal_factor{factor}.npz"), **out)


def upscale_fixture(dump: str, tmp: str) -> None:
    """tests/golden/upscale.npz: the reference's upscaledFrame
    (plugins/reconstruction/upscale/upscale.cpp) over a sequence of frames
    at a film factor of 2, each fed the state the one before left: the
    temporal fixture's factor-2 frames (their lenses, FP16 G-buffer
    distances and the reference's own temporal images as the drawn frames),
    then three still frames that settle, a restart, and two frames at a film
    factor of 4 without a G-buffer (every sample sky)."""
    import oracle.port as op
    t = np.load(os.path.join(HERE, "temporal_factor2.npz"))
    dw, dh = int(t["width"]), int(t["height"])
    rng = np.random.default_rng(77)
    seq = []
    for f in range(int(t["frames"])):
        seq.append(dict(factor=2, phase=int(t[f"{f}.phase"]), moved=int(t[f"{f}.moved"]), restarted=0, lens=t[f"{f}.lens"], before=t[f"{f}.before"],
                        internal=t[f"{f}.image"].reshape(-1, 3), distance=t[f"{f}.gbuffer.distance"]))
    last = seq[-1]
    for k in range(3):
        seq.append(dict(last, phase=BAYER[2][(len(seq)) % 4], moved=0, before=last["lens"],
                        internal=np.clip(last["internal"] * (1 + 0.05 * rng.normal(size=last["internal"].shape)), 0, None).astype(np.float32)))
    seq.append(dict(seq[-1], phase=BAYER[2][len(seq) % 4], restarted=1))
    small = (dw // 2, dh // 2)
    for k in range(2):
        internal = (0.5 + 0.4 * np.sin(np.arange(small[0] * small[1] * 3) * 0.37)).astype(np.float32).reshape(-1, 3)
        seq.append(dict(factor=4, phase=BAYER[4][k], moved=0, restarted=0, lens=last["lens"], before=last["lens"], internal=internal, distance=None))
    out = {"frames": len(seq)}
    state = None  # (width, height, colour, depth, moved, settling)
    for f, fr in enumerate(seq):
        factor = fr["factor"]
        ddw, ddh = (dw, dh) if factor == 2 else small
        w, h = ddw * factor, ddh * factor
        kept = int(state is not None and state[0] == w and state[1] == h and not fr["restarted"])
        before_moved = state[4] if state is not None else 0
        before_settling = state[5] if state is not None else 0
        path = os.path.join(tmp, f"upscale_{f}.bin")
        with open(path, "wb") as fh:
            fh.write(struct.pack("<10i", w, h, factor, fr["phase"], fr["moved"], fr["restarted"], 1 if state is not None and kept else 0,
                                 before_moved, before_settling, 0 if fr["distance"] is None else 1))
            fh.write(np.asarray(fr["lens"], "<f8").tobytes())
            fh.write(np.asarray(fr["before"], "<f8").tobytes())
            fh.write(np.asarray(fr["internal"], "<f4").tobytes())
            if fr["distance"] is not None:
                fh.write(np.asarray(fr["distance"], "<f4").tobytes())
            if state is not None and kept:
                rec = np.zeros(w * h, [("c", "<f8", 3), ("d", "<f4")])
                rec["c"], rec["d"] = state[2], state[3]
                fh.write(rec.tobytes())
        res = os.path.join(tmp, f"upscale_{f}.out")
        subprocess.run([dump, "upscale", path, res], check=True)
        raw = open(res, "rb").read()
        moved_after, settling_after = struct.unpack("<2i", raw[:8])
        px = np.frombuffer(raw[8:8 + w * h * 28], [("c", "<f8", 3), ("d", "<f4")])
        image = np.frombuffer(raw[8 + w * h * 28:], "<f4").reshape(-1, 3)
        for key in ("factor", "phase", "moved", "restarted", "lens", "before", "internal"):
            out[f"{f}.{key}"] = fr[key]
        if fr["distance"] is not None:
            out[f"{f}.distance"] = fr["distance"]
        out[f"{f}.kept"] = kept
        out[f"{f}.before_moved"], out[f"{f}.before_settling"] = before_moved, before_settling
        out[f"{f}.colour"], out[f"{f}.depth"], out[f"{f}.image"] = px["c"].copy(), px["d"].copy(), image.copy()
        out[f"{f}.moved_after"], out[f"{f}.settling_after"] = moved_after, settling_after
        state = (w, h, px["c"].copy(), px["d"].copy(), moved_after, settling_after)
        print(" upscale frame", f, "factor", factor, "phase", fr["phase"], "kept", kept, "moved", fr["moved"], "settling after", settling_after,
              "image", image.mean(0))
    np.savez_compressed(os.path.join(HERE, "upscale.npz"), **out)


def sobol_fixture(dump: str, tmp: str) -> None:
    """tests/golden/sobol.npz: the reference's sobolNumber and sobolPair
    (plugins/sampler/sobol/sobol.cpp) of 20000 seeded keys: streams of 64
    random bits, sample indices below 2^17 (past the 16 bits the sequence's
    place keeps), coordinates below 28."""
    rng = np.random.default_rng(28)
    n = 20000
    keys = np.zeros(n, [("stream", "<u8"), ("index", "<u4"), ("coordinate", "<u4")])
    keys["stream"] = rng.integers(0, 2 ** 63, n, dtype=np.uint64) * 2 + rng.integers(0, 2, n, dtype=np.uint64)
    keys["index"] = rng.integers(0, 1 << 17, n)
    keys["coordinate"] = rng.integers(0, 28, n)
    path, res = os.path.join(tmp, "sobol.bin"), os.path.join(tmp, "sobol.out")
    keys.tofile(path)
    subprocess.run([dump, "sobol", path, res], check=True)
    values = np.fromfile(res, "<f8").reshape(n, 3)
    np.savez_compressed(os.path.join(HERE, "sobol.npz"), stream=keys["stream"], index=keys["index"], coordinate=keys["coordinate"],
                        number=values[:, 0], pair=values[:, 1:])
    print(" sobol keys", n)


def upsample_fixture(dump: str, tmp: str) -> None:
    """tests/golden/upsample.npz: the reference's upsampledImage
    (plugins/reconstruction/upsample/upsample.cpp) of seeded drawn frames at
    film factors 2, 3 and 4 (shown 96 x 48)."""
    rng = np.random.default_rng(91)
    out = {}
    for factor in (2, 3, 4):
        w, h = 96, 48
        drawn = (rng.random((h // factor) * (w // factor) * 3) * rng.choice([0.5, 2.0, 30.0], (h // factor) * (w // factor) * 3)).astype(np.float32)
        path, res = os.path.join(tmp, f"upsample_{factor}.bin"), os.path.join(tmp, f"upsample_{factor}.out")
        with open(path, "wb") as fh:
            fh.write(struct.pack("<3i", w, h, factor))
            fh.write(drawn.astype("<f4").tobytes())
        subprocess.run([dump, "upsample", path, res], check=True)
        out[f"{factor}.drawn"] = drawn.reshape(-1, 3)
        out[f"{factor}.shown"] = np.fromfile(res, "<f4").reshape(-1, 3)
        out[f"{factor}.size"] = np.array([w, h])
    np.savez_compressed(os.path.join(HERE, "upsample.npz"), **out)
    print(" upsample factors 2, 3, 4")


# The benchmark's own octree of config 2 and the cells sampled from it for
# tests/golden/cutdeep_c2.npz
DEEP_BUILD = (7, 11, 32)
DEEP_SAMPLE = 2000


def deep_cut_fixture(dump: str, tmp: str) -> None:
    """tests/golden/cutdeep_c2.npz: the reference's cutCell of a seeded
    sample of the cells of the octree the benchmark builds over config 2
    (down to level 11), each cut from the root along its path as the
    reference's own recursion does; the product's host build must hold the
    same programs there."""
    import ctypes

    import kodanuki_gb300 as K
    sc = Scene.load(os.path.join(HERE, "scenes", "c2.npz"))
    L = K.library()
    h = ctypes.c_void_p()
    assert L.kdn_open(-1, ctypes.byref(h)) == K.KDN_OK
    b = K.Backend.__new__(K.Backend)
    b.lib, b.handle, b.scene = L, h, None
    b.load(sc)
    b.build(*DEEP_BUILD)
    n = b.world_stats()["cells"]
    index = np.sort(np.random.default_rng(77).choice(n, DEEP_SAMPLE, replace=False)).astype(np.uint64)
    targets = np.array([(lvl, *place) for lvl, place, _, _ in (b.world_cell(int(i)) for i in index)], np.uint32)
    b.close()
    tp = os.path.join(tmp, "deep.targets")
    with open(tp, "wb") as fh:
        fh.write(struct.pack("<I", len(targets)))
        fh.write(targets.astype("<u4").tobytes())
    sdf = os.path.join(tmp, "c2_deep.sdf")
    gen, kw, _, _ = SCENES["c2"]
    open(sdf, "w").write(gen(**kw))
    cp = os.path.join(tmp, "deep.cut")
    subprocess.run([dump, "cells", sdf, tp, cp], check=True)
    cells = read_cut(cp)
    head = np.array([(c[0], *c[1], c[2], len(c[3])) for c in cells], np.uint32)
    objects, results, counts, digests = [], [], [], []
    for c in cells:
        for obj, res, steps in c[3]:
            objects.append(obj)
            results.append(res)
            counts.append(len(steps))
            digests.append(step_digest(steps))
    np.savez_compressed(os.path.join(HERE, "cutdeep_c2.npz"), build=np.array(DEEP_BUILD), index=index, head=head, objects=np.array(objects, np.uint32),
                        results=np.array(results, np.uint32), counts=np.array(counts, np.uint32), digests=np.array(digests, np.uint64))
    print(" deep cut cells", len(cells), "of", n, "levels", np.bincount(head[:, 0]).tolist(), "programs", len(objects))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-bin", default=os.path.join(ROOT, "oracle", "_ref"))
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    dump = os.path.join(args.ref_bin, "kdn_ref_dump")
    render = os.path.join(args.ref_bin, "kodanuki")
    os.makedirs(os.path.join(HERE, "scenes"), exist_ok=True)
    tmp = tempfile.mkdtemp()
    if args.only in (None, "denoise"):
        denoise_fixture(dump, tmp)
    if args.only in (None, "temporal"):
        temporal_fixture(dump, tmp)
        temporal_fixture(dump, tmp, factor=2)
    if args.only in (None, "temporal", "upscale"):
        upscale_fixture(dump, tmp)
    if args.only in (None, "upsample"):
        upsample_fixture(dump, tmp)
    if args.only in (None, "sobol"):
        sobol_fixture(dump, tmp)
    if args.only in (None, "cutdeep"):
        deep_cut_fixture(dump, tmp)
    for name, (gen, kw, nrays, depth) in SCENES.items():
        if args.only and name != args.only and not (args.only == "serve" and name.startswith("serve_")):
            continue
        sdf = os.path.join(tmp, name + ".sdf")
        open(sdf, "w").write(gen(**kw))
        js = os.path.join(tmp, name + ".json")
        subprocess.run([dump, "scene", sdf, js], check=True)
        scene = Scene.from_reference_json(json.load(open(js)))
        scene.save(os.path.join(HERE, "scenes", name + ".npz"))
        print(name, "programs", scene.program_count, "steps", len(scene.steps))
        if name in IMAGES:
            reference_images(render, sdf, name, tmp, scene)
        if name in SOBOL_IMAGES:
            reference_images(render, sdf, name, tmp, scene, sampler="sobol")
        if name in SKY_MAP_IMAGES:
            reference_images(render, sdf, name, tmp, scene, sampler="sky_map")
        if name in EACH_LAMP_IMAGES:
            reference_images(render, sdf, name, tmp, scene, sampler="each_lamp_first")
        if name in SIZED_IMAGES:
            reference_sized_images(render, sdf, name, tmp, scene)
        if nrays:
            rng = np.random.default_rng(1234)
            rays = np.concatenate([camera_rays(scene, nrays // 2, rng), scattered_rays(scene, nrays - nrays // 2, rng)])
            rp = os.path.join(tmp, name + ".rays")
            hp = os.path.join(tmp, name + ".hits")
            rays.tofile(rp)
            subprocess.run([dump, "trace", sdf, rp, hp], check=True)
            raw = np.fromfile(hp, np.uint8).reshape(-1, 44)
            kind = raw[:, 0:4].copy().view("<u4")[:, 0]
            geo = raw[:, 4:32].copy().view("<f4")
            ids = raw[:, 32:40].copy().view("<u4")
            share = raw[:, 40:44].copy().view("<f4")[:, 0]
            far = float(scene.render["far"])
            target = np.array(scene.camera["target"])
            np.savez_compressed(os.path.join(HERE, f"trace_{name}.npz"), rays=rays, kind=kind, distance=geo[:, 0], point=geo[:, 1:4],
                                normal=geo[:, 4:7], leaf=ids[:, 0], other=ids[:, 1], share=share,
                                reach_lower=target - far, reach_size=np.full(3, 2 * far))
            print(" trace", len(rays), "hit", int((kind == 1).sum()))
        if depth:
            cp = os.path.join(tmp, name + ".cut")
            subprocess.run([dump, "cut", sdf, str(depth), cp], check=True)
            cells = read_cut(cp)
            head = np.array([(c[0], *c[1], c[2], len(c[3])) for c in cells], np.uint32)
            objects, results, counts, allsteps = [], [], [], []
            for c in cells:
                for obj, res, steps in c[3]:
                    objects.append(obj)
                    results.append(res)
                    counts.append(len(steps))
                    allsteps.append(steps)
            steps = np.concatenate(allsteps) if allsteps else np.zeros(0, STEP_DTYPE)
            extra = {"steps": steps} if len(steps) < 100_000 else {"digests": np.array([step_digest(s) for s in allsteps], np.uint64)}
            np.savez_compressed(os.path.join(HERE, f"cut_{name}.npz"), depth=depth, head=head, objects=np.array(objects, np.uint32),
                                results=np.array(results, np.uint32), counts=np.array(counts, np.uint32), **extra)
            print(" cut cells", len(cells), "programs", len(objects))


if __name__ == "__main__":
    main()
