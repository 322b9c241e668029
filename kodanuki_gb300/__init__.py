"""kodanuki_gb300 -- GB300 backend for the Kodanuki spectral SDF path tracer.

The product is ``libkdn_gb300.so`` (C ABI in include/kdn.h), built in-tree
by :mod:`kodanuki_gb300.build`.  This module is the host-side mirror of the
reference's backend interface for Python callers and tests: it loads the
library (and fails loudly when it is missing), uploads a compiled scene's
blocks and runs the entry points.

    from kodanuki_gb300 import Backend
    from kodanuki_gb300.scene import Scene
    scene = Scene.load("tests/golden/scenes/c1.npz")
    with Backend() as b:
        b.load(scene)
        b.build(min_depth=6, max_depth=10, split_steps=96)
        hits = b.extend(rays)
        image = b.render(width=256, height=256, samples=16)
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .scene import STEP_DTYPE, Scene

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libkdn_gb300.so")

KDN_OK, KDN_BAD_ARG, KDN_OOM, KDN_TIMEOUT, KDN_CUDA_ERROR, KDN_NOT_READY, KDN_NO_DEVICE = range(7)

# core/batch.h:125 Ray (36 bytes) and core/batch.h:157 Hit (56 bytes).
RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("direction", "<f4", 3), ("far", "<f4"), ("inside", "u1"), ("pad", "u1", 3), ("within", "<u4")])
HIT_DTYPE = np.dtype([("kind", "u1"), ("pad0", "u1", 3), ("distance", "<f4"), ("point", "<f4", 3), ("normal", "<f4", 3), ("leaf", "<u4"),
                      ("other", "<u4"), ("share", "<f4"), ("loosened", "<f4"), ("leaf_kind", "u1"), ("pad1", "u1", 3), ("cell", "<u4")])
PROGRAM_REF_DTYPE = np.dtype([("first", "<u4"), ("count", "<u4"), ("result", "<u4")])
MATERIAL_DTYPE = np.dtype([("kind", "<u4"), ("albedo", "<f4", 3), ("roughness", "<f4"), ("refraction", "<f4"), ("dispersion", "<f4"),
                           ("absorb", "<f4", 3), ("glow", "<f4", 3), ("strength", "<f4"), ("flags", "<u4"),
                           ("scatter", "<f4"), ("lean", "<f4"), ("pad", "<u4")])
LIGHT_DTYPE = np.dtype([("kind", "<u4"), ("radius", "<f4"), ("angle", "<f4"), ("pad", "<f4"), ("at", "<f8", 3), ("direction", "<f8", 3),
                        ("along", "<f8", 3), ("across", "<f8", 3), ("power", "<f8", 3)])
SKY_DTYPE = np.dtype([("zenith", "<f8", 3), ("horizon", "<f8", 3), ("ground", "<f8", 3), ("glow", "<f8", 3), ("strength", "<f8"),
                      ("spread", "<f8"), ("kind", "<u4"), ("haze", "<f4"), ("stars", "<u4"), ("star_count", "<f4"),
                      ("star_strength", "<f4"), ("star_angle", "<f4")])
CAMERA_DTYPE = np.dtype([("eye", "<f8", 3), ("target", "<f8", 3), ("up", "<f8", 3), ("fov", "<f8"), ("aperture", "<f8"), ("focus", "<f8")])
REGION_DTYPE = np.dtype([("lower", "<f8", 3), ("size", "<f8", 3)])
PATTERN_DTYPE = np.dtype([("first", "<u4"), ("count", "<u4"), ("result", "<u4"), ("argument_first", "<u4"), ("argument_count", "<u4"),
                          ("stop_first", "<u4"), ("stop_count", "<u4"), ("world", "<u4")])
PLACEMENT_DTYPE = np.dtype([("linear", "<f8", (3, 3)), ("origin", "<f8", 3)])
BOUNDARY_DTYPE = np.dtype([("rarer", "<f8", (17, 32)), ("denser", "<f8", (17, 32)), ("rarer_average", "<f8", 17), ("denser_average", "<f8", 17),
                           ("rarer_through", "<f8", 17)])
FINISH_DTYPE = np.dtype([("kind", "<u4"), ("sharp", "<u4"), ("exact", "<u4"), ("loses_much", "<u4"), ("width", "<f8"), ("facet_share", "<f8"),
                         ("body", "<f8"), ("index", "<f8"), ("coat_front", "<f8"), ("coat_twice", "<f8"), ("coat_room", "<f8"),
                         ("escape_average", "<f8"), ("escape", "<f8", 32), ("film", "<f8", 2)])
assert RAY_DTYPE.itemsize == 36 and HIT_DTYPE.itemsize == 56 and MATERIAL_DTYPE.itemsize == 72 and LIGHT_DTYPE.itemsize == 136
assert FINISH_DTYPE.itemsize == 352 and SKY_DTYPE.itemsize == 136


class BuildOptions(ctypes.Structure):
    _fields_ = [("min_depth", ctypes.c_int32), ("max_depth", ctypes.c_int32), ("split_steps", ctypes.c_uint32), ("pad", ctypes.c_uint32)]


class Frame(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("samples", ctypes.c_int32), ("surfaces", ctypes.c_int32),
                ("seed", ctypes.c_int32), ("first", ctypes.c_uint32), ("accumulate", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("factor", ctypes.c_uint32), ("phase", ctypes.c_uint32), ("collisions", ctypes.c_int32), ("split", ctypes.c_uint32)]


# core/shown.cpp bayerPhase: the order a film factor's phases are drawn in
BAYER = {1: [0], 2: [0, 3, 1, 2], 3: [0, 7, 5, 2, 6, 4, 3, 1, 8], 4: [0, 10, 2, 8, 5, 15, 7, 13, 1, 11, 3, 9, 4, 14, 6, 12]}


FRAME_DENOISE = 1  # include/kdn.h KDN_FRAME_DENOISE
FRAME_RESTART = 2  # include/kdn.h KDN_FRAME_RESTART
FRAME_TEMPORAL = 4  # include/kdn.h KDN_FRAME_TEMPORAL
FRAME_UPSAMPLE = 8  # include/kdn.h KDN_FRAME_UPSAMPLE
FRAME_SOBOL = 16  # include/kdn.h KDN_FRAME_SOBOL
FRAME_SKY_MAP = 32  # include/kdn.h KDN_FRAME_SKY_MAP
FRAME_EACH_LAMP = 64  # include/kdn.h KDN_FRAME_EACH_LAMP


class FrameStats(ctypes.Structure):
    _fields_ = [("total_ms", ctypes.c_double), ("trace_ms", ctypes.c_double), ("shade_ms", ctypes.c_double), ("other_ms", ctypes.c_double),
                ("segments", ctypes.c_uint64), ("march_steps", ctypes.c_uint64), ("program_steps", ctypes.c_uint64),
                ("launches", ctypes.c_uint32), ("longest_march", ctypes.c_uint32), ("capped_rays", ctypes.c_uint64),
                ("trace_launches", ctypes.c_uint32), ("carried_rays", ctypes.c_uint32)]


class KdnError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"kdn status {status}: {message}")
        self.status = status


# Every symbol include/kdn.h declares.
EXPORTS = [
    "kdn_status_string", "kdn_last_error", "kdn_open", "kdn_close", "kdn_upload_block", "kdn_build", "kdn_world_stats",
    "kdn_world_cell", "kdn_extend", "kdn_extend_device", "kdn_render", "kdn_render_device", "kdn_frame_stats_get", "kdn_flush_l2",
    "kdn_frame_surfaces", "kdn_frame_record", "kdn_world_march", "kdn_world_locate", "kdn_temporal_device", "kdn_denoise", "kdn_denoise_device", "kdn_denoise_static",
    "kdn_open_sharing", "kdn_set_frame_budget", "kdn_serve_open", "kdn_serve_add_scene", "kdn_serve_submit", "kdn_serve_wait", "kdn_serve_end_session",
    "kdn_serve_latency", "kdn_serve_last_error", "kdn_serve_close", "kdn_serve_cancel_queued", "kdn_set_sm_limit", "kdn_serve_reset_latency",
    "kdn_guide_open", "kdn_guide_close", "kdn_guide_last_error", "kdn_guide_sizes", "kdn_guide_get_params", "kdn_guide_set_params",
    "kdn_guide_gradients", "kdn_guide_train", "kdn_guide_query", "kdn_guide_clear_samples", "kdn_guide_ready", "kdn_set_guide",
    "kdn_guide_select", "kdn_set_march_budget", "kdn_upscale_device", "kdn_upsample_device",
]

REQUEST_INTERACTIVE = 4


class ServeOptions(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("slots", ctypes.c_uint32), ("budget_bytes", ctypes.c_uint64), ("batch_slots", ctypes.c_uint32),
                ("batch_sm_percent", ctypes.c_uint32), ("batch_frame_bytes", ctypes.c_uint64)]


class Request(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_uint32), ("width", ctypes.c_int32), ("height", ctypes.c_int32), ("samples", ctypes.c_int32),
                ("surfaces", ctypes.c_int32), ("seed", ctypes.c_int32), ("flags", ctypes.c_uint32), ("pad", ctypes.c_uint32),
                ("session", ctypes.c_uint64)]


class Served(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("frame", ctypes.c_uint32), ("queued_ms", ctypes.c_double), ("render_ms", ctypes.c_double),
                ("latency_ms", ctypes.c_double)]


class DenoiseFrame(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("demodulated", ctypes.c_uint32), ("pad", ctypes.c_uint32),
                ("eye", ctypes.c_double * 3), ("forward", ctypes.c_double * 3), ("right", ctypes.c_double * 3), ("up", ctypes.c_double * 3),
                ("reach", ctypes.c_double), ("aspect", ctypes.c_double)]



class TemporalFrame(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("moved", ctypes.c_uint32), ("recounted", ctypes.c_uint32),
                ("kept", ctypes.c_uint32), ("factor", ctypes.c_uint32), ("phase", ctypes.c_uint32), ("before_factor", ctypes.c_uint32),
                ("before_phase", ctypes.c_uint32), ("pad", ctypes.c_uint32), ("now", ctypes.c_double * 14), ("before", ctypes.c_double * 14)]


class UpscaleFrame(ctypes.Structure):
    """include/kdn.h kdn_upscale_frame."""
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("factor", ctypes.c_uint32), ("phase", ctypes.c_uint32),
                ("kept", ctypes.c_uint32), ("settling", ctypes.c_uint32), ("now", ctypes.c_double * 14), ("before", ctypes.c_double * 14)]


class UpscaleBuffers(ctypes.Structure):
    """include/kdn.h kdn_upscale_buffers: device pointers."""
    _fields_ = [(name, ctypes.c_void_p) for name in ("internal", "distance", "before", "after", "image")]


class TemporalBuffers(ctypes.Structure):
    """include/kdn.h kdn_temporal_buffers: device pointers."""
    _fields_ = [(name, ctypes.c_void_p) for name in (
        "light", "first_distance", "first_normal", "first_albedo", "first_leaf", "centre_distance", "centre_normal", "centre_albedo",
        "centre_leaf", "before_colour", "before_moment", "before_length", "before_distance", "before_normal", "before_leaf", "colour",
        "moment", "length", "image")]


_lib = None


def library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libkdn_gb300.so.  There is no fallback: a missing library is an
    error, and :func:`kodanuki_gb300.build.build` makes it."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    L.kdn_status_string.restype = ctypes.c_char_p
    L.kdn_status_string.argtypes = [ctypes.c_int]
    L.kdn_last_error.restype = ctypes.c_char_p
    L.kdn_last_error.argtypes = [P]
    L.kdn_open.argtypes = [ctypes.c_int, ctypes.POINTER(P)]
    L.kdn_close.argtypes = [P]
    L.kdn_upload_block.argtypes = [P, ctypes.c_char_p, P, ctypes.c_size_t, ctypes.c_size_t]
    L.kdn_build.argtypes = [P, ctypes.POINTER(BuildOptions)]
    L.kdn_world_stats.argtypes = [P, P]
    L.kdn_world_cell.argtypes = [P, ctypes.c_uint64, P, P, P, P, P, ctypes.c_size_t]
    L.kdn_extend.argtypes = [P, P, ctypes.c_uint32, P]
    L.kdn_extend_device.argtypes = [P, P, ctypes.c_uint32, P, P]
    L.kdn_render.argtypes = [P, ctypes.POINTER(Frame), P]
    L.kdn_render_device.argtypes = [P, ctypes.POINTER(Frame), P, P]
    L.kdn_frame_stats_get.argtypes = [P, ctypes.POINTER(FrameStats)]
    L.kdn_flush_l2.argtypes = [P]
    L.kdn_frame_surfaces.argtypes = [P, P, P, P, P]
    L.kdn_frame_record.argtypes = [P, P, P, P, P, P]
    L.kdn_world_march.argtypes = [P, ctypes.c_uint64, P, ctypes.c_uint32, P, ctypes.c_size_t, P]
    L.kdn_world_locate.argtypes = [P, P, ctypes.c_uint32, P, P]
    L.kdn_temporal_device.argtypes = [P, ctypes.POINTER(TemporalFrame), ctypes.POINTER(TemporalBuffers), P]
    L.kdn_upscale_device.argtypes = [P, ctypes.POINTER(UpscaleFrame), ctypes.POINTER(UpscaleBuffers), P]
    L.kdn_upsample_device.argtypes = [P, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint32, P, P, P]
    L.kdn_denoise.argtypes = [P, ctypes.POINTER(DenoiseFrame), P, P, P, P, P, P, P, P]
    L.kdn_denoise_device.argtypes = [P, ctypes.POINTER(DenoiseFrame), P, P, P, P, P, P, P, P, P]
    L.kdn_denoise_static.argtypes = [ctypes.POINTER(DenoiseFrame), P, P, P, P, P, P, P, P, P]
    L.kdn_open_sharing.argtypes = [P, ctypes.c_int, ctypes.POINTER(P)]
    L.kdn_set_frame_budget.argtypes = [P, ctypes.c_uint64]
    L.kdn_set_sm_limit.argtypes = [P, ctypes.c_int]
    L.kdn_set_march_budget.argtypes = [P, ctypes.c_uint32]
    L.kdn_serve_reset_latency.argtypes = [P]
    L.kdn_serve_open.argtypes = [ctypes.POINTER(ServeOptions), ctypes.POINTER(P)]
    L.kdn_serve_add_scene.argtypes = [P, P, ctypes.POINTER(ctypes.c_uint32)]
    L.kdn_serve_submit.argtypes = [P, ctypes.POINTER(Request), P, ctypes.POINTER(ctypes.c_uint64)]
    L.kdn_serve_wait.argtypes = [P, ctypes.c_uint64, ctypes.POINTER(Served)]
    L.kdn_serve_end_session.argtypes = [P, ctypes.c_uint64]
    L.kdn_serve_latency.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64)]
    L.kdn_serve_last_error.restype = ctypes.c_char_p
    L.kdn_serve_last_error.argtypes = [P]
    L.kdn_serve_close.argtypes = [P]
    L.kdn_serve_cancel_queued.argtypes = [P, ctypes.POINTER(ctypes.c_uint64)]
    L.kdn_guide_open.argtypes = [ctypes.c_int, P, ctypes.POINTER(P)]
    L.kdn_guide_close.argtypes = [P]
    L.kdn_guide_last_error.restype = ctypes.c_char_p
    L.kdn_guide_last_error.argtypes = []
    L.kdn_guide_sizes.argtypes = [P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    L.kdn_guide_get_params.argtypes = [P, P, P]
    L.kdn_guide_set_params.argtypes = [P, P, P]
    L.kdn_guide_gradients.argtypes = [P, P, ctypes.c_uint32, P, P, P]
    L.kdn_guide_train.argtypes = [P, P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, P]
    L.kdn_guide_query.argtypes = [P, P, ctypes.c_uint32, P]
    L.kdn_guide_clear_samples.argtypes = [P]
    L.kdn_guide_ready.argtypes = [P]
    L.kdn_set_guide.argtypes = [P, P, ctypes.c_float, ctypes.c_uint32]
    L.kdn_guide_select.argtypes = [P, ctypes.POINTER(Frame), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    for name in EXPORTS:
        fn = getattr(L, name)
        if name not in ("kdn_status_string", "kdn_last_error", "kdn_serve_last_error", "kdn_guide_last_error"):
            fn.restype = ctypes.c_int
    _lib = L
    return L


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


def scene_blocks(scene: Scene) -> dict[str, np.ndarray]:
    """The blocks a reference host would upload for a compiled scene
    (core/block.h Block; the names of include/kdn.h)."""
    refs = np.zeros(scene.program_count, PROGRAM_REF_DTYPE)
    refs["first"] = scene.program_first[:-1]
    refs["count"] = np.diff(scene.program_first)
    refs["result"] = scene.program_result
    m = scene.materials
    mats = np.zeros(len(m["kind"]), MATERIAL_DTYPE)
    mats["kind"] = m["kind"]
    mats["albedo"] = m["albedo"]
    mats["roughness"] = m["roughness"]
    mats["refraction"] = m["refraction"]
    mats["dispersion"] = m["dispersion"]
    mats["absorb"] = m["absorb"]
    mats["glow"] = m["glow"]
    mats["strength"] = m["strength"]
    mats["flags"] = m["patterned"]
    mats["scatter"] = m["scatter"] if "scatter" in m else 0
    mats["lean"] = m["lean"] if "lean" in m else 0
    finishes = None
    if "finish_kind" in m:
        finishes = np.zeros(len(m["finish_kind"]), FINISH_DTYPE)
        for k in ("kind", "sharp", "exact", "loses_much", "width", "facet_share", "body", "index", "escape_average", "escape", "film"):
            finishes[k] = m["finish_" + k]
        finishes["coat_front"] = m["finish_coating"][:, 0]
        finishes["coat_twice"] = m["finish_coating"][:, 1]
        finishes["coat_room"] = m["finish_coating"][:, 2]
    l = scene.lights
    lights = np.zeros(len(l["kind"]), LIGHT_DTYPE)
    for k in ("kind", "radius", "angle", "at", "direction", "along", "across", "power"):
        lights[k] = l[k]
    sky = np.zeros(1, SKY_DTYPE)
    for k in ("zenith", "horizon", "ground"):
        sky[k] = scene.sky[k]
    for k in ("glow", "strength", "spread", "kind", "haze", "stars", "star_count", "star_strength", "star_angle"):
        if k in scene.sky:
            sky[k] = scene.sky[k]
    cam = np.zeros(1, CAMERA_DTYPE)
    for k in ("eye", "target", "up", "fov", "aperture", "focus"):
        cam[k] = scene.camera[k]
    region = np.zeros(1, REGION_DTYPE)
    region["lower"] = scene.region_lower
    region["size"] = scene.region_size
    blocks = {
        "scene.steps": np.ascontiguousarray(scene.steps),
        "scene.programs": refs,
        "scene.leaves": np.ascontiguousarray(scene.leaf_material, np.uint32),
        "looks.materials": mats,
        "lighting.lights": lights,
        "lighting.sky": sky,
        "shot.camera": cam,
        "geometry.region": region,
    }
    if finishes is not None:
        blocks["transport.finishes"] = finishes
    if "finish_boundary" in m and np.any((np.asarray(m["kind"]) == 3) & (np.asarray(m["finish_exact"]) == 0)):
        flat = np.ascontiguousarray(m["finish_boundary"], np.float64)
        boundaries = np.zeros(len(flat), BOUNDARY_DTYPE)
        boundaries["rarer"] = flat[:, :544].reshape(-1, 17, 32)
        boundaries["denser"] = flat[:, 544:1088].reshape(-1, 17, 32)
        boundaries["rarer_average"] = flat[:, 1088:1105]
        boundaries["denser_average"] = flat[:, 1105:1122]
        boundaries["rarer_through"] = flat[:, 1122:1139]
        blocks["transport.boundaries"] = boundaries
    pat = scene.patterns
    if pat and np.any(np.asarray(m["patterned"]) != 0):
        count = np.diff(pat["first"])
        patterns = np.zeros(len(count), PATTERN_DTYPE)
        patterns["first"] = pat["first"][:-1]
        patterns["count"] = count
        patterns["result"] = pat["result"]
        patterns["argument_first"] = pat["argument_first"][:-1]
        patterns["argument_count"] = np.diff(pat["argument_first"])
        patterns["stop_first"] = pat["stop_first"][:-1]
        patterns["stop_count"] = np.diff(pat["stop_first"])
        patterns["world"] = pat["world"]
        blocks["looks.patterns"] = patterns
        blocks["looks.pattern_steps"] = np.ascontiguousarray(pat["steps"])
        blocks["looks.pattern_arguments"] = np.ascontiguousarray(pat["arguments"], np.float64)
        blocks["looks.stops"] = np.ascontiguousarray(pat["stops"], np.float32).reshape(-1)
        if scene.leaf_placement is not None:
            placements = np.zeros(len(scene.leaf_placement), PLACEMENT_DTYPE)
            placements["linear"] = scene.leaf_placement[:, :9].reshape(-1, 3, 3)
            placements["origin"] = scene.leaf_placement[:, 9:]
            blocks["looks.placements"] = placements
    return blocks


class Backend:
    """One kdn context on one CUDA device."""

    def __init__(self, device: int = 0):
        self.lib = library()
        self.handle = ctypes.c_void_p()
        st = self.lib.kdn_open(device, ctypes.byref(self.handle))
        if st != KDN_OK:
            raise KdnError(st, self.lib.kdn_last_error(None).decode())
        self.scene: Scene | None = None

    def _check(self, st: int) -> None:
        if st != KDN_OK:
            raise KdnError(st, self.lib.kdn_last_error(self.handle).decode())

    def close(self) -> None:
        if self.handle:
            self.lib.kdn_close(self.handle)
            self.handle = ctypes.c_void_p()

    def __enter__(self) -> "Backend":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, name: str, array: np.ndarray) -> None:
        a = np.ascontiguousarray(array)
        self._check(self.lib.kdn_upload_block(self.handle, name.encode(), _ptr(a), a.shape[0], a.dtype.itemsize))

    def load(self, scene: Scene) -> None:
        for name, arr in scene_blocks(scene).items():
            self.upload(name, arr)
        self.scene = scene

    def build(self, min_depth: int = 6, max_depth: int = 10, split_steps: int = 96) -> None:
        o = BuildOptions(min_depth, max_depth, split_steps, 0)
        self._check(self.lib.kdn_build(self.handle, ctypes.byref(o)))

    def world_stats(self) -> dict:
        out = np.zeros(4, np.uint64)
        self._check(self.lib.kdn_world_stats(self.handle, _ptr(out)))
        return dict(cells=int(out[0]), leaves=int(out[1]), programs=int(out[2]), steps=int(out[3]))

    def world_cell(self, i: int):
        """(level, place, occupancy, [(object, result, steps)]) of cell i in
        depth-first pre-order, the programs in the reference's Step form."""
        head = np.zeros(6, np.uint32)
        self._check(self.lib.kdn_world_cell(self.handle, i, _ptr(head), None, None, None, None, 0))
        n = int(head[5])
        objects = np.zeros(max(n, 1), np.uint32)
        results = np.zeros(max(n, 1), np.uint32)
        counts = np.zeros(max(n, 1), np.uint32)
        self._check(self.lib.kdn_world_cell(self.handle, i, _ptr(head), _ptr(objects), _ptr(results), _ptr(counts), None, 0))
        steps = np.zeros(max(int(counts[:n].sum()), 1), STEP_DTYPE)
        self._check(self.lib.kdn_world_cell(self.handle, i, _ptr(head), _ptr(objects), _ptr(results), _ptr(counts), _ptr(steps), steps.shape[0]))
        progs, off = [], 0
        for k in range(n):
            c = int(counts[k])
            progs.append((int(objects[k]), int(results[k]), steps[off:off + c]))
            off += c
        return int(head[0]), (int(head[1]), int(head[2]), int(head[3])), int(head[4]), progs

    def extend(self, rays: np.ndarray) -> np.ndarray:
        """ExtendRays over host arrays (core/step.cpp:132)."""
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        hits = np.zeros(r.shape[0], HIT_DTYPE)
        self._check(self.lib.kdn_extend(self.handle, _ptr(r), r.shape[0], _ptr(hits)))
        return hits

    def set_guide(self, guide, share: float = 0.5, flags: int = 3) -> None:
        """Frames draw with the learned guide (GUIDE_SAMPLE, once trained)
        and train it on their paths (GUIDE_TRAIN); None: plain frames."""
        h = guide.handle if guide is not None else None
        self._check(self.lib.kdn_set_guide(self.handle, h, share, flags if guide is not None else 0))

    def guide_select(self, width: int, height: int, samples: int, surfaces: int | None = None, seed: int = 1):
        """Pilot frames decide whether the attached guide's sampling stays on
        (kdn_guide_select): returns (guided, plain cost, guided cost)."""
        sc = self.scene
        f = Frame(width, height, samples, surfaces if surfaces is not None else int(sc.render["surfaces"]), seed, 0, 0, 0, 0, 0,
                  int(sc.render.get("collisions", 0)))
        g, pc, gc = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.kdn_guide_select(self.handle, ctypes.byref(f), ctypes.byref(g), ctypes.byref(pc), ctypes.byref(gc)))
        return bool(g.value), pc.value, gc.value

    def render(self, width: int, height: int, samples: int, surfaces: int | None = None, seed: int | None = None,
               first: int = 0, accumulate: bool = False, denoise: bool = False, restart: bool = False, factor: int = 1,
               phase: int = 0, temporal_only: bool = False, upsample: bool = False, sobol: bool = False,
               sky_map: bool = False, each_lamp_first: bool = False) -> np.ndarray:
        """Draw `samples` samples a pixel and return the pixel means
        (linear RGB, float32, height x width x 3), or with `denoise` the
        means through the reconstruction chain (temporal + a-trous, or the
        temporal member alone with `temporal_only`; at a film `factor` of 2
        to 4 the frame is drawn at 1/factor of the size, aimed at `phase`,
        and the chain ends in the upscale member, or in the upsample member
        with `upsample`, which without `denoise` blows up the means).
        `sobol`: the first 28 dimensions of the draws from the scrambled
        Sobol sequence (--use sampler=sobol); `sky_map`: the sky aimed at by
        its chart (--use sampler=sky_map); `each_lamp_first`: the first four
        lamps' own lines at the first vertex (--use sampler=each_lamp_first)."""
        sc = self.scene
        f = Frame(width, height, samples, surfaces if surfaces is not None else int(sc.render["surfaces"]),
                  seed if seed is not None else int(sc.render["seed"]), first, 1 if accumulate else 0,
                  (FRAME_DENOISE if denoise else 0) | (FRAME_RESTART if restart else 0) | (FRAME_TEMPORAL if temporal_only else 0) |
                  (FRAME_UPSAMPLE if upsample else 0) | (FRAME_SOBOL if sobol else 0) | (FRAME_SKY_MAP if sky_map else 0) |
                  (FRAME_EACH_LAMP if each_lamp_first else 0), factor, phase, int(sc.render.get("collisions", 0)),
                  int(sc.render.get("split", 1)))
        out = np.zeros((height, width, 3), np.float32)
        self._check(self.lib.kdn_render(self.handle, ctypes.byref(f), _ptr(out)))
        return out

    def share(self, priority: int = 0) -> "Backend":
        """A context drawing this one's world (include/kdn.h kdn_open_sharing);
        close it before this one."""
        b = Backend.__new__(Backend)
        b.lib = self.lib
        b.handle = ctypes.c_void_p()
        self._check(self.lib.kdn_open_sharing(self.handle, priority, ctypes.byref(b.handle)))
        b.scene = self.scene
        return b

    def set_frame_budget(self, nbytes: int) -> None:
        self._check(self.lib.kdn_set_frame_budget(self.handle, nbytes))

    def set_march_budget(self, steps: int) -> None:
        """March steps a ray may take in one trace launch of this context's
        frames before it goes on in the next (kdn_set_march_budget; 0: none).
        Frames are the same to the bit with any budget."""
        self._check(self.lib.kdn_set_march_budget(self.handle, steps))

    def frame_stats(self) -> FrameStats:
        s = FrameStats()
        self._check(self.lib.kdn_frame_stats_get(self.handle, ctypes.byref(s)))
        return s

    def world_march(self, i: int, points: np.ndarray) -> np.ndarray:
        """The march form of cell i's kept programs run on the host at the
        points (n x 3): programs x n float32 (include/kdn.h kdn_world_march)."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        count = ctypes.c_uint32()
        cap = 64 * max(pts.shape[0], 1)  # a leaf keeps at most 64 programs
        values = np.zeros(cap, np.float32)
        self._check(self.lib.kdn_world_march(self.handle, i, _ptr(pts), pts.shape[0], _ptr(values), cap, ctypes.byref(count)))
        return values[: count.value * pts.shape[0]].reshape(count.value, pts.shape[0])

    def world_locate(self, points: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """The leaf of each point by the trace kernel's grid locate and by the
        descent from the root, on the host (include/kdn.h kdn_world_locate)."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        a = np.zeros(len(pts), np.uint32)
        b = np.zeros(len(pts), np.uint32)
        self._check(self.lib.kdn_world_locate(self.handle, _ptr(pts), len(pts), _ptr(a), _ptr(b)))
        return a, b

    def frame_record(self, width: int, height: int) -> dict:
        """The record of the last frame drawn with denoise=True: each pixel's
        light of that call and the first surface of its last sample
        (include/kdn.h kdn_frame_record); FP16 fields as float16 arrays."""
        light = np.zeros((height, width, 3), np.float32)
        distance = np.zeros((height, width), np.float16)
        normal = np.zeros((height, width, 3), np.float16)
        albedo = np.zeros((height, width, 3), np.float16)
        leaf = np.zeros((height, width), np.uint32)
        self._check(self.lib.kdn_frame_record(self.handle, _ptr(light), _ptr(distance), _ptr(normal), _ptr(albedo), _ptr(leaf)))
        return {"light": light, "distance": distance, "normal": normal, "albedo": albedo, "leaf": leaf}

    def frame_surfaces(self, width: int, height: int) -> dict:
        """The first surfaces of the last frame drawn with denoise=True
        (include/kdn.h kdn_frame_surfaces); FP16 fields as float16 arrays."""
        distance = np.zeros((height, width), np.float16)
        normal = np.zeros((height, width, 3), np.float16)
        albedo = np.zeros((height, width, 3), np.float16)
        leaf = np.zeros((height, width), np.uint32)
        self._check(self.lib.kdn_frame_surfaces(self.handle, _ptr(distance), _ptr(normal), _ptr(albedo), _ptr(leaf)))
        return {"distance": distance, "normal": normal, "albedo": albedo, "leaf": leaf}

    def flush_l2(self) -> None:
        self._check(self.lib.kdn_flush_l2(self.handle))

    def denoise(self, width: int, height: int, demodulated: bool, lens, colour, moment, length, distance, normal, albedo, leaf) -> np.ndarray:
        """The a-trous denoiser over host feature buffers (include/kdn.h
        kdn_denoise).  lens: eye, forward, right, up (3 each), reach,
        aspect.  distance, normal and albedo are stored as FP16."""
        f = DenoiseFrame(width, height, 1 if demodulated else 0, 0)
        lens = np.asarray(lens, np.float64)
        for k in range(3):
            f.eye[k], f.forward[k], f.right[k], f.up[k] = lens[k], lens[3 + k], lens[6 + k], lens[9 + k]
        f.reach, f.aspect = float(lens[12]), float(lens[13])
        arrs = [np.ascontiguousarray(colour, np.float32), np.ascontiguousarray(moment, np.float32), np.ascontiguousarray(length, np.float32),
                np.ascontiguousarray(distance, np.float16), np.ascontiguousarray(normal, np.float16), np.ascontiguousarray(albedo, np.float16),
                np.ascontiguousarray(leaf, np.uint32)]
        out = np.zeros((width * height, 3), np.float32)
        self._check(self.lib.kdn_denoise(self.handle, ctypes.byref(f), *[_ptr(a) for a in arrs], _ptr(out)))
        return out


class Server:
    """The serving loop (include/kdn.h kdn_serve_*): resident scenes,
    requests submitted as they arrive and drawn side by side, progressive
    sessions, latency percentiles."""

    def __init__(self, device: int = 0, slots: int = 4, budget_bytes: int = 0, batch_slots: int = 0, batch_sm_percent: int = 0,
                 batch_frame_bytes: int = 0):
        self.lib = library()
        self.handle = ctypes.c_void_p()
        o = ServeOptions(device, slots, budget_bytes, batch_slots, batch_sm_percent, batch_frame_bytes)
        st = self.lib.kdn_serve_open(ctypes.byref(o), ctypes.byref(self.handle))
        if st != KDN_OK:
            raise KdnError(st, "kdn_serve_open")
        self.outputs: dict[int, np.ndarray] = {}
        self.scenes: list[Backend] = []

    def _check(self, st: int) -> None:
        if st != KDN_OK:
            raise KdnError(st, self.lib.kdn_serve_last_error(self.handle).decode())

    def add_scene(self, backend: "Backend") -> int:
        """Register a built scene (the Backend stays open until the server closes)."""
        sid = ctypes.c_uint32()
        self._check(self.lib.kdn_serve_add_scene(self.handle, backend.handle, ctypes.byref(sid)))
        self.scenes.append(backend)
        return int(sid.value)

    def submit(self, scene: int, width: int, height: int, samples: int, surfaces: int = 8, seed: int = 1, denoise: bool = False,
               interactive: bool = False, session: int = 0) -> int:
        r = Request(scene, width, height, samples, surfaces, seed, (FRAME_DENOISE if denoise else 0) | (REQUEST_INTERACTIVE if interactive else 0), 0, session)
        out = np.zeros((height, width, 3), np.float32)
        ticket = ctypes.c_uint64()
        self._check(self.lib.kdn_serve_submit(self.handle, ctypes.byref(r), _ptr(out), ctypes.byref(ticket)))
        self.outputs[int(ticket.value)] = out
        return int(ticket.value)

    def wait(self, ticket: int) -> tuple[int, dict, np.ndarray]:
        """(status, {frame, queued_ms, render_ms, latency_ms}, image)."""
        served = Served()
        self.lib.kdn_serve_wait(self.handle, ticket, ctypes.byref(served))
        out = self.outputs.pop(ticket)
        return int(served.status), {"frame": int(served.frame), "queued_ms": served.queued_ms, "render_ms": served.render_ms,
                                    "latency_ms": served.latency_ms}, out

    def end_session(self, session: int) -> None:
        self._check(self.lib.kdn_serve_end_session(self.handle, session))

    def reset_latency(self) -> None:
        self._check(self.lib.kdn_serve_reset_latency(self.handle))

    def cancel_queued(self) -> int:
        n = ctypes.c_uint64()
        self._check(self.lib.kdn_serve_cancel_queued(self.handle, ctypes.byref(n)))
        return int(n.value)

    def latency(self, interactive_only: bool = False) -> dict:
        p50, p99, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()
        self._check(self.lib.kdn_serve_latency(self.handle, 1 if interactive_only else 0, ctypes.byref(p50), ctypes.byref(p99), ctypes.byref(n)))
        return {"p50_ms": p50.value, "p99_ms": p99.value, "count": int(n.value)}

    def close(self) -> None:
        if self.handle:
            self.lib.kdn_serve_close(self.handle)
            self.handle = ctypes.c_void_p()

    def __enter__(self) -> "Server":
        return self

    def __exit__(self, *exc) -> None:
        self.close()


GUIDE_SAMPLE = 1
GUIDE_TRAIN = 2


class GuideOptions(ctypes.Structure):
    _fields_ = [("table_log2", ctypes.c_uint32), ("seed", ctypes.c_uint32), ("learning_rate", ctypes.c_float),
                ("region_lo", ctypes.c_float * 3), ("region_hi", ctypes.c_float * 3), ("batch", ctypes.c_uint32),
                ("max_steps", ctypes.c_uint32), ("sample_capacity", ctypes.c_uint32)]


class Guide:
    """The learned guide (kdn_guide_*): a hash-grid encoding and a 3 x 64
    network whose outputs are eight vMF lobes, trained and queried on the
    device's tensor cores."""

    def __init__(self, device: int = 0, table_log2: int = 19, seed: int = 1, learning_rate: float = 1e-2,
                 region=((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)), batch: int = 0, max_steps: int = 0, sample_capacity: int = 0):
        self.lib = library()
        o = GuideOptions()
        o.table_log2, o.seed, o.learning_rate = table_log2, seed, learning_rate
        for k in range(3):
            o.region_lo[k], o.region_hi[k] = float(region[0][k]), float(region[1][k])
        o.batch, o.max_steps, o.sample_capacity = batch, max_steps, sample_capacity
        self.options = o
        self.handle = ctypes.c_void_p()
        self._check(self.lib.kdn_guide_open(device, ctypes.byref(o), ctypes.byref(self.handle)))
        w, t = ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self.lib.kdn_guide_sizes(self.handle, ctypes.byref(w), ctypes.byref(t)))
        self.weight_count, self.table_count = w.value, t.value
        self.table_log2 = table_log2

    def _check(self, status: int) -> None:
        if status != KDN_OK:
            raise KdnError(status, self.lib.kdn_guide_last_error().decode())

    def close(self) -> None:
        if self.handle:
            self.lib.kdn_guide_close(self.handle)
            self.handle = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def params(self):
        w = np.zeros(self.weight_count, np.float32)
        t = np.zeros(self.table_count, np.float32)
        self._check(self.lib.kdn_guide_get_params(self.handle, _ptr(w), _ptr(t)))
        return w, t

    def set_params(self, w: np.ndarray, t: np.ndarray) -> None:
        w = np.ascontiguousarray(w, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        self._check(self.lib.kdn_guide_set_params(self.handle, _ptr(w), _ptr(t)))

    def gradients(self, samples: np.ndarray):
        s = np.ascontiguousarray(samples, np.float32)
        loss = np.zeros(1, np.float32)
        dw = np.zeros(self.weight_count, np.float32)
        dt = np.zeros(self.table_count, np.float32)
        self._check(self.lib.kdn_guide_gradients(self.handle, _ptr(s), len(s), _ptr(loss), _ptr(dw), _ptr(dt)))
        return float(loss[0]), dw, dt

    def train(self, samples: np.ndarray, batch: int = 16384, steps: int = 0) -> float:
        s = np.ascontiguousarray(samples, np.float32)
        loss = np.zeros(1, np.float32)
        self._check(self.lib.kdn_guide_train(self.handle, _ptr(s), len(s), batch, steps, _ptr(loss)))
        return float(loss[0])

    def query(self, rows: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(rows, np.float32)
        out = np.zeros((len(r), 40), np.float32)
        self._check(self.lib.kdn_guide_query(self.handle, _ptr(r), len(r), _ptr(out)))
        return out
