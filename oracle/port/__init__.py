"""ctypes view of the oracle's C library (kdn_port.h), built in-tree."""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_build")
LIB = os.path.join(OUT, "libkdn_oracle.so")
SOURCES = ["geometry.c", "spectral.c", "transport.c", "denoise.c", "temporal.c", "upscale.c"]

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (plain C, -ffp-contract=off as the
    reference is built) into oracle/_build/libkdn_oracle.so."""
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    newest = max(os.path.getmtime(s) for s in srcs + [os.path.join(HERE, "kdn_port.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fno-math-errno", "-D_GNU_SOURCE",
           "-o", LIB + ".tmp"] + srcs + ["-lm", "-lpthread"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class Step(ctypes.Structure):
    _fields_ = [("opcode", ctypes.c_uint8), ("a", ctypes.c_uint32), ("b", ctypes.c_uint32), ("c", ctypes.c_uint32),
                ("value", ctypes.c_double), ("leaf", ctypes.c_uint32)]


class Program(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_void_p), ("count", ctypes.c_uint32), ("result", ctypes.c_uint32)]


RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("direction", "<f4", 3), ("far", "<f4"), ("inside", "<u4"), ("within", "<u4")])
HIT_DTYPE = np.dtype([("kind", "<u4"), ("distance", "<f4"), ("point", "<f4", 3), ("normal", "<f4", 3), ("leaf", "<u4"),
                      ("other", "<u4"), ("share", "<f4"), ("object", "<u4"), ("steps", "<u4")])

_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.kp_octree_build.restype = _P
        L.kp_octree_build.argtypes = [_P, ctypes.c_uint32, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_uint32]
        L.kp_octree_free.argtypes = [_P]
        L.kp_octree_cells.restype = ctypes.c_uint64
        L.kp_octree_cells.argtypes = [_P]
        L.kp_octree_cell.restype = ctypes.c_uint32
        L.kp_octree_cell.argtypes = [_P, ctypes.c_uint64, _P]
        L.kp_octree_cell_program.argtypes = [_P, ctypes.c_uint64, ctypes.c_uint32, _P, ctypes.POINTER(Program)]
        L.kp_sphere_trace.argtypes = [_P, ctypes.c_uint32, _P, _P, _P, _P, ctypes.c_uint32, _P]
        L.kp_sphere_trace_rule.argtypes = [_P, ctypes.c_uint32, _P, _P, _P, _P, ctypes.c_uint32, _P, ctypes.c_int]
        L.kp_normal_at.argtypes = [_P, _P, ctypes.c_double, _P, _P]
        L.kp_octree_trace.argtypes = [_P, _P, _P, ctypes.c_uint32, _P]
        L.kp_mixed_bits.restype = ctypes.c_uint64
        L.kp_mixed_bits.argtypes = [ctypes.c_uint64]
        L.kp_hashed.restype = ctypes.c_double
        L.kp_hashed.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        L.kp_sampled_wavelengths.argtypes = [ctypes.c_double, _P, _P, _P]
        L.kp_wavelength_share.restype = ctypes.c_double
        L.kp_wavelength_share.argtypes = [ctypes.c_double, ctypes.c_uint32]
        L.kp_spectrum_of.argtypes = [_P, _P, _P]
        L.kp_colour_of.argtypes = [_P, _P, _P, _P]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class Programs:
    """The scene's object programs as a C array of kp_program, kept alive."""

    def __init__(self, scene):
        self.steps = np.ascontiguousarray(scene.steps)
        self.array = (Program * scene.program_count)()
        base = self.steps.ctypes.data
        for i in range(scene.program_count):
            self.array[i].steps = base + int(scene.program_first[i]) * 32
            self.array[i].count = int(scene.program_first[i + 1] - scene.program_first[i])
            self.array[i].result = int(scene.program_result[i])
        self.count = scene.program_count


def sphere_trace(scene, rays: np.ndarray, lower, size, rule: int = 0) -> np.ndarray:
    """sphere_trace.cpp:216 sphereTraced over the scene's object programs in
    double; rule 1 stops by the FP32 device march's tolerance instead of the
    reference's (kp_sphere_trace_rule)."""
    progs = Programs(scene)
    hits = np.zeros(len(rays), HIT_DTYPE)
    lo = np.asarray(lower, np.float64)
    sz = np.asarray(size, np.float64)
    mat = np.ascontiguousarray(scene.leaf_material, np.uint32)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    lib().kp_sphere_trace_rule(ctypes.addressof(progs.array), progs.count, _ptr(mat), _ptr(lo), _ptr(sz), _ptr(rays), len(rays), _ptr(hits), rule)
    return hits


def normal_at(scene, rays: np.ndarray, objects: np.ndarray, ts: np.ndarray):
    """sphereNormal of each ray's object program at p(t): (normals n x 3,
    gradient lengths n) in double (kp_normal_at)."""
    progs = Programs(scene)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    out = np.zeros((len(rays), 3), np.float64)
    grad = np.zeros(len(rays), np.float64)
    L = lib()
    base = ctypes.addressof(progs.array)
    size = ctypes.sizeof(Program)
    for i in range(len(rays)):
        L.kp_normal_at(base + size * int(objects[i]), rays[i:i + 1].ctypes.data, float(ts[i]), out[i].ctypes.data, grad[i:i + 1].ctypes.data)
    return out, grad


class Octree:
    """The oracle's cut octree over a scene (kp_octree_build)."""

    def __init__(self, scene, min_depth: int, max_depth: int, split_steps: int):
        self.progs = Programs(scene)
        self.scene = scene
        lo = np.asarray(scene.region_lower, np.float64)
        sz = np.asarray(scene.region_size, np.float64)
        self.handle = lib().kp_octree_build(ctypes.addressof(self.progs.array), self.progs.count, _ptr(lo), _ptr(sz),
                                            min_depth, max_depth, split_steps)

    def __del__(self):
        if getattr(self, "handle", None):
            lib().kp_octree_free(self.handle)
            self.handle = None

    def cells(self) -> int:
        return int(lib().kp_octree_cells(self.handle))

    def cell(self, i: int):
        """(level, place, occupancy, [(object, result, steps array)]) of cell i
        in depth-first pre-order."""
        head = np.zeros(5, np.uint32)
        n = lib().kp_octree_cell(self.handle, i, _ptr(head))
        progs = []
        for k in range(n):
            obj = ctypes.c_uint32()
            p = Program()
            lib().kp_octree_cell_program(self.handle, i, k, ctypes.byref(obj), ctypes.byref(p))
            from kodanuki_gb300.scene import STEP_DTYPE
            buf = (ctypes.c_char * (p.count * 32)).from_address(p.steps)
            steps = np.frombuffer(bytes(buf), STEP_DTYPE).copy()
            progs.append((obj.value, p.result, steps))
        return int(head[0]), tuple(int(x) for x in head[1:4]), int(head[4]), progs

    def trace(self, rays: np.ndarray) -> np.ndarray:
        hits = np.zeros(len(rays), HIT_DTYPE)
        mat = np.ascontiguousarray(self.scene.leaf_material, np.uint32)
        lib().kp_octree_trace(self.handle, _ptr(mat), _ptr(rays), len(rays), _ptr(hits))
        return hits


class Material(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("exact", ctypes.c_uint32), ("albedo", ctypes.c_double * 3), ("index", ctypes.c_double),
                ("dispersion", ctypes.c_double), ("width", ctypes.c_double), ("facet_share", ctypes.c_double), ("body", ctypes.c_double),
                ("coat_front", ctypes.c_double), ("coat_twice", ctypes.c_double), ("coat_room", ctypes.c_double),
                ("escape_average", ctypes.c_double), ("escape", ctypes.c_double * 32), ("glow", ctypes.c_double * 3),
                ("absorb", ctypes.c_double * 3), ("pattern", Program), ("pattern_arguments", ctypes.c_void_p),
                ("stops", ctypes.c_void_p), ("stop_count", ctypes.c_uint32), ("world", ctypes.c_uint32),
                ("loses_much", ctypes.c_uint32), ("boundary", ctypes.c_void_p), ("film", ctypes.c_double * 2),
                ("scatter", ctypes.c_double), ("lean", ctypes.c_double)]


def _materials(scene):
    """The scene's materials as a C array of kp_material, with the arrays
    their patterns point into (kept alive by the caller)."""
    m = scene.materials
    n = len(m["kind"])
    mats = (Material * n)()
    keep = []
    pat = scene.patterns
    for i in range(n):
        mats[i].kind = int(m["kind"][i])
        mats[i].exact = int(m["finish_exact"][i]) if "finish_exact" in m else 0
        for c in range(3):
            mats[i].albedo[c] = float(m["albedo"][i][c])
            # material.cpp:325 glowOf: glow x double(strength)
            mats[i].glow[c] = float(m["glow"][i][c]) * float(np.float32(m["strength"][i])) if "glow" in m else 0.0
            mats[i].absorb[c] = float(m["absorb"][i][c]) if "absorb" in m else 0.0
        mats[i].index = float(m["finish_index"][i]) if "finish_index" in m else 1.0
        mats[i].dispersion = float(m["dispersion"][i]) if int(m["kind"][i]) == 3 else 0.0
        if "scatter" in m and int(m["kind"][i]) == 3:
            mats[i].scatter = float(m["scatter"][i])
            mats[i].lean = float(m["lean"][i])
        if "finish_width" in m:
            mats[i].width = float(m["finish_width"][i])
            mats[i].facet_share = float(m["finish_facet_share"][i])
            mats[i].body = float(m["finish_body"][i])
            mats[i].coat_front, mats[i].coat_twice, mats[i].coat_room = (float(x) for x in m["finish_coating"][i])
            mats[i].escape_average = float(m["finish_escape_average"][i])
            for k in range(32):
                mats[i].escape[k] = float(m["finish_escape"][i][k])
        if "finish_film" in m and int(m["kind"][i]) != 0:
            # material.cpp:106 filmOf: thickness (nm, 0 for none) and index
            mats[i].film[0], mats[i].film[1] = (float(x) for x in m["finish_film"][i])
        if "finish_boundary" in m and int(m["kind"][i]) == 3:
            boundary = np.ascontiguousarray(m["finish_boundary"][i], np.float64)
            keep.append(boundary)
            mats[i].boundary = boundary.ctypes.data
            mats[i].loses_much = int(m["finish_loses_much"][i])
        if pat and int(pat["first"][i + 1]) > int(pat["first"][i]):
            steps = np.ascontiguousarray(pat["steps"][pat["first"][i]:pat["first"][i + 1]])
            args = np.ascontiguousarray(pat["arguments"][pat["argument_first"][i]:pat["argument_first"][i + 1]], np.float64)
            stops = np.ascontiguousarray(pat["stops"][pat["stop_first"][i]:pat["stop_first"][i + 1]], np.float64)
            keep += [steps, args, stops]
            mats[i].pattern.steps = steps.ctypes.data
            mats[i].pattern.count = len(steps)
            mats[i].pattern.result = int(pat["result"][i])
            mats[i].pattern_arguments = args.ctypes.data if len(args) else None
            mats[i].stops = stops.ctypes.data
            mats[i].stop_count = len(stops)
            mats[i].world = int(pat["world"][i])
    return mats, keep


def _placements(scene):
    if scene.leaf_placement is None:
        return None
    return np.ascontiguousarray(scene.leaf_placement, np.float64)


class Lamp(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("square", ctypes.c_uint32), ("at", ctypes.c_double * 3), ("along", ctypes.c_double * 3),
                ("across", ctypes.c_double * 3), ("power", ctypes.c_double * 3), ("radius", ctypes.c_double),
                ("direction", ctypes.c_double * 3), ("angle", ctypes.c_double)]


class View(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_double * 3), ("target", ctypes.c_double * 3), ("up", ctypes.c_double * 3), ("fov", ctypes.c_double),
                ("zenith", ctypes.c_double * 3), ("horizon", ctypes.c_double * 3), ("ground", ctypes.c_double * 3),
                ("width", ctypes.c_int32), ("height", ctypes.c_int32), ("spp", ctypes.c_int32), ("surfaces", ctypes.c_int32),
                ("seed", ctypes.c_int32), ("lamp_count", ctypes.c_uint32), ("material_count", ctypes.c_uint32),
                ("factor", ctypes.c_uint32), ("phase", ctypes.c_uint32), ("sobol", ctypes.c_uint32), ("sky_map", ctypes.c_uint32),
                ("each_lamp", ctypes.c_uint32), ("middle", ctypes.c_double * 3), ("collisions", ctypes.c_int32),
                ("sky_kind", ctypes.c_uint32), ("haze", ctypes.c_double), ("glow", ctypes.c_double * 3), ("strength", ctypes.c_double),
                ("spread", ctypes.c_double), ("aperture", ctypes.c_double), ("focus", ctypes.c_double), ("split", ctypes.c_uint32),
                ("stars", ctypes.c_uint32), ("star_count", ctypes.c_double), ("star_strength", ctypes.c_double), ("star_angle", ctypes.c_double)]


_trees: dict = {}


def _octree_for(scene, build: dict) -> "Octree":
    key = (id(scene), build["min_depth"], build["max_depth"], build["split_steps"])
    if key not in _trees:
        _trees[key] = Octree(scene, build["min_depth"], build["max_depth"], build["split_steps"])
    return _trees[key]


def render_band(scene, width: int, height: int, spp: int, surfaces: int, seed: int, row0: int, rows: int, threads: int,
                build: dict | None = None, factor: int = 1, phase: int = 0, sobol: bool = False, sky_map: bool = False,
                each_lamp_first: bool = False) -> np.ndarray:
    """The oracle renderer over rows [row0, row0 + rows) of a frame: summed
    RGB per pixel (rows x width x 3, divide by spp for the means).  With a
    film factor above 1, width x height is the drawn frame and each pixel's
    samples aim at the shown pixel of `phase`.  `sobol`: --use sampler=sobol;
    `sky_map`: --use sampler=sky_map; `each_lamp_first`: --use
    sampler=each_lamp_first."""
    build = build or dict(min_depth=6, max_depth=10, split_steps=96)
    tree = _octree_for(scene, build)
    mats, keep = _materials(scene)
    n = len(mats)
    l = scene.lights
    nl = len(l["kind"])
    lamps = (Lamp * max(nl, 1))()
    for i in range(nl):
        lamps[i].kind = int(l["kind"][i])
        for c in range(3):
            lamps[i].at[c] = float(l["at"][i][c])
            lamps[i].along[c] = float(l["along"][i][c])
            lamps[i].across[c] = float(l["across"][i][c])
            lamps[i].power[c] = float(l["power"][i][c])
        lamps[i].radius = float(l["radius"][i])
        for c in range(3):
            lamps[i].direction[c] = float(l["direction"][i][c])
        lamps[i].angle = float(l["angle"][i])
    v = View()
    for c in range(3):
        v.eye[c] = scene.camera["eye"][c]
        v.target[c] = scene.camera["target"][c]
        v.up[c] = scene.camera["up"][c]
        v.zenith[c] = scene.sky["zenith"][c]
        v.horizon[c] = scene.sky["horizon"][c]
        v.ground[c] = scene.sky["ground"][c]
    v.fov = scene.camera["fov"]
    v.width, v.height, v.spp, v.surfaces, v.seed = width, height, spp, surfaces, seed
    v.lamp_count, v.material_count = nl, n
    v.factor, v.phase, v.sobol, v.sky_map, v.each_lamp = factor, phase, int(sobol), int(sky_map), int(each_lamp_first)
    v.collisions = int(scene.render.get("collisions", 0)) or 256
    v.sky_kind = int(scene.sky.get("kind", 0))
    v.aperture = float(np.float32(scene.camera.get("aperture", 0)))
    v.split = max(int(scene.render.get("split", 1)), 1)
    v.stars = int(scene.sky.get("stars", 0))
    v.star_count = float(np.float32(scene.sky.get("star_count", 0)))
    v.star_strength = float(np.float32(scene.sky.get("star_strength", 0)))
    v.star_angle = float(np.float32(scene.sky.get("star_angle", 0)))
    v.focus = float(np.float32(scene.camera.get("focus", 0)))
    v.haze = float(np.float32(scene.sky.get("haze", 0)))
    v.strength = float(np.float32(scene.sky.get("strength", 0)))
    v.spread = float(np.float32(scene.sky.get("spread", 0)))
    for c in range(3):
        v.glow[c] = float(scene.sky.get("glow", [0, 0, 0])[c])
    lower = np.asarray(scene.region_lower, np.float64)
    size = np.asarray(scene.region_size, np.float64)
    for a in range(3):
        v.middle[a] = lower[a] + 0.5 * size[a]
    sums = np.zeros((rows, width, 3), np.float64)
    mat_leaf = np.ascontiguousarray(scene.leaf_material, np.uint32)
    L = lib()
    placements = _placements(scene)
    L.kp_render_band.argtypes = [_P, _P, _P, _P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]
    L.kp_render_band(tree.handle, _ptr(mat_leaf), ctypes.addressof(mats), ctypes.addressof(lamps), ctypes.byref(v),
                     _ptr(placements) if placements is not None else None, row0, rows, threads, _ptr(sums))
    del keep
    return sums


def lens_of(scene, width: int, height: int) -> np.ndarray:
    """core/camera.cpp:9 lensOf: eye, forward, right, up (3 each), reach,
    aspect, in double."""
    cam = scene.camera
    eye = np.asarray(cam["eye"], np.float64)
    forward = np.asarray(cam["target"], np.float64) - eye
    forward /= np.sqrt(forward @ forward)
    right = np.cross(forward, np.asarray(cam["up"], np.float64))
    right /= np.sqrt(right @ right)
    up = np.cross(right, forward)
    return np.concatenate([eye, forward, right, up, [np.tan(float(cam["fov"]) / 2), width / height]])


def traced_surfaces(scene, width: int, height: int, build: dict | None = None, lens=None, offsets=None) -> dict:
    """core/surfaces.cpp:133 tracedSurfaces: one ray through each pixel's
    centre (core/camera.cpp:34 filmDirection), the first surface's distance
    from the eye, normal facing the ray, albedo (mixed across a blend seam,
    material.cpp:345 bsdfAt) and leaf; a missed ray keeps batch.cpp:46
    missedSurface.  Pixel-major arrays of width * height.  `lens` (14
    doubles) replaces the scene's camera, `offsets` (n x 2, in [0, 1)) the
    pixel centres."""
    build = build or dict(min_depth=6, max_depth=10, split_steps=96)
    tree = _octree_for(scene, build)
    lens = lens_of(scene, width, height) if lens is None else np.asarray(lens, np.float64)
    eye, forward, right, up, reach, aspect = lens[0:3], lens[3:6], lens[6:9], lens[9:12], lens[12], lens[13]
    y, x = np.mgrid[0:height, 0:width]
    off = np.full((width * height, 2), 0.5) if offsets is None else np.asarray(offsets, np.float64)
    u = 2 * (x.ravel() + off[:, 0]) / width - 1
    v = 1 - 2 * (y.ravel() + off[:, 1]) / height
    heading = forward[None, :] + right[None, :] * (u * reach * aspect)[:, None] + up[None, :] * (v * reach)[:, None]
    heading /= np.sqrt((heading * heading).sum(1))[:, None]
    rays = np.zeros(width * height, RAY_DTYPE)
    rays["origin"] = eye.astype(np.float32)
    rays["direction"] = heading.astype(np.float32)
    rays["far"] = np.inf
    rays["inside"] = 0
    rays["within"] = 0xFFFFFFFF
    hits = tree.trace(rays)
    found = hits["kind"] != 0
    normal = hits["normal"].astype(np.float64)
    facing = (normal * rays["direction"].astype(np.float64)).sum(1) >= 0
    normal[facing] *= -1
    normal[~found] = 0
    albedo = albedos(scene, hits["leaf"], hits["other"], hits["share"], hits["point"], normal)
    albedo[~found] = 0
    delta = hits["point"].astype(np.float32) - rays["origin"]
    distance = np.sqrt((delta * delta).sum(1, dtype=np.float32)).astype(np.float32)
    distance[~found] = np.inf
    leaf = np.where(found, hits["leaf"], 0xFFFFFFFF).astype(np.uint32)
    return {"distance": distance, "normal": normal, "albedo": albedo, "leaf": leaf}


def albedos(scene, leaf, other, share, point, normal) -> np.ndarray:
    """material.cpp:345 bsdfAt's albedo at n hits (the normal facing the
    ray): the material's colour or its ramp over its pattern program, mixed
    across a blend seam (n x 3, double)."""
    mats, keep = _materials(scene)
    placements = _placements(scene)
    leaf_material = np.ascontiguousarray(scene.leaf_material, np.uint32)
    leaf = np.ascontiguousarray(leaf, np.uint32)
    other = np.ascontiguousarray(other, np.uint32)
    share = np.ascontiguousarray(share, np.float32)
    point = np.ascontiguousarray(point, np.float64)
    normal = np.ascontiguousarray(normal, np.float64)
    out = np.zeros((len(leaf), 3), np.float64)
    L = lib()
    L.kp_albedos.argtypes = [_P, ctypes.c_uint32, _P, ctypes.c_uint32, _P, ctypes.c_uint32, _P, _P, _P, _P, _P, _P]
    L.kp_albedos(ctypes.addressof(mats), len(mats), _ptr(leaf_material), len(leaf_material), _ptr(placements) if placements is not None else None,
                 len(leaf), _ptr(leaf), _ptr(other), _ptr(share), _ptr(point), _ptr(normal), _ptr(out))
    del keep
    return out


def upscale(width: int, height: int, factor: int, phase: int, moved: bool, kept: bool, settling: bool, lens_now, lens_before, internal,
            distance=None, before_colour=None, before_depth=None):
    """The oracle's upscale member over one frame (kp_upscale): the drawn
    frame `internal` (drawn size x 3) to the shown size, with the G-buffer's
    distances at the drawn size (or none: every sample sky) and the state
    before (shown size; read when kept).  Returns the state after (colour n
    x 3 double, depth n float) and the image (n x 3 float)."""
    L = lib()
    L.kp_upscale.argtypes = [ctypes.c_int] * 7 + [_P] * 9
    n = width * height
    internal = np.ascontiguousarray(internal, np.float32)
    dist = None if distance is None else np.ascontiguousarray(distance, np.float32)
    bc = np.zeros((n, 3)) if before_colour is None else np.ascontiguousarray(before_colour, np.float64)
    bd = np.zeros(n, np.float32) if before_depth is None else np.ascontiguousarray(before_depth, np.float32)
    colour = np.zeros((n, 3))
    depth = np.zeros(n, np.float32)
    image = np.zeros((n, 3), np.float32)
    ln = np.ascontiguousarray(lens_now, np.float64)
    lb = np.ascontiguousarray(lens_before, np.float64)
    L.kp_upscale(width, height, factor, phase, int(moved), int(kept), int(settling), _ptr(ln), _ptr(lb), _ptr(internal),
                 _ptr(dist) if dist is not None else None, _ptr(bc), _ptr(bd), _ptr(colour), _ptr(depth), _ptr(image))
    return colour, depth, image


def sobol_numbers(stream, index, dimension) -> np.ndarray:
    """plugins/sampler/sobol/sobol.cpp sobolNumber of (stream, index,
    dimension) triples (arrays; dimensions below 28)."""
    L = lib()
    L.kp_sobol_tables.argtypes = [_P]
    L.kp_sobol_number.argtypes = [_P, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32]
    L.kp_sobol_number.restype = ctypes.c_double
    tables = np.zeros(28 * 512, np.uint32)
    L.kp_sobol_tables(_ptr(tables))
    return np.array([L.kp_sobol_number(_ptr(tables), int(s), int(i), int(d)) for s, i, d in zip(stream, index, dimension)])


def upsample(width: int, height: int, factor: int, drawn) -> np.ndarray:
    """The oracle's upsample member (kp_upsample): the drawn frame (drawn
    size x 3) bilinearly to width x height (n x 3 float)."""
    L = lib()
    L.kp_upsample.argtypes = [ctypes.c_int] * 3 + [_P] * 2
    drawn = np.ascontiguousarray(drawn, np.float32)
    shown = np.zeros((width * height, 3), np.float32)
    L.kp_upsample(width, height, factor, _ptr(drawn), _ptr(shown))
    return shown


def upscale_settling(kept: bool, moved: bool, before_moved: bool, before_settling: int) -> tuple[bool, int]:
    """upscale.cpp:557 settlingFrames and the count the state keeps: whether
    this frame settles (blends at alpha 1) and the count after."""
    settling = (0 if moved else (4 if before_moved else before_settling)) if kept else 0
    return settling > 0, max(settling - 1, 0)


def bsdf_answers(scene, ids, records) -> dict:
    """material.cpp:1076 respondBsdf and :1366 sampleBsdf at n vertices of
    the scene's materials: ids (n x 2 uint32: material, medium or
    0xFFFFFFFF), records (n x 17 double: albedo[3], normal[3], outgoing[3],
    incoming[3], wavelength share, draw numbers u, v, lobe, side)."""
    mats, keep = _materials(scene)
    ids = np.ascontiguousarray(ids, np.uint32).reshape(-1, 2)
    records = np.ascontiguousarray(records, np.float64).reshape(-1, 17)
    n = len(ids)
    out = {"value": np.zeros((n, 4)), "density": np.zeros(n), "seen": np.zeros((n, 2), np.uint32), "incoming": np.zeros((n, 3)),
           "weight": np.zeros((n, 4)), "drawn_density": np.zeros(n)}
    L = lib()
    L.kp_bsdf_answers.argtypes = [_P, ctypes.c_uint32, ctypes.c_uint32] + [_P] * 8
    L.kp_bsdf_answers(ctypes.addressof(mats), len(mats), n, _ptr(ids), _ptr(records), _ptr(out["value"]), _ptr(out["density"]), _ptr(out["seen"]),
                      _ptr(out["incoming"]), _ptr(out["weight"]), _ptr(out["drawn_density"]))
    del keep
    return out


def denoise(width: int, height: int, demodulated: int, lens, colour, moment, length, distance, normal, leaf, albedo) -> np.ndarray:
    """The oracle's a-trous denoiser over one frame's feature buffers."""
    L = lib()
    L.kp_denoise.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P]
    arrs = [np.ascontiguousarray(a, t) for a, t in ((lens, np.float64), (colour, np.float64), (moment, np.float64), (length, np.float32),
                                                     (distance, np.float32), (normal, np.float64), (leaf, np.uint32), (albedo, np.float64))]
    out = np.zeros((width * height, 3), np.float32)
    L.kp_denoise(width, height, demodulated, *[_ptr(a) for a in arrs], _ptr(out))
    return out


SURFACE_DTYPE = np.dtype([("distance", "<f4"), ("normal", "<f4", 3), ("leaf", "<u4"), ("albedo", "<f4", 3)])
TPIXEL_DTYPE = np.dtype([("colour", "<f8", 3), ("moment", "<f8"), ("length", "<f4"), ("distance", "<f4"), ("normal", "<f8", 3), ("leaf", "<u4"),
                         ("albedo", "<f8", 3)], align=True)


def surfaces_array(surf: dict) -> np.ndarray:
    out = np.zeros(len(surf["leaf"]), SURFACE_DTYPE)
    for key in ("distance", "normal", "leaf", "albedo"):
        out[key] = surf[key]
    return out


def temporal(width: int, height: int, moved: bool, recounted: bool, kept: bool, lens_now, lens_before, light, first: dict, centre: dict,
             before: np.ndarray | None, film=(1, 0, 1, 0)):
    """The oracle's temporal member over one frame (kp_temporal) on the drawn
    grid: the state after (TPIXEL_DTYPE) and the image.  film: this frame's
    film factor and phase, then the state before's."""
    L = lib()
    L.kp_temporal.argtypes = [ctypes.c_int] * 5 + [_P] * 9
    film_arr = np.ascontiguousarray(film, np.int32)
    n = width * height
    prev = np.zeros(n, TPIXEL_DTYPE) if before is None else np.ascontiguousarray(before, TPIXEL_DTYPE)
    after = np.zeros(n, TPIXEL_DTYPE)
    image = np.zeros((n, 3), np.float32)
    ln = np.ascontiguousarray(lens_now, np.float64)
    lb = np.ascontiguousarray(lens_before, np.float64)
    li = np.ascontiguousarray(light, np.float64)
    fs = surfaces_array(first)
    cs = surfaces_array(centre)
    L.kp_temporal(width, height, int(moved), int(recounted), int(kept), _ptr(film_arr), _ptr(ln), _ptr(lb), _ptr(li), _ptr(fs), _ptr(cs), _ptr(prev),
                  _ptr(after), _ptr(image))
    return after, image
