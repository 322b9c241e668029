"""Seeded synthetic scenes in the reference renderer's `.sdf` language.

The reference ships hand-written scenes only, so the workloads are written
here from a seed: the same text is loaded by the reference renderer (which
compiles it to object programs, target/docs/reference_language.md) and by
the fixture exporter that turns the compiled scene into the blocks this
backend consumes.  Every random draw comes from ``random.Random(seed)``, so
a (config, seed) pair names one scene.

Emitters that the workloads describe as blackbodies are converted to
linear-RGB power here (the reference has RGB lights only, its
``Light.power`` in sdf/scene.h), by integrating Planck's law against the
CIE 1931 observer (the analytic multi-lobe fit of Wyman, Sloan and Shirley,
JCGT 2013) and the sRGB primaries.
"""
from __future__ import annotations

import math
import random

__all__ = ["blackbody_rgb", "scene_config1", "scene_config2", "scene_room", "scene_serving", "SCENES"]


def _cie_xyz(nm: float) -> tuple[float, float, float]:
    def g(x, mu, s1, s2):
        s = s1 if x < mu else s2
        t = (x - mu) / s
        return math.exp(-0.5 * t * t)

    x = 1.056 * g(nm, 599.8, 37.9, 31.0) + 0.362 * g(nm, 442.0, 16.0, 26.7) - 0.065 * g(nm, 501.1, 20.4, 26.2)
    y = 0.821 * g(nm, 568.8, 46.9, 40.5) + 0.286 * g(nm, 530.9, 16.3, 31.1)
    z = 1.217 * g(nm, 437.0, 11.8, 36.0) + 0.681 * g(nm, 459.0, 26.0, 13.8)
    return x, y, z


def blackbody_rgb(kelvin: float, luminance: float = 1.0) -> list[float]:
    """Linear sRGB of a blackbody at ``kelvin``, scaled so that its CIE Y is
    ``luminance``.  Planck's law is integrated over 380-780 nm in 1 nm steps."""
    h, c, k = 6.62607015e-34, 2.99792458e8, 1.380649e-23
    X = Y = Z = 0.0
    for i in range(380, 781):
        lam = i * 1e-9
        b = (2 * h * c * c) / (lam ** 5) / (math.exp(h * c / (lam * k * kelvin)) - 1)
        x, y, z = _cie_xyz(float(i))
        X += b * x
        Y += b * y
        Z += b * z
    X, Z = X / Y * luminance, Z / Y * luminance
    Y = luminance
    r = 3.2406 * X - 1.5372 * Y - 0.4986 * Z
    g = -0.9689 * X + 1.8758 * Y + 0.0415 * Z
    b = 0.0557 * X - 0.2040 * Y + 1.0570 * Z
    return [max(r, 0.0), max(g, 0.0), max(b, 0.0)]


def _f(x: float) -> str:
    return repr(round(float(x), 6))


def _v(v) -> str:
    return "[" + ", ".join(_f(x) for x in v) + "]"


_SHAPES = """function sphere(r) {
	return length(p) - r;
}

function box(size, r) {
	let q = abs(p) - size / 2 + r;
	return length(max(q, 0)) + min(max(q.x, max(q.y, q.z)), 0) - r;
}

function plane(normal, offset) {
	return dot(p, normal) - offset;
}

function lattice(step, r) {
	let q = p - step * floor(p / step + 0.5);
	return length(q) - r;
}
"""


def _header(width, height, samples, surfaces, seed, eye, target, fov, far=60.0):
    return (
        _SHAPES
        + "\nrender {\n"
        + f"\twidth    = {width};\n\theight   = {height};\n\tsamples  = {samples};\n"
        + f"\tbatch    = {samples};\n\tsplit    = 1;\n\tsurfaces = {surfaces};\n\tseed     = {seed};\n\tfar      = {_f(far)};\n}}\n\n"
        + "camera {\n"
        + f"\teye    = {_v(eye)};\n\ttarget = {_v(target)};\n\tfov    = {_f(fov)};\n}}\n\n"
    )


def _sky(rgb):
    return (
        "sky gradient {\n"
        + f"\tzenith  = {_v(rgb)};\n\thorizon = {_v(rgb)};\n\tground  = {_v(rgb)};\n}}\n\n"
    )


def _quad(corner, along, across, power):
    return (
        "light quad {\n"
        + f"\tat     = {_v(corner)};\n\talong  = {_v(along)};\n\tacross = {_v(across)};\n\tpower  = {_v(power)};\n}}\n\n"
    )


def scene_config1(seed: int = 1, width: int = 256, height: int = 256, samples: int = 16, surfaces: int = 8, count: int = 64) -> str:
    """64 primitives (spheres r~U(0.1,0.5), boxes half-extents ~U(0.1,0.4)
    rounded 0.02) uniform in [-2,2]^3 inside one merge(0.05), above a ground
    plane; plastic(albedo~U(0.2,0.8)^3, roughness~U(0.05,0.5)); one quad
    light emitting 5000 K; black sky."""
    rng = random.Random(seed)
    out = [_header(width, height, samples, surfaces, seed, [0.0, -8.5, 3.2], [0.0, 0.0, -0.6], 0.75)]
    out.append(_sky([0.0, 0.0, 0.0]))
    out.append(_quad([-1.25, 1.25, 4.5], [2.5, 0.0, 0.0], [0.0, -2.5, 0.0], blackbody_rgb(5000.0, 60.0)))
    out.append("let ground = plastic([0.5, 0.5, 0.5], roughness = 0.5);\n\n")
    out.append("paint(ground) plane([0, 0, 1], -2.2);\n\n")
    out.append("merge(0.05) {\n")
    for _ in range(count):
        albedo = [rng.uniform(0.2, 0.8) for _ in range(3)]
        rough = rng.uniform(0.05, 0.5)
        pos = [rng.uniform(-2.0, 2.0) for _ in range(3)]
        mat = f"plastic({_v(albedo)}, roughness = {_f(rough)})"
        if rng.random() < 0.5:
            shape = f"sphere({_f(rng.uniform(0.1, 0.5))})"
        else:
            half = [rng.uniform(0.1, 0.4) for _ in range(3)]
            shape = f"box({_v([2 * h for h in half])}, 0.02)"
        out.append(f"\tpaint({mat}) at({_v(pos)}) {shape};\n")
    out.append("}\n")
    return "".join(out)


def scene_config2(seed: int = 1, width: int = 1920, height: int = 1080, samples: int = 64, surfaces: int = 16, groups: int = 512) -> str:
    """4096 primitives in groups of 8 joined by union, subtraction (cut) or
    smooth union k~U(0.01,0.1), plus floor-based 3-axis repetition inside a
    function; materials 40% matte, 40% metal (GGX conductor), 20% glass with
    Cauchy dispersion (A=1.76, B=0.01 um^2); two quad lights and a constant
    6500 K environment."""
    rng = random.Random(seed)
    out = [_header(width, height, samples, surfaces, seed, [0.5, -15.0, 6.5], [0.0, 0.0, -0.5], 0.8)]
    out.append(_sky(blackbody_rgb(6500.0, 0.25)))
    out.append(_quad([-4.0, -1.0, 7.0], [3.0, 0.0, 0.0], [0.0, -2.0, 0.0], blackbody_rgb(5000.0, 120.0)))
    out.append(_quad([2.0, 3.0, 6.0], [2.0, 0.0, 0.0], [0.0, -2.0, 0.0], blackbody_rgb(3500.0, 80.0)))
    out.append("paint(matte([0.45, 0.45, 0.45])) plane([0, 0, 1], -3);\n\n")
    mats = []
    for i in range(groups):
        r = rng.random()
        if r < 0.4:
            mats.append(f"matte({_v([rng.uniform(0.2, 0.8) for _ in range(3)])})")
        elif r < 0.8:
            mats.append(f"metal({_v([rng.uniform(0.5, 0.95) for _ in range(3)])}, roughness = {_f(rng.uniform(0.05, 0.5))})")
        else:
            mats.append("glass(refraction = 1.76, dispersion = 0.01, roughness = 0)")
    for i in range(groups):
        center = [rng.uniform(-8.0, 8.0), rng.uniform(-6.0, 10.0), rng.uniform(-2.5, 2.5)]
        kind = rng.random()
        if kind < 0.35:
            head = "merge {"
        elif kind < 0.65:
            head = f"merge({_f(rng.uniform(0.01, 0.1))}) {{"
        else:
            head = f"cut({_f(rng.uniform(0.01, 0.05))}) {{"
        out.append(f"paint({mats[i]}) at({_v(center)}) {head}\n")
        for j in range(8):
            pos = [rng.uniform(-0.45, 0.45) for _ in range(3)]
            if i % 16 == 5 and j == 0:
                shape = f"clip {{\n\t\tlattice(0.18, 0.05);\n\t\tbox({_v([0.7, 0.7, 0.7])}, 0.02);\n\t}}"
                out.append(f"\tat({_v(pos)}) {shape}\n")
                continue
            if rng.random() < 0.5:
                shape = f"sphere({_f(rng.uniform(0.08, 0.3))})"
            else:
                shape = f"box({_v([rng.uniform(0.15, 0.5) for _ in range(3)])}, 0.02)"
            out.append(f"\tat({_v(pos)}) {shape};\n")
        out.append("}\n\n")
    return "".join(out)


def scene_room(seed: int = 1, width: int = 1920, height: int = 1080, samples: int = 16, surfaces: int = 8, count: int = 64) -> str:
    """The config-1 primitives inside a closed room of five box walls and a
    ceiling whose only opening is an aperture of about 5% of the ceiling,
    lit from above through it: indirect-dominated transport."""
    rng = random.Random(seed)
    out = [_header(width, height, samples, surfaces, seed, [0.0, -4.6, 0.4], [0.0, 0.0, -0.6], 1.0)]
    out.append(_sky([0.0, 0.0, 0.0]))
    out.append(_quad([-0.5, 0.5, 6.0], [1.0, 0.0, 0.0], [0.0, -1.0, 0.0], blackbody_rgb(5000.0, 400.0)))
    out.append("let wall = matte([0.7, 0.7, 0.7]);\n\n")
    out.append("with paint(wall) {\n")
    out.append("\tat([0, 0, -3.2]) box([10.4, 10.4, 0.4], 0);\n")
    out.append("\tat([-5, 0, 0]) box([0.4, 10.4, 6.8], 0);\n")
    out.append("\tat([5, 0, 0]) box([0.4, 10.4, 6.8], 0);\n")
    out.append("\tat([0, 5, 0]) box([10.4, 0.4, 6.8], 0);\n")
    out.append("\tat([0, -5, 0]) box([10.4, 0.4, 6.8], 0);\n")
    out.append("\tcut {\n\t\tat([0, 0, 3.2]) box([10.4, 10.4, 0.4], 0);\n\t\tat([0, 0, 3.2]) box([2.2, 2.2, 1.0], 0);\n\t}\n")
    out.append("}\n\n")
    out.append("merge(0.05) {\n")
    for _ in range(count):
        albedo = [rng.uniform(0.2, 0.8) for _ in range(3)]
        pos = [rng.uniform(-2.0, 2.0) for _ in range(3)]
        mat = f"matte({_v(albedo)})"
        if rng.random() < 0.5:
            shape = f"sphere({_f(rng.uniform(0.1, 0.5))})"
        else:
            shape = f"box({_v([2 * rng.uniform(0.1, 0.4) for _ in range(3)])}, 0.02)"
        out.append(f"\tpaint({mat}) at({_v(pos)}) {shape};\n")
    out.append("}\n")
    return "".join(out)


def scene_glow(seed: int = 1, width: int = 256, height: int = 256, samples: int = 16, surfaces: int = 8, count: int = 12) -> str:
    """Glowing surfaces (a material's glow times its strength, seen where a
    ray arrives from outside): config-1 primitives in one merge(0.05), a
    third glowing dark mattes, a third glowing plastics, the rest plain
    plastics, so blend seams mix glowing and plain leaves; one glowing
    smooth glass sphere, whose inside hits see no glow; a dim quad light
    and a dim grey sky."""
    rng = random.Random(seed)
    out = [_header(width, height, samples, surfaces, seed, [0.0, -8.5, 3.2], [0.0, 0.0, -0.6], 0.75)]
    out.append(_sky([0.02, 0.02, 0.03]))
    out.append(_quad([-1.25, 1.25, 4.5], [2.5, 0.0, 0.0], [0.0, -2.5, 0.0], blackbody_rgb(5000.0, 20.0)))
    out.append("paint(plastic([0.5, 0.5, 0.5], roughness = 0.5)) plane([0, 0, 1], -2.2);\n\n")
    out.append(f"paint(glass(refraction = 1.5, roughness = 0, glow = {_v([0.9, 0.4, 0.1])}, strength = 2)) at([0.4, -2.6, -1.4]) sphere(0.6);\n\n")
    out.append("merge(0.05) {\n")
    for k in range(count):
        albedo = [rng.uniform(0.2, 0.8) for _ in range(3)]
        glow = [rng.uniform(0.1, 1.0) for _ in range(3)]
        strength = rng.uniform(1.0, 8.0)
        pos = [rng.uniform(-2.0, 2.0) for _ in range(3)]
        if k % 3 == 0:
            mat = f"matte([0.05, 0.05, 0.05], glow = {_v(glow)}, strength = {_f(strength)})"
        elif k % 3 == 1:
            mat = f"plastic({_v(albedo)}, roughness = {_f(rng.uniform(0.05, 0.5))}, glow = {_v(glow)}, strength = {_f(strength)})"
        else:
            mat = f"plastic({_v(albedo)}, roughness = {_f(rng.uniform(0.05, 0.5))})"
        if rng.random() < 0.5:
            shape = f"sphere({_f(rng.uniform(0.2, 0.6))})"
        else:
            shape = f"box({_v([2 * rng.uniform(0.15, 0.45) for _ in range(3)])}, 0.02)"
        out.append(f"\tpaint({mat}) at({_v(pos)}) {shape};\n")
    out.append("}\n")
    return "".join(out)


def scene_glass(seed: int = 1, width: int = 256, height: int = 256, samples: int = 16, surfaces: int = 12, count: int = 8, rough: bool = False) -> str:
    """Absorbing glass bodies (each leg inside keeps exp(-absorb x length)
    a wavelength): ``count`` glass spheres and rounded boxes,
    absorb~U(0.1,2.5)^3, every other one dispersive, over a merge(0.05) of
    plastic primitives on a ground plane; one quad light, a dim sky.  The
    glass is smooth, or with ``rough`` of roughness U(0.05, 0.5) for all
    but every fourth body."""
    rng = random.Random(seed)
    out = [_header(width, height, samples, surfaces, seed, [0.0, -8.5, 3.2], [0.0, 0.0, -0.6], 0.75)]
    out.append(_sky([0.08, 0.08, 0.1]))
    out.append(_quad([-1.25, 1.25, 4.5], [2.5, 0.0, 0.0], [0.0, -2.5, 0.0], blackbody_rgb(5000.0, 60.0)))
    out.append("paint(plastic([0.5, 0.5, 0.5], roughness = 0.5)) plane([0, 0, 1], -2.2);\n\n")
    for k in range(count):
        absorb = [rng.uniform(0.1, 2.5) for _ in range(3)]
        pos = [rng.uniform(-2.0, 2.0), rng.uniform(-2.5, 0.5), rng.uniform(-1.8, 1.0)]
        dispersion = ", dispersion = 0.01" if k % 2 else ""
        roughness = _f(rng.uniform(0.05, 0.5)) if rough and k % 4 else "0"
        mat = f"glass(refraction = 1.5{dispersion}, roughness = {roughness}, absorb = {_v(absorb)})"
        if rng.random() < 0.5:
            shape = f"sphere({_f(rng.uniform(0.3, 0.7))})"
        else:
            shape = f"box({_v([2 * rng.uniform(0.2, 0.5) for _ in range(3)])}, 0.05)"
        out.append(f"paint({mat}) at({_v(pos)}) {shape};\n")
    out.append("\nmerge(0.05) {\n")
    for _ in range(count):
        albedo = [rng.uniform(0.2, 0.8) for _ in range(3)]
        pos = [rng.uniform(-2.0, 2.0), rng.uniform(0.5, 2.5), rng.uniform(-1.8, 1.0)]
        mat = f"plastic({_v(albedo)}, roughness = {_f(rng.uniform(0.05, 0.5))})"
        if rng.random() < 0.5:
            shape = f"sphere({_f(rng.uniform(0.2, 0.6))})"
        else:
            shape = f"box({_v([2 * rng.uniform(0.15, 0.45) for _ in range(3)])}, 0.02)"
        out.append(f"\tpaint({mat}) at({_v(pos)}) {shape};\n")
    out.append("}\n")
    return "".join(out)


def scene_films(seed: int = 1, width: int = 256, height: int = 256, samples: int = 16, surfaces: int = 12, count: int = 12) -> str:
    """Thin films (``film = [thickness, index]``): ``count`` bodies cycling
    through a filmed metal (oxide-like, 250-600 nm of index 1.8-2.4), a
    filmed plastic (300-700 nm of 1.3-1.6), a filmed glass of refraction
    1.5 (smooth, rough, or dispersive), and a soap bubble (a glass of
    refraction 1 under 250-550 nm of index 1.33, which bends nothing but is
    no passable glass), over a plastic ground; one quad light, a dim sky.
    The bodies neither touch one another nor reach the ground (bounding
    spheres kept 0.05 apart): a path in a body that does not absorb, in a
    scene where another glass does, that leaves its body through a touching
    one's surface or the ground's open half-space and escapes to the sky
    would be kept exp(-0 x inf), a NaN, in the reference
    (absorption.cpp:28 keptThrough) as here."""
    rng = random.Random(seed)
    out = [_header(width, height, samples, surfaces, seed, [0.0, -8.5, 3.2], [0.0, 0.0, -0.6], 0.75)]
    out.append(_sky([0.1, 0.1, 0.12]))
    out.append(_quad([-1.25, 1.25, 4.5], [2.5, 0.0, 0.0], [0.0, -2.5, 0.0], blackbody_rgb(5000.0, 60.0)))
    out.append("paint(plastic([0.5, 0.5, 0.5], roughness = 0.5)) plane([0, 0, 1], -2.2);\n\n")
    placed = []
    for k in range(count):
        role = k % 4
        if role == 0:
            film = _v([round(rng.uniform(250.0, 600.0)), rng.uniform(1.8, 2.4)])
            mat = f"metal({_v([rng.uniform(0.5, 0.95) for _ in range(3)])}, roughness = {_f(rng.uniform(0.05, 0.4))}, film = {film})"
        elif role == 1:
            film = _v([round(rng.uniform(300.0, 700.0)), rng.uniform(1.3, 1.6)])
            mat = f"plastic({_v([rng.uniform(0.2, 0.8) for _ in range(3)])}, roughness = {_f(rng.uniform(0.05, 0.4))}, film = {film})"
        elif role == 2:
            film = _v([round(rng.uniform(250.0, 600.0)), rng.uniform(1.3, 2.0)])
            variant = (k // 4) % 3
            extra = [", roughness = 0", f", roughness = {_f(rng.uniform(0.05, 0.3))}", ", roughness = 0, dispersion = 0.01"][variant]
            mat = f"glass(refraction = 1.5{extra}, absorb = {_v([rng.uniform(0.1, 1.0) for _ in range(3)])}, film = {film})"
        else:
            film = _v([round(rng.uniform(250.0, 550.0)), 1.33])
            mat = f"glass(refraction = 1, roughness = 0, film = {film})"
        if role == 3 or rng.random() < 0.6:
            radius = rng.uniform(0.3, 0.7)
            shape, bound = f"sphere({_f(radius)})", radius
        else:
            size = [2 * rng.uniform(0.2, 0.5) for _ in range(3)]
            shape, bound = f"box({_v(size)}, 0.05)", 0.5 * math.sqrt(sum(x * x for x in size))
        for _ in range(1000):
            pos = [rng.uniform(-2.4, 2.4), rng.uniform(-2.2, 2.2), rng.uniform(-1.3, 1.2)]
            if pos[2] - bound > -2.15 and all(math.dist(pos, q) > bound + b + 0.05 for q, b in placed):
                break
        else:
            continue
        placed.append((pos, bound))
        out.append(f"paint({mat}) at({_v(pos)}) {shape};\n")
    return "".join(out)


def scene_config5(seed: int = 1, width: int = 3840, height: int = 2160, samples: int = 256, surfaces: int = 32, side: int = 256) -> str:
    """The stress scene: a city of side x side rounded boxes on a grid
    (0.25 apart, footprints 0.16-0.2, heights 0.4 x LogNormal(0, 0.5)),
    each its own object, plastics and metals; above its middle a cluster of
    24 dispersive glass spheres (refraction 1.5, dispersion 0.02) that
    throws caustics on the roofs; a warm quad light high over the centre and
    a dim sky."""
    rng = random.Random(seed)
    span = 0.25 * side
    out = [_header(width, height, samples, surfaces, seed, [0.0, -0.62 * span, 0.3 * span], [0.0, 0.0, 0.0], 0.9, far=1.6 * span)]
    out.append(_sky([0.06, 0.07, 0.09]))
    out.append(_quad([-0.1 * span, 0.1 * span, 0.45 * span], [0.2 * span, 0.0, 0.0], [0.0, -0.2 * span, 0.0], blackbody_rgb(5000.0, 40.0)))
    out.append("paint(matte([0.35, 0.35, 0.35])) plane([0, 0, 1], 0);\n\n")
    mats = [f"plastic({_v([rng.uniform(0.3, 0.8) for _ in range(3)])}, roughness = {_f(rng.uniform(0.1, 0.6))})" for _ in range(6)]
    mats += [f"metal({_v([rng.uniform(0.6, 0.95) for _ in range(3)])}, roughness = {_f(rng.uniform(0.05, 0.3))})" for _ in range(2)]
    for k, m in enumerate(mats):
        out.append(f"let m{k} = {m};\n")
    out.append("\n")
    for i in range(side):
        for j in range(side):
            h = 0.4 * math.exp(rng.gauss(0.0, 0.5))
            wx, wy = rng.uniform(0.16, 0.2), rng.uniform(0.16, 0.2)
            pos = [(i - side / 2 + 0.5) * 0.25, (j - side / 2 + 0.5) * 0.25, h / 2]
            out.append(f"paint(m{rng.randrange(len(mats))}) at({_v(pos)}) box({_v([wx, wy, h])}, 0.02);\n")
    out.append("\nwith paint(glass(refraction = 1.5, dispersion = 0.02, roughness = 0)) {\n")
    for _ in range(24):
        pos = [rng.uniform(-1.5, 1.5), rng.uniform(-1.5, 1.5), rng.uniform(3.0, 4.5)]
        out.append(f"\tat({_v(pos)}) sphere({_f(rng.uniform(0.2, 0.45))});\n")
    out.append("}\n")
    return "".join(out)


def scene_skylit(seed: int = 1, width: int = 256, height: int = 256, samples: int = 16, surfaces: int = 8, count: int = 12) -> str:
    """Lit by the sky: config-1 primitives (plastics and metals) on a
    plastic ground under a bright gradient sky (blue zenith, white horizon,
    dark ground) and one dim quad lamp that does not outshine it, so that
    --use sampler=sky_map charts the sky."""
    rng = random.Random(seed)
    out = [_header(width, height, samples, surfaces, seed, [0.0, -8.5, 3.2], [0.0, 0.0, -0.6], 0.75)]
    out.append("sky gradient {\n\tzenith  = [0.6, 0.8, 1.4];\n\thorizon = [1.0, 1.0, 1.0];\n\tground  = [0.15, 0.13, 0.1];\n}\n\n")
    out.append(_quad([-0.5, 0.5, 4.5], [1.0, 0.0, 0.0], [0.0, -1.0, 0.0], blackbody_rgb(5000.0, 8.0)))
    out.append("paint(plastic([0.5, 0.5, 0.5], roughness = 0.5)) plane([0, 0, 1], -2.2);\n\n")
    out.append("merge(0.05) {\n")
    for k in range(count):
        pos = [rng.uniform(-2.0, 2.0) for _ in range(3)]
        if k % 3 == 2:
            mat = f"metal({_v([rng.uniform(0.5, 0.95) for _ in range(3)])}, roughness = {_f(rng.uniform(0.1, 0.4))})"
        else:
            mat = f"plastic({_v([rng.uniform(0.2, 0.8) for _ in range(3)])}, roughness = {_f(rng.uniform(0.1, 0.5))})"
        if rng.random() < 0.5:
            shape = f"sphere({_f(rng.uniform(0.25, 0.6))})"
        else:
            shape = f"box({_v([2 * rng.uniform(0.15, 0.45) for _ in range(3)])}, 0.02)"
        out.append(f"\tpaint({mat}) at({_v(pos)}) {shape};\n")
    out.append("}\n")
    return "".join(out)


def scene_lamps(seed: int = 1, width: int = 256, height: int = 256, samples: int = 16, surfaces: int = 8, count: int = 12) -> str:
    """Lit by many lamps: config-1 primitives (plastics and metals) on a
    plastic ground under a black sky, lit by four small sphere lamps of
    unlike colour and power around the scene and two quad lamps above it,
    so that --use sampler=each_lamp_first gives the first four lamps a line
    of their own at the first vertex and the reservoir the other two."""
    rng = random.Random(seed)
    out = [_header(width, height, samples, surfaces, seed, [0.0, -8.5, 3.2], [0.0, 0.0, -0.6], 0.75)]
    out.append(_sky([0.0, 0.0, 0.0]))
    for k in range(4):
        turn = 2.0 * math.pi * (k + rng.uniform(0.1, 0.9)) / 4.0
        at = [3.0 * math.cos(turn), 3.0 * math.sin(turn), rng.uniform(0.5, 3.0)]
        power = blackbody_rgb(rng.uniform(2500.0, 9000.0), rng.uniform(6.0, 30.0))
        out.append("light sphere {\n" + f"\tat     = {_v(at)};\n\tradius = {_f(rng.uniform(0.05, 0.3))};\n\tpower  = {_v(power)};\n}}\n\n")
    out.append(_quad([-1.5, 1.0, 4.5], [1.0, 0.0, 0.0], [0.0, -1.0, 0.0], blackbody_rgb(5000.0, 25.0)))
    out.append(_quad([0.5, 1.5, 4.0], [1.2, 0.0, 0.0], [0.0, -0.6, 0.0], blackbody_rgb(3500.0, 15.0)))
    out.append("paint(plastic([0.5, 0.5, 0.5], roughness = 0.5)) plane([0, 0, 1], -2.2);\n\n")
    out.append("merge(0.05) {\n")
    for k in range(count):
        pos = [rng.uniform(-2.0, 2.0) for _ in range(3)]
        if k % 3 == 2:
            mat = f"metal({_v([rng.uniform(0.5, 0.95) for _ in range(3)])}, roughness = {_f(rng.uniform(0.1, 0.4))})"
        else:
            mat = f"plastic({_v([rng.uniform(0.2, 0.8) for _ in range(3)])}, roughness = {_f(rng.uniform(0.1, 0.5))})"
        if rng.random() < 0.5:
            shape = f"sphere({_f(rng.uniform(0.25, 0.6))})"
        else:
            shape = f"box({_v([2 * rng.uniform(0.15, 0.45) for _ in range(3)])}, 0.02)"
        out.append(f"\tpaint({mat}) at({_v(pos)}) {shape};\n")
    out.append("}\n")
    return "".join(out)


def scene_far_lights(seed: int = 1, width: int = 256, height: int = 256, samples: int = 16, surfaces: int = 8, count: int = 12) -> str:
    """Lit by every kind of light but the area lamps: config-1 primitives
    (plastics and rough metals) on a plastic ground under a dim gradient
    sky, lit by a point light, a directional light, a sun (a disc 0.05
    radians across) and a moon (0.06 radians, its lit share set by the
    sun's direction)."""
    rng = random.Random(seed)
    out = [_header(width, height, samples, surfaces, seed, [0.0, -8.5, 3.2], [0.0, 0.0, -0.6], 0.75)]
    out.append("sky gradient {\n\tzenith  = [0.04, 0.05, 0.09];\n\thorizon = [0.08, 0.08, 0.08];\n\tground  = [0.02, 0.02, 0.02];\n}\n\n")
    out.append("light point {\n\tat    = [1.6, -1.8, 2.6];\n" + f"\tpower = {_v(blackbody_rgb(3200.0, 18.0))};\n}}\n\n")
    out.append("light directional {\n\tdirection = [0.3, -0.6, 0.7];\n" + f"\tpower     = {_v(blackbody_rgb(7000.0, 0.6))};\n}}\n\n")
    out.append("light sun {\n\tdirection = [-0.5, 0.3, 0.62];\n\tangle     = 0.05;\n" + f"\tpower     = {_v(blackbody_rgb(5500.0, 1.6))};\n}}\n\n")
    out.append("light moon {\n\tdirection = [0.55, 0.45, 0.5];\n\tangle     = 0.06;\n" + f"\tpower     = {_v(blackbody_rgb(4500.0, 0.5))};\n}}\n\n")
    out.append("paint(plastic([0.5, 0.5, 0.5], roughness = 0.5)) plane([0, 0, 1], -2.2);\n\n")
    out.append("merge(0.05) {\n")
    for k in range(count):
        pos = [rng.uniform(-2.0, 2.0) for _ in range(3)]
        if k % 3 == 2:
            mat = f"metal({_v([rng.uniform(0.5, 0.95) for _ in range(3)])}, roughness = {_f(rng.uniform(0.15, 0.4))})"
        else:
            mat = f"plastic({_v([rng.uniform(0.2, 0.8) for _ in range(3)])}, roughness = {_f(rng.uniform(0.1, 0.5))})"
        if rng.random() < 0.5:
            shape = f"sphere({_f(rng.uniform(0.25, 0.6))})"
        else:
            shape = f"box({_v([2 * rng.uniform(0.15, 0.45) for _ in range(3)])}, 0.02)"
        out.append(f"\tpaint({mat}) at({_v(pos)}) {shape};\n")
    out.append("}\n")
    return "".join(out)


def scene_scattering(seed: int = 1, width: int = 256, height: int = 256, samples: int = 16, surfaces: int = 8, count: int = 8) -> str:
    """Scattering bodies: a rough glass ball that scatters forward (refraction
    1.35, roughness 0.2, scatter 4, lean 0.3, a faint blue absorption), a
    smooth glass box that scatters backward (refraction 1.5, scatter 2.5,
    lean -0.2) and a smooth glass ball that scatters evenly (scatter 1.5),
    among config-1 plastics on a plastic ground; one quad light, a dim sky."""
    rng = random.Random(seed)
    out = [_header(width, height, samples, surfaces, seed, [0.0, -8.5, 3.2], [0.0, 0.0, -0.6], 0.75)]
    out.append(_sky([0.05, 0.05, 0.06]))
    out.append(_quad([-1.25, 1.25, 4.5], [2.5, 0.0, 0.0], [0.0, -2.5, 0.0], blackbody_rgb(5000.0, 40.0)))
    out.append("paint(plastic([0.5, 0.5, 0.5], roughness = 0.5)) plane([0, 0, 1], -2.2);\n\n")
    out.append("paint(glass(refraction = 1.35, absorb = [0.05, 0.08, 0.2], roughness = 0.2, scatter = 4, lean = 0.3)) at([-1.1, 0.2, -1.2]) sphere(0.9);\n")
    out.append("paint(glass(refraction = 1.5, scatter = 2.5, lean = -0.2)) at([1.2, -0.3, -1.5]) box([1.2, 1.2, 1.2], 0.05);\n")
    out.append("paint(glass(refraction = 1.45, scatter = 1.5)) at([0.1, 1.4, -1.6]) sphere(0.6);\n\n")
    # the plastics stay clear of the glass bodies (a body must not overlap another)
    bodies = [([-1.1, 0.2, -1.2], 1.1), ([1.2, -0.3, -1.5], 1.1), ([0.1, 1.4, -1.6], 0.8)]
    out.append("merge(0.05) {\n")
    placed = 0
    while placed < count:
        pos = [rng.uniform(-2.5, 2.5), rng.uniform(-2.0, 2.5), rng.uniform(-1.9, 0.5)]
        r = rng.uniform(0.2, 0.4)
        if any(math.dist(pos, c) < rr + r + 0.1 for c, rr in bodies):
            continue
        albedo = [rng.uniform(0.2, 0.8) for _ in range(3)]
        out.append(f"\tpaint(plastic({_v(albedo)}, roughness = {_f(rng.uniform(0.1, 0.5))})) at({_v(pos)}) sphere({_f(r)});\n")
        placed += 1
    out.append("}\n")
    return "".join(out)


def scene_lens(seed: int = 1, width: int = 256, height: int = 256, samples: int = 16, surfaces: int = 8, count: int = 12) -> str:
    """Through a thin lens: config-1 primitives (plastics and metals) on a
    plastic ground, seen through a lens of radius 0.25 sharp 8 units ahead
    (the nearer and further primitives blurred); one quad light, a dim sky."""
    rng = random.Random(seed)
    head = _header(width, height, samples, surfaces, seed, [0.0, -8.5, 3.2], [0.0, 0.0, -0.6], 0.75)
    head = head.replace("\tfov    = 0.75;\n", "\tfov    = 0.75;\n\taperture = 0.25;\n\tfocus    = 8;\n")
    assert "aperture" in head
    out = [head, _sky([0.05, 0.05, 0.06])]
    out.append(_quad([-1.25, 1.25, 4.5], [2.5, 0.0, 0.0], [0.0, -2.5, 0.0], blackbody_rgb(5000.0, 40.0)))
    out.append("paint(plastic([0.5, 0.5, 0.5], roughness = 0.5)) plane([0, 0, 1], -2.2);\n\n")
    out.append("merge(0.05) {\n")
    for k in range(count):
        pos = [rng.uniform(-2.5, 2.5), rng.uniform(-3.0, 3.0), rng.uniform(-2.0, 0.5)]
        if k % 3 == 2:
            mat = f"metal({_v([rng.uniform(0.5, 0.95) for _ in range(3)])}, roughness = {_f(rng.uniform(0.1, 0.4))})"
        else:
            mat = f"plastic({_v([rng.uniform(0.2, 0.8) for _ in range(3)])}, roughness = {_f(rng.uniform(0.1, 0.5))})"
        shape = f"sphere({_f(rng.uniform(0.25, 0.6))})" if rng.random() < 0.5 else f"box({_v([2 * rng.uniform(0.15, 0.45) for _ in range(3)])}, 0.02)"
        out.append(f"\tpaint({mat}) at({_v(pos)}) {shape};\n")
    out.append("}\n")
    return "".join(out)


def scene_split(seed: int = 1, width: int = 256, height: int = 256, samples: int = 16, surfaces: int = 8, count: int = 12) -> str:
    """The many-lamp scene (scene_lamps) drawn with render.split = 4: each
    group of four samples shares its camera ray, wavelengths and first
    vertex's aim, and each branches on its own from there."""
    text = scene_lamps(seed, width, height, samples, surfaces, count)
    assert "\tsplit    = 1;\n" in text
    return text.replace("\tsplit    = 1;\n", "\tsplit    = 4;\n", 1)


def scene_stars(seed: int = 1, width: int = 256, height: int = 256, samples: int = 16, surfaces: int = 8, count: int = 12) -> str:
    """A starry night: config-1 primitives (plastics and polished metals that
    mirror the stars) on a dark ground under a dim night-blue sky with 3000
    stars of discs 0.04 radians across, lit also by a dim quad lamp; the
    camera looks level enough to see the stars above the horizon."""
    rng = random.Random(seed)
    out = [_header(width, height, samples, surfaces, seed, [0.0, -8.5, 1.2], [0.0, 0.0, 0.4], 0.9)]
    out.append("sky gradient {\n\tzenith  = [0.005, 0.008, 0.02];\n\thorizon = [0.01, 0.012, 0.02];\n\tground  = [0.002, 0.002, 0.002];\n}\n\n")
    out.append("stars {\n\tcount    = 3000;\n\tstrength = 60;\n\tangle    = 0.04;\n}\n\n")
    out.append(_quad([-0.5, 0.5, 4.5], [1.0, 0.0, 0.0], [0.0, -1.0, 0.0], blackbody_rgb(4000.0, 4.0)))
    out.append("paint(plastic([0.3, 0.3, 0.3], roughness = 0.5)) plane([0, 0, 1], -2.2);\n\n")
    out.append("merge(0.05) {\n")
    for k in range(count):
        pos = [rng.uniform(-2.0, 2.0), rng.uniform(-2.0, 2.0), rng.uniform(-2.0, 0.5)]
        if k % 2 == 1:
            mat = f"metal({_v([rng.uniform(0.7, 0.95) for _ in range(3)])}, roughness = {_f(rng.uniform(0.02, 0.1))})"
        else:
            mat = f"plastic({_v([rng.uniform(0.2, 0.8) for _ in range(3)])}, roughness = {_f(rng.uniform(0.1, 0.5))})"
        shape = f"sphere({_f(rng.uniform(0.25, 0.6))})" if rng.random() < 0.5 else f"box({_v([2 * rng.uniform(0.15, 0.45) for _ in range(3)])}, 0.02)"
        out.append(f"\tpaint({mat}) at({_v(pos)}) {shape};\n")
    out.append("}\n")
    return "".join(out)


def scene_physical_sky(seed: int = 1, width: int = 256, height: int = 256, samples: int = 16, surfaces: int = 8, count: int = 12) -> str:
    """Under a physical sky: config-1 primitives (plastics and metals) on a
    plastic ground lit by a low sun (a disc 0.05 radians across) through
    the air and haze of a physical sky with a glow about the sun; the camera
    looks level enough to see the sky above the horizon."""
    rng = random.Random(seed)
    out = [_header(width, height, samples, surfaces, seed, [0.0, -8.5, 1.2], [0.0, 0.0, 0.2], 0.9)]
    out.append("sky physical {\n\thaze     = 1.3;\n\tground   = [0.28, 0.30, 0.26];\n\tglow     = [1, 0.8, 0.55];\n"
               "\tstrength = 0.5;\n\tspread   = 0.12;\n}\n\n")
    out.append("light sun {\n\tdirection = [-0.5, 0.6, 0.35];\n\tangle     = 0.05;\n\tpower     = [3.1, 3, 2.8];\n}\n\n")
    out.append("paint(plastic([0.5, 0.5, 0.5], roughness = 0.5)) plane([0, 0, 1], -2.2);\n\n")
    out.append("merge(0.05) {\n")
    for k in range(count):
        pos = [rng.uniform(-2.0, 2.0), rng.uniform(-2.0, 2.0), rng.uniform(-2.0, 0.5)]
        if k % 3 == 2:
            mat = f"metal({_v([rng.uniform(0.5, 0.95) for _ in range(3)])}, roughness = {_f(rng.uniform(0.1, 0.4))})"
        else:
            mat = f"plastic({_v([rng.uniform(0.2, 0.8) for _ in range(3)])}, roughness = {_f(rng.uniform(0.1, 0.5))})"
        if rng.random() < 0.5:
            shape = f"sphere({_f(rng.uniform(0.25, 0.6))})"
        else:
            shape = f"box({_v([2 * rng.uniform(0.15, 0.45) for _ in range(3)])}, 0.02)"
        out.append(f"\tpaint({mat}) at({_v(pos)}) {shape};\n")
    out.append("}\n")
    return "".join(out)


_PATTERNS = """function bands(count) {
	return 0.5 + 0.5 * sin(p.z * count);
}

function cells(size) {
	let c = floor(p.x * size) + floor(p.y * size) + floor(p.z * size);
	return c - 2 * floor(c / 2);
}

function facing(axis) {
	return clamp(dot(n, axis) * 0.5 + 0.5, 0, 1);
}
"""


def scene_patterns(seed: int = 1, width: int = 256, height: int = 256, samples: int = 16, surfaces: int = 8, count: int = 12) -> str:
    """Patterned albedos (a ramp of 2-4 colour stops read off a pattern
    program of the point and the normal): a world-space cell pattern on the
    ground, and config-1 primitives in one merge(0.05), some turned, painted
    with bands (sine of height), cells (a 3-D checker) or facing (the
    normal against an axis) in the painted shape's space, or plain, so
    blend seams mix patterned and plain leaves; one quad light."""
    rng = random.Random(seed)
    out = [_header(width, height, samples, surfaces, seed, [0.0, -8.5, 3.2], [0.0, 0.0, -0.6], 0.75).replace(_SHAPES, _SHAPES + "\n" + _PATTERNS)]
    out.append(_sky([0.05, 0.05, 0.06]))
    out.append(_quad([-1.25, 1.25, 4.5], [2.5, 0.0, 0.0], [0.0, -2.5, 0.0], blackbody_rgb(5000.0, 60.0)))
    out.append("paint(matte(world(ramp(cells(1), [0.25, 0.25, 0.25], [0.7, 0.7, 0.7])))) plane([0, 0, 1], -2.2);\n\n")
    out.append("merge(0.05) {\n")
    for k in range(count):
        stops = ", ".join(_v([rng.uniform(0.1, 0.9) for _ in range(3)]) for _ in range(2 + k % 3))
        pos = [rng.uniform(-2.0, 2.0) for _ in range(3)]
        pattern = [f"bands({_f(rng.uniform(4.0, 12.0))})", f"cells({_f(rng.uniform(2.0, 6.0))})",
                   f"facing({_v([rng.uniform(-1.0, 1.0) for _ in range(3)])})", None][k % 4]
        albedo = f"ramp({pattern}, {stops})" if pattern else _v([rng.uniform(0.2, 0.8) for _ in range(3)])
        mat = f"matte({albedo})" if k % 2 == 0 else f"plastic({albedo}, roughness = {_f(rng.uniform(0.1, 0.5))})"
        turn = f" turn(z, {_f(rng.uniform(0.0, 3.0))})" if k % 3 == 0 else ""
        if rng.random() < 0.5:
            shape = f"sphere({_f(rng.uniform(0.25, 0.6))})"
        else:
            shape = f"box({_v([2 * rng.uniform(0.15, 0.45) for _ in range(3)])}, 0.02)"
        out.append(f"\tpaint({mat}) at({_v(pos)}){turn} {shape};\n")
    out.append("}\n")
    return "".join(out)


def scene_serving(seed: int, count: int, width: int = 640, height: int = 480, samples: int = 4) -> str:
    """A config-1-style scene of ``count`` primitives spread over a box that
    grows with the count, split into merge(0.05) groups of 64."""
    rng = random.Random(seed)
    reach = 2.0 * (count / 64.0) ** (1.0 / 3.0)
    out = [_header(width, height, samples, 8, seed, [0.0, -4.2 * reach, 1.6 * reach], [0.0, 0.0, -0.3 * reach], 0.75)]
    out.append(_sky([0.05, 0.05, 0.06]))
    out.append(_quad([-0.6 * reach, 0.6 * reach, 2.2 * reach], [1.2 * reach, 0.0, 0.0], [0.0, -1.2 * reach, 0.0], blackbody_rgb(5000.0, 60.0)))
    out.append(f"paint(plastic([0.5, 0.5, 0.5], roughness = 0.5)) plane([0, 0, 1], {_f(-1.1 * reach)});\n\n")
    for g in range(0, count, 64):
        out.append("merge(0.05) {\n")
        for _ in range(min(64, count - g)):
            albedo = [rng.uniform(0.2, 0.8) for _ in range(3)]
            pos = [rng.uniform(-reach, reach) for _ in range(3)]
            # roughness on a 0.01 grid: the compiled scene's finish tables
            # (one per material, derived from the roughness) repeat and
            # compress, which keeps the 16384-primitive scene small
            mat = f"plastic({_v(albedo)}, roughness = {_f(round(rng.uniform(0.05, 0.5), 2))})"
            if rng.random() < 0.5:
                shape = f"sphere({_f(rng.uniform(0.1, 0.5))})"
            else:
                shape = f"box({_v([2 * rng.uniform(0.1, 0.4) for _ in range(3)])}, 0.02)"
            out.append(f"\tpaint({mat}) at({_v(pos)}) {shape};\n")
        out.append("}\n\n")
    return "".join(out)


SCENES = {
    "config1": scene_config1,
    "config2": scene_config2,
    "room": scene_room,
}
