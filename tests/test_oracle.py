"""The oracle (oracle/port) against the reference's own outputs.

The fixtures under tests/golden were written by the reference renderer
(tests/golden/make_golden.py); the oracle must reproduce them to the bit
before the GPU path is judged against it."""
import os

import numpy as np
import pytest

import oracle.port as op
from helpers import GOLDEN, compare_cells, golden_rays, scene


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_cut_lists_match_reference(name):
    sc = scene(name)
    cut = np.load(os.path.join(GOLDEN, f"cut_{name}.npz"))
    d = int(cut["depth"])
    tree = op.Octree(sc, d, d, 1 << 30)
    assert tree.cells() == len(cut["head"])
    assert compare_cells(tree.cell, cut) == 0


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_sphere_trace_matches_reference(name):
    sc = scene(name)
    rays, tr = golden_rays(name)
    r = np.zeros(len(rays), op.RAY_DTYPE)
    r["origin"], r["direction"], r["far"], r["inside"], r["within"] = rays["origin"], rays["direction"], rays["far"], rays["inside"], rays["within"]
    h = op.sphere_trace(sc, r, tr["reach_lower"], tr["reach_size"])
    assert (h["kind"] == tr["kind"]).all()
    hit = tr["kind"] == 1
    assert (h["leaf"][hit] == tr["leaf"][hit]).all()
    assert (h["other"][hit] == tr["other"][hit]).all()
    assert (h["distance"] == tr["distance"]).all()
    assert (h["normal"] == tr["normal"]).all()
    assert (h["share"] == tr["share"]).all()


def test_octree_trace_agrees_with_whole_scene_trace():
    """Reading the field from a cell's kept programs gives the hits of the
    march over every object (the kept programs are exact in their cell)."""
    sc = scene("c1")
    rays, tr = golden_rays("c1")
    r = np.zeros(len(rays), op.RAY_DTYPE)
    r["origin"], r["direction"], r["far"], r["inside"], r["within"] = rays["origin"], rays["direction"], rays["far"], rays["inside"], rays["within"]
    tree = op.Octree(sc, 5, 9, 96)
    h = tree.trace(r)
    both = (h["kind"] == 1) & (tr["kind"] == 1)
    assert (h["kind"] == tr["kind"]).mean() > 0.995
    assert (h["leaf"][both] == tr["leaf"][both]).mean() > 0.995
    rel = np.abs(h["distance"][both] - tr["distance"][both]) / np.maximum(tr["distance"][both], 1e-6)
    assert np.quantile(rel, 0.99) < 1e-5


def denoise_cases():
    z = np.load(os.path.join(GOLDEN, "denoise.npz"))
    d = {k: z[k] for k in z.files}
    names = sorted({k.split(".", 1)[0] for k in d if "." in k})
    return d, names


def test_denoiser_matches_reference():
    """The oracle's a-trous denoiser reproduces the reference's
    denoisedFrame float for float on every fixture field."""
    d, names = denoise_cases()
    assert len(names) >= 6
    for name in names:
        f = {k.split(".", 1)[1]: v for k, v in d.items() if k.startswith(name + ".")}
        out = op.denoise(int(d["width"]), int(d["height"]), int(f["demodulated"]), d["lens"], f["colour"], f["moment"], f["length"],
                         f["distance"], f["normal"], f["leaf"], f["albedo"])
        assert np.array_equal(out, f["out"]), name


@pytest.mark.parametrize("name", ["room_small", "c1_small", "c2_small", "glow_small", "glass_small", "patterns_small", "rough_small", "films_small",
                                  "skylit_small", "lamps_small", "far_small", "scatter_small", "physical_small", "lens_small",
                                  "split_small", "stars_small"])
def test_renderer_matches_reference_frames(name):
    """The oracle's frames against the reference renderer's own
    (tests/golden/image_*.npz, 12 seeds at the scene's spp): both are
    unbiased estimates of the same image, so each channel's image mean
    agrees within 4 standard errors of the two seed sets, and at most 1.5%
    of pixel channels are more than 3 standard errors apart."""
    sc = scene(name)
    ref = np.load(os.path.join(GOLDEN, f"image_{name}.npz"))
    frames = ref["frames"].astype(np.float64)
    spp = int(ref["spp"])
    h, w = sc.render["height"], sc.render["width"]
    build = dict(min_depth=5, max_depth=10, split_steps=64)
    got = np.stack([op.render_band(sc, w, h, spp, int(sc.render["surfaces"]), s, 0, h, os.cpu_count() or 4, build) / spp for s in range(1, 9)])
    z = (got.mean(0) - frames.mean(0)) / np.sqrt(got.var(0, ddof=1) / len(got) + frames.var(0, ddof=1) / len(frames) + 1e-12)
    ca, cb = got.mean(axis=(1, 2)), frames.mean(axis=(1, 2))
    cz = (ca.mean(0) - cb.mean(0)) / np.sqrt(ca.var(0, ddof=1) / len(ca) + cb.var(0, ddof=1) / len(cb))
    print(f"{name}: oracle {ca.mean(0)} reference {cb.mean(0)} z {cz} far px {(np.abs(z) > 3).mean():.4f}")
    assert np.all(np.abs(cz) < 4)
    assert (np.abs(z) > 3).mean() <= 0.015


@pytest.mark.parametrize("name", ["films_small", "glass_small", "rough_small", "c2_small"])
def test_bsdf_matches_reference_answers(name):
    """respondBsdf and sampleBsdf (material.cpp:1076, :1366) at 200 seeded
    vertices a material (tests/golden/bsdf_*.npz, the reference's own
    answers through oracle/_ref's kdn_ref_dump bsdf): thin films on metal,
    plastic and glass (soap bubbles included), rough and smooth glass from
    either side, dispersion, matte and metal.  The reference keeps a
    vertex's indices as floats (FloatSpectrum) where the oracle keeps
    doubles, so the bars are relative (floor 1e-3): values and densities
    within 1e-5, drawn weights within 1e-4 and directions within 1e-6; found
    and through agree everywhere."""
    d = np.load(os.path.join(GOLDEN, f"bsdf_{name}.npz"))
    got = op.bsdf_answers(scene(name), d["ids"], d["records"])

    def rel(a, b):
        return np.abs(a - b) / np.maximum(np.abs(b), 1e-3)

    assert np.array_equal(got["seen"], d["seen"])
    drawn = d["seen"][:, 0] == 1
    assert rel(got["value"], d["value"]).max() < 1e-5
    assert rel(got["density"], d["density"]).max() < 1e-5
    assert np.abs(got["incoming"] - d["incoming"])[drawn].max() < 1e-6
    assert rel(got["weight"], d["weight"])[drawn].max() < 1e-4
    assert rel(got["drawn_density"], d["drawn_density"])[drawn].max() < 1e-4
    if name == "films_small":
        # the films are there: a filmed glass's lanes are drawn apart
        kinds = np.asarray(scene(name).materials["kind"])[d["ids"][:, 0]]
        spread = d["weight"].max(1) - d["weight"].min(1)
        assert (spread[(kinds == 3) & drawn] > 1e-2).sum() > 200


def test_sobol_numbers_match_reference():
    """plugins/sampler/sobol/sobol.cpp sobolNumber of 20000 seeded keys
    (tests/golden/sobol.npz: the reference's own numbers, streams of 64
    bits, indices past 2^16, every coordinate below 28), and its pairs,
    to the bit."""
    z = np.load(os.path.join(GOLDEN, "sobol.npz"))
    got = op.sobol_numbers(z["stream"], z["index"], z["coordinate"])
    assert np.array_equal(got, z["number"])
    even = z["coordinate"] & np.uint32(0xFFFFFFFE)
    assert np.array_equal(op.sobol_numbers(z["stream"], z["index"], even), z["pair"][:, 0])
    assert np.array_equal(op.sobol_numbers(z["stream"], z["index"], even + 1), z["pair"][:, 1])


@pytest.mark.parametrize("name, sampler", [("c1_small", "sobol"), ("glass_small", "sobol"), ("skylit_small", "sky_map"), ("lamps_small", "each_lamp_first")])
def test_sampler_frames_match_reference(name, sampler):
    """The oracle drawing with --use sampler=sobol (the scrambled Sobol
    sequence), sampler=sky_map (the sky aimed at by its chart) or
    sampler=each_lamp_first (the first four lamps' own lines at the first
    vertex) against the reference's own frames drawn so
    (tests/golden/image_<name>_<sampler>.npz, 16 seeds at 64 spp), to the
    bar of the other frame tests.  The Sobol sequence and the lamps' own
    lines do what they are for: the reference's frames' variance across
    seeds is below its plain frames'.  (The sky map does not on its scene:
    its smooth, bright sky is found as well by the BSDF's draws, and the
    reference's frames with the map vary 1.2x more than without.)"""
    sc = scene(name)
    ref = np.load(os.path.join(GOLDEN, f"image_{name}_{sampler}.npz"))
    frames = ref["frames"].astype(np.float64)
    spp = int(ref["spp"])
    h, w = sc.render["height"], sc.render["width"]
    build = dict(min_depth=5, max_depth=10, split_steps=64)
    got = np.stack([op.render_band(sc, w, h, spp, int(sc.render["surfaces"]), s, 0, h, os.cpu_count() or 4, build, **{sampler: True}) / spp
                    for s in range(1, 9)])
    z = (got.mean(0) - frames.mean(0)) / np.sqrt(got.var(0, ddof=1) / len(got) + frames.var(0, ddof=1) / len(frames) + 1e-12)
    ca, cb = got.mean(axis=(1, 2)), frames.mean(axis=(1, 2))
    cz = (ca.mean(0) - cb.mean(0)) / np.sqrt(ca.var(0, ddof=1) / len(ca) + cb.var(0, ddof=1) / len(cb))
    plain = np.load(os.path.join(GOLDEN, f"image_{name}.npz"))["frames"].astype(np.float64)
    gain = plain.var(0, ddof=1).mean() / frames.var(0, ddof=1).mean()
    print(f"{name} {sampler}: oracle {ca.mean(0)} reference {cb.mean(0)} z {cz} far px {(np.abs(z) > 3).mean():.4f}; variance gain over plain {gain:.2f}")
    assert np.all(np.abs(cz) < 4)
    assert (np.abs(z) > 3).mean() <= 0.015
    if sampler in ("sobol", "each_lamp_first"):
        assert gain > 1.0


def test_split_draws_the_same_frame_in_expectation():
    """render.split: groups of four samples sharing a first vertex (its
    camera ray, wavelengths and aim, the aim weighed as one of the group)
    draw the same frame in expectation as independent samples: the
    oracle's frames at splits 1 and 4 of the same scene agree within 4
    standard errors on every channel's mean."""
    import copy
    sc = scene("split_small")
    h, w = sc.render["height"], sc.render["width"]
    build = dict(min_depth=5, max_depth=10, split_steps=64)
    means = {}
    for split in (1, 4):
        s2 = copy.copy(sc)
        s2.render = dict(sc.render, split=split)
        frames = np.stack([op.render_band(s2, w, h, 64, int(sc.render["surfaces"]), k, 0, h, os.cpu_count() or 4, build) / 64 for k in range(1, 9)])
        m = frames.mean(axis=(1, 2))
        means[split] = (m.mean(0), m.var(0, ddof=1) / len(m))
    z = (means[4][0] - means[1][0]) / np.sqrt(means[4][1] + means[1][1])
    print(f"split 4 against 1: {means[4][0]} {means[1][0]} z {z}")
    assert np.all(np.abs(z) < 4)
