"""The C ABI library: it loads, exports what include/kdn.h declares, checks
its arguments, and its host-side world build cuts cells exactly as the
reference's cutCell does (no device needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

import kodanuki_gb300 as K
from helpers import GOLDEN, compare_cells, host_backend, scene

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    text = open(os.path.join(ROOT, "include", "kdn.h")).read()
    return sorted(set(re.findall(r"\b(kdn_[a-z_0-9]+)\s*\(", text)))


def test_exports_every_declared_symbol():
    L = K.library()
    names = declared()
    assert len(names) >= 14
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(K.EXPORTS)


def test_status_strings():
    L = K.library()
    assert L.kdn_status_string(0) == b"ok"
    assert L.kdn_status_string(99) == b"unknown status"


def test_block_checks():
    b = host_backend()
    with pytest.raises(K.KdnError) as e:
        b.upload("scene.nothing", np.zeros(4, np.uint32))
    assert e.value.status == K.KDN_BAD_ARG
    with pytest.raises(K.KdnError) as e:
        b.upload("scene.leaves", np.zeros(4, np.uint64))
    assert e.value.status == K.KDN_BAD_ARG
    with pytest.raises(K.KdnError) as e:
        b.upload("shot.camera", np.zeros(2, K.CAMERA_DTYPE))
    assert e.value.status == K.KDN_BAD_ARG
    with pytest.raises(K.KdnError) as e:
        b.build()
    assert e.value.status == K.KDN_NOT_READY
    b.close()


def test_pattern_blocks():
    """A scene with patterned albedos carries the looks.patterns,
    pattern_steps, pattern_arguments, stops and placements blocks, each
    with the reference's element size."""
    b = host_backend()
    sc = scene("patterns_small")
    blocks = K.scene_blocks(sc)
    for name in ("looks.patterns", "looks.pattern_steps", "looks.pattern_arguments", "looks.stops", "looks.placements"):
        assert name in blocks
    assert blocks["looks.patterns"].dtype.itemsize == 32
    assert blocks["looks.placements"].dtype.itemsize == 96
    pats = blocks["looks.patterns"]
    patterned = np.asarray(sc.materials["patterned"]) != 0
    assert np.all((pats["count"] > 0) == patterned)
    assert np.all(pats["count"][patterned] <= 64)
    assert len(blocks["looks.placements"]) == len(sc.leaf_material)
    b.load(sc)
    with pytest.raises(K.KdnError) as e:
        b.upload("looks.patterns", np.zeros(4, np.uint32))
    assert e.value.status == K.KDN_BAD_ARG
    with pytest.raises(K.KdnError) as e:
        b.upload("looks.placements", np.zeros((2, 12), np.float32))
    assert e.value.status == K.KDN_BAD_ARG
    b.close()


def test_bad_program_is_refused():
    b = host_backend()
    sc = scene("c1")
    b.load(sc)
    bad = sc.steps.copy()
    k = int(np.nonzero(bad["opcode"] >= 8)[0][0])
    bad["a"][k] = 10_000  # a step reading a later step
    b.upload("scene.steps", bad)
    with pytest.raises(K.KdnError) as e:
        b.build()
    assert e.value.status == K.KDN_BAD_ARG
    b.close()


def test_host_only_context_has_no_device_entry_points():
    b = host_backend()
    b.load(scene("c1"))
    b.build(4, 4, 1 << 30)
    with pytest.raises(K.KdnError) as e:
        b.extend(np.zeros(4, K.RAY_DTYPE))
    assert e.value.status == K.KDN_NO_DEVICE
    b.close()


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_world_build_matches_reference_cut(name):
    cut = np.load(os.path.join(GOLDEN, f"cut_{name}.npz"))
    d = int(cut["depth"])
    b = host_backend()
    b.load(scene(name))
    b.build(d, d, 1 << 30)
    assert b.world_stats()["cells"] == len(cut["head"])
    assert compare_cells(b.world_cell, cut) == 0
    b.close()


def test_bench_world_cells_match_reference_cut():
    """The octree the benchmark builds over config 2 (levels 7 to 11, split
    while a cell's programs pass 32 steps): a seeded sample of its cells,
    every level down to 11, holds exactly the programs the reference's
    cutCell gives those cells when cut from the root along their paths
    (tests/golden/cutdeep_c2.npz)."""
    fx = np.load(os.path.join(GOLDEN, "cutdeep_c2.npz"))
    b = host_backend()
    b.load(scene("c2"))
    b.build(*[int(x) for x in fx["build"]])
    index = fx["index"]
    assert compare_cells(lambda k: b.world_cell(int(index[k])), fx) == 0
    assert int(fx["head"][:, 0].max()) == 11
    b.close()


def test_world_build_matches_oracle_adaptive():
    """The adaptive build (split while a cell's programs are long) agrees
    with the oracle's build cell for cell."""
    import oracle.port as op
    sc = scene("c1")
    b = host_backend()
    b.load(sc)
    b.build(5, 9, 96)
    tree = op.Octree(sc, 5, 9, 96)
    n = tree.cells()
    assert b.world_stats()["cells"] == n
    from helpers import same_steps
    for i in range(0, n, max(1, n // 400)):
        l1, p1, o1, g1 = b.world_cell(i)
        l2, p2, o2, g2 = tree.cell(i)
        assert (l1, p1, o1, len(g1)) == (l2, p2, o2, len(g2))
        for (a1, r1, s1), (a2, r2, s2) in zip(g1, g2):
            assert a1 == a2 and r1 == r2 and same_steps(s1, s2)
    b.close()
