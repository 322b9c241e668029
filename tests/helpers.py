"""Shared test helpers: scenes, rays, and a host-only backend context."""
from __future__ import annotations

import ctypes
import os

import numpy as np

import kodanuki_gb300 as K
from kodanuki_gb300.scene import Scene

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def scene(name: str) -> Scene:
    return Scene.load(os.path.join(GOLDEN, "scenes", name + ".npz"))


def host_backend() -> K.Backend:
    """A context without a device (KDN_HOST_ONLY): blocks and the world build."""
    L = K.library()
    h = ctypes.c_void_p()
    assert L.kdn_open(-1, ctypes.byref(h)) == K.KDN_OK
    b = K.Backend.__new__(K.Backend)
    b.lib = L
    b.handle = h
    b.scene = None
    return b


def golden_rays(name: str):
    """The seeded rays of tests/golden/trace_<name>.npz, as kdn rays."""
    z = np.load(os.path.join(GOLDEN, f"trace_{name}.npz"))
    tr = {k: z[k] for k in z.files}
    r = tr["rays"]
    rays = np.zeros(len(r), K.RAY_DTYPE)
    rays["origin"] = r[:, 0:3]
    rays["direction"] = r[:, 3:6]
    rays["far"] = r[:, 6]
    rays["inside"] = r[:, 7] != 0
    rays["within"] = 0xFFFFFFFF
    return rays, tr


def step_digest(steps: np.ndarray) -> int:
    """The 64-bit FNV-1a digest tests/golden/make_golden.py keeps per cut program."""
    rec = np.zeros(len(steps), np.dtype([("op", "<u4"), ("a", "<u4"), ("b", "<u4"), ("c", "<u4"), ("v", "<u8"), ("leaf", "<u4")]))
    rec["op"], rec["a"], rec["b"], rec["c"] = steps["opcode"], steps["a"], steps["b"], steps["c"]
    rec["v"] = steps["value"].view("<u8")
    rec["leaf"] = steps["leaf"]
    h = 0xCBF29CE484222325
    for byte in rec.tobytes():
        h = ((h ^ byte) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h


def same_steps(a: np.ndarray, b: np.ndarray) -> bool:
    """Step arrays equal field by field, values to the bit."""
    if len(a) != len(b):
        return False
    for f in ("opcode", "a", "b", "c", "leaf"):
        if (a[f] != b[f]).any():
            return False
    return a["value"].view("<u8").tolist() == b["value"].view("<u8").tolist()


def compare_cells(cells_of, cut) -> int:
    """How many cells of a build (cells_of(i) -> (level, place, occupancy,
    [(object, result, steps)])) differ from a reference cut fixture."""
    cut = {k: cut[k] for k in cut.files} if hasattr(cut, "files") else cut
    offs = [0] + np.cumsum(cut["counts"]).astype(int).tolist()
    bad = 0
    pi = 0
    for i in range(len(cut["head"])):
        lvl, place, occ, progs = cells_of(i)
        if (lvl, *place, occ, len(progs)) != tuple(int(x) for x in cut["head"][i]):
            bad += 1
            pi += int(cut["head"][i][5])
            continue
        for obj, res, steps in progs:
            if "steps" in cut:
                same = same_steps(steps, cut["steps"][offs[pi]:offs[pi + 1]])
            else:
                same = len(steps) == int(cut["counts"][pi]) and step_digest(steps) == int(cut["digests"][pi])
            if obj != cut["objects"][pi] or res != cut["results"][pi] or not same:
                bad += 1
            pi += 1
    return bad
