"""The march form the trace kernel runs, checked on the host.

The host build lays every kept program out as the device reads it (register
slots, immediates, operands forwarded from the step before, the common
operations renumbered) and kdn_world_march runs it through the same
interpreter the kernel runs (kodanuki_gb300/csrc/program.cuh).  Here that is
compared, at random points of random cells, with a plain double evaluation
of the cell's kept programs in the reference's own Step form
(sdf/program.cpp:57 runStep): the two must agree to FP32 rounding.
"""
import numpy as np
import pytest

from helpers import host_backend, scene

# sdf/program.h:20 opcodes
(CONSTANT, ARGUMENT, PX, PY, PZ, NX, NY, NZ, ADD, SUB, MUL, DIV, NEG, SQRT, ABS, FLOOR, SIN, COS, SIGN, ATAN2, POW, MIN, MAX, SMIN, POSSQ,
 LESS, LESSEQ, EQUAL, NOTEQUAL, AND, OR, NOT, SELECT) = range(33)


def evaluate(steps: np.ndarray, result: int, p: np.ndarray) -> np.ndarray:
    """A Step program at points p (n x 3), in double, step by step."""
    v = []
    for s in steps:
        op, a, b, c = int(s["opcode"]), int(s["a"]), int(s["b"]), int(s["c"])
        A = v[a] if a < len(v) else None
        B = v[b] if b < len(v) else None
        C = v[c] if c < len(v) else None
        if op == CONSTANT:
            r = np.full(len(p), float(s["value"]))
        elif op in (ARGUMENT, NX, NY, NZ):
            r = np.zeros(len(p))
        elif op in (PX, PY, PZ):
            r = p[:, op - PX].astype(np.float64)
        elif op == ADD:
            r = A + B
        elif op == SUB:
            r = A - B
        elif op == MUL:
            r = A * B
        elif op == DIV:
            r = A / B
        elif op == NEG:
            r = -A
        elif op == SQRT:
            r = np.sqrt(A)
        elif op == ABS:
            r = np.abs(A)
        elif op == FLOOR:
            r = np.floor(A)
        elif op == SIN:
            r = np.sin(A)
        elif op == COS:
            r = np.cos(A)
        elif op == SIGN:
            r = np.sign(A)
        elif op == ATAN2:
            r = np.arctan2(A, B)
        elif op == POW:
            r = np.power(A, B)
        elif op == MIN:
            r = np.where(B < A, B, A)
        elif op == MAX:
            r = np.where(A < B, B, A)
        elif op == SMIN:
            blend = np.maximum(C - np.abs(A - B), 0.0) / C
            r = np.minimum(A, B) - blend * blend * C * 0.25
        elif op == POSSQ:
            q = np.maximum(A, 0.0)
            r = q * q
        elif op == LESS:
            r = (A < B).astype(float)
        elif op == LESSEQ:
            r = (A <= B).astype(float)
        elif op == EQUAL:
            r = (A == B).astype(float)
        elif op == NOTEQUAL:
            r = (A != B).astype(float)
        elif op == AND:
            r = ((A != 0) & (B != 0)).astype(float)
        elif op == OR:
            r = ((A != 0) | (B != 0)).astype(float)
        elif op == NOT:
            r = (A == 0).astype(float)
        elif op == SELECT:
            r = np.where(A != 0, B, C)
        else:
            raise ValueError(op)
        v.append(r)
    return v[result]


@pytest.mark.parametrize("name,build", [("c2", (7, 10, 96)), ("c1", (6, 9, 64)), ("room", (5, 8, 64))])
def test_march_form_matches_programs(name, build):
    sc = scene(name)
    b = host_backend()
    try:
        b.load(sc)
        b.build(*build)
        cells = b.world_stats()["cells"]
        rng = np.random.default_rng(7)
        lower = np.asarray(sc.region_lower, np.float64)
        size = np.asarray(sc.region_size, np.float64)
        checked = steps_checked = 0
        worst = 0.0
        for i in rng.permutation(cells)[:4000]:
            level, (x, y, z), occupancy, progs = b.world_cell(int(i))
            if not progs:
                continue
            side = size / (1 << level)
            corner = lower + side * np.array([x, y, z])
            pts = (corner + side * rng.random((16, 3))).astype(np.float32)
            got = b.world_march(int(i), pts)
            if got.shape[0] == 0:
                continue  # an inner cell: the march reads leaves alone
            assert got.shape == (len(progs), 16)
            for k, (obj, res, steps) in enumerate(progs):
                want = evaluate(steps, int(res), pts.astype(np.float64))
                err = np.abs(got[k].astype(np.float64) - want) / (1.0 + np.abs(want))
                worst = max(worst, float(err.max()))
                steps_checked += len(steps)
            checked += 1
            if checked >= 300:
                break
        print(f"{name}: {checked} cells, {steps_checked} steps, worst relative error {worst:.2e}")
        assert checked >= 50
        assert worst <= 2e-5
    finally:
        b.close()


@pytest.mark.parametrize("name,build", [("c2", (7, 11, 32)), ("room", (5, 8, 64))])
def test_grid_locate_matches_descent(name, build):
    """The trace kernel's locate (a grid of the octree's level 6 set right
    against its walls, then the descent) names the leaf the descent from the
    root names, for points anywhere, on cell walls and outside the region."""
    sc = scene(name)
    b = host_backend()
    try:
        b.load(sc)
        b.build(*build)
        rng = np.random.default_rng(11)
        lower = np.asarray(sc.region_lower, np.float32)
        size = np.asarray(sc.region_size, np.float32)
        inside = lower + size * rng.random((20000, 3)).astype(np.float32)
        # points on the walls of every level: the descent's own midpoints
        walls = []
        for level in range(1, 12):
            k = rng.integers(0, 1 << level, (2000, 3))
            w = lower.astype(np.float64) + size.astype(np.float64) * k / (1 << level)
            walls.append(w.astype(np.float32))
        outside = lower + size * (rng.random((2000, 3)).astype(np.float32) * 1.4 - 0.2)
        pts = np.concatenate([inside] + walls + [outside])
        by_grid, by_descent = b.world_locate(pts)
        assert np.array_equal(by_grid, by_descent)
    finally:
        b.close()
