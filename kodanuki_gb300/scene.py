"""A compiled scene as the blocks the backend consumes.

A scene is what the reference renderer's loader leaves behind
(syntax/evaluator.cpp:2898 loadScene): the object programs
(sdf/scene.cpp:290 objectPrograms, one straight-line program per object),
the material of each leaf, the materials, the lights, the sky, the camera,
the render settings and the region the geometry is built over
(plugins/geometry/tree/build.cpp:405 sceneRegion).  It is stored as one
``.npz`` of plain arrays; ``steps`` uses the reference's ``Step`` layout
(sdf/program.h:56: opcode, a, b, c, value, leaf).
"""
from __future__ import annotations

import dataclasses
import json

import numpy as np

STEP_DTYPE = np.dtype([("opcode", "u1"), ("a", "<u4"), ("b", "<u4"), ("c", "<u4"), ("value", "<f8"), ("leaf", "<u4")], align=True)

# material/energy.h Boundary: 17 index ratios x 32 views, twice, then three
# rows of 17.
BOUNDARY_RATIOS, ENERGY_VIEWS = 17, 32
BOUNDARY_DOUBLES = 2 * BOUNDARY_RATIOS * ENERGY_VIEWS + 3 * BOUNDARY_RATIOS

# sdf/scene.h MaterialKind and LightKind, in the reference's order.
MATTE, PLASTIC, METAL, GLASS, MEDIUM = range(5)
POINT, DIRECTIONAL, SPHERE, QUAD, SUN, MOON = range(6)


@dataclasses.dataclass
class Scene:
    steps: np.ndarray            # STEP_DTYPE, every program end to end
    program_first: np.ndarray    # u32 [P+1]
    program_result: np.ndarray   # u32 [P]
    leaf_material: np.ndarray    # u32 [L]
    materials: dict              # name -> array over materials
    lights: dict                 # name -> array over lights
    sky: dict
    camera: dict
    render: dict
    region_lower: np.ndarray     # f64 [3]
    region_size: np.ndarray      # f64 [3]
    # sdf/scene.h Placement of each leaf, f64 [L, 12]: linear row by row,
    # then origin (what a pattern read in the painted shape's space uses)
    leaf_placement: np.ndarray | None = None
    # sdf/scene.h Albedo over the materials, end to end: the pattern
    # programs' steps (first/result per material, count 0 for a flat
    # colour), the arguments they read, the ramps' stops (3 floats a stop)
    # and whether each is read in world space
    patterns: dict = dataclasses.field(default_factory=dict)

    @property
    def program_count(self) -> int:
        return int(self.program_result.shape[0])

    def program(self, i: int) -> tuple[np.ndarray, int]:
        return self.steps[self.program_first[i]:self.program_first[i + 1]], int(self.program_result[i])

    def save(self, path: str) -> None:
        # the steps field by field: a column of opcodes, of operands, of
        # values compresses far better than the interleaved records
        arrays = {f"steps_{f}": np.ascontiguousarray(self.steps[f]) for f in STEP_DTYPE.names}
        arrays.update({
            "program_first": self.program_first,
            "program_result": self.program_result,
            "leaf_material": self.leaf_material,
            "region_lower": self.region_lower,
            "region_size": self.region_size,
        })
        for k, v in self.materials.items():
            arrays["material_" + k] = v
        for k, v in self.lights.items():
            arrays["light_" + k] = v
        if self.leaf_placement is not None:
            arrays["leaf_placement"] = self.leaf_placement
        for k, v in self.patterns.items():
            arrays["pattern_" + k] = v
        arrays["meta"] = np.frombuffer(json.dumps({"sky": self.sky, "camera": self.camera, "render": self.render}).encode(), np.uint8)
        np.savez_compressed(path, **arrays)

    @staticmethod
    def load(path: str) -> "Scene":
        z = np.load(path)
        meta = json.loads(bytes(z["meta"]).decode())
        mats = {k[len("material_"):]: z[k] for k in z.files if k.startswith("material_")}
        lights = {k[len("light_"):]: z[k] for k in z.files if k.startswith("light_")}
        patterns = {k[len("pattern_"):]: z[k] for k in z.files if k.startswith("pattern_")}
        placement = z["leaf_placement"] if "leaf_placement" in z.files else None
        if "steps" in z.files:
            steps = z["steps"]
        else:
            steps = np.zeros(len(z["steps_opcode"]), STEP_DTYPE)
            for f in STEP_DTYPE.names:
                steps[f] = z[f"steps_{f}"]
        return Scene(steps, z["program_first"], z["program_result"], z["leaf_material"], mats, lights,
                     meta["sky"], meta["camera"], meta["render"], z["region_lower"], z["region_size"], placement, patterns)

    @staticmethod
    def from_reference_json(d: dict) -> "Scene":
        """Convert the exporter's JSON (oracle/ref/ref_dump.cpp ``scene``)."""
        rows, first, result = [], [0], []
        for p in d["programs"]:
            rows.extend(tuple(s) for s in p["steps"])
            first.append(len(rows))
            result.append(p["result"])
        steps = np.zeros(len(rows), STEP_DTYPE)
        if rows:
            arr = np.array(rows, dtype=object)
            steps["opcode"] = arr[:, 0].astype(np.uint8)
            steps["a"] = arr[:, 1].astype(np.uint32)
            steps["b"] = arr[:, 2].astype(np.uint32)
            steps["c"] = arr[:, 3].astype(np.uint32)
            steps["value"] = arr[:, 4].astype(np.float64)
            steps["leaf"] = arr[:, 5].astype(np.uint32)
        ms = d["materials"]
        mats = {
            "kind": np.array([m["kind"] for m in ms], np.uint8),
            "albedo": np.array([(m["stops"] + [0, 0, 0])[:3] for m in ms], np.float32),
            "patterned": np.array([m["pattern"] >= 0 for m in ms], np.uint8),
            "roughness": np.array([m["roughness"] for m in ms], np.float32),
            "refraction": np.array([m["refraction"] for m in ms], np.float32),
            "dispersion": np.array([m["dispersion"] for m in ms], np.float32),
            "absorb": np.array([m["absorb"] for m in ms], np.float64).reshape(-1, 3),
            "glow": np.array([m["glow"] for m in ms], np.float64).reshape(-1, 3),
            "strength": np.array([m["strength"] for m in ms], np.float32),
            "scatter": np.array([m.get("scatter", 0) for m in ms], np.float32),
            "lean": np.array([m.get("lean", 0) for m in ms], np.float32),
        }
        fs = d.get("finishes", [])
        if fs:
            mats.update({
                "finish_kind": np.array([f["kind"] for f in fs], np.uint32),
                "finish_sharp": np.array([f["sharp"] for f in fs], np.uint32),
                "finish_exact": np.array([f["exact"] for f in fs], np.uint32),
                "finish_loses_much": np.array([f["losesMuch"] for f in fs], np.uint32),
                "finish_width": np.array([f["width"] for f in fs], np.float64),
                "finish_facet_share": np.array([f["facetShare"] for f in fs], np.float64),
                "finish_body": np.array([f["body"] for f in fs], np.float64),
                "finish_index": np.array([f["index"] for f in fs], np.float64),
                "finish_coating": np.array([f["coating"] for f in fs], np.float64).reshape(-1, 3),
                "finish_escape_average": np.array([f["escapeAverage"] for f in fs], np.float64),
                "finish_escape": np.array([f["escape"] for f in fs], np.float64).reshape(-1, 32),
                "finish_film": np.array([f["film"] for f in fs], np.float64).reshape(-1, 2),
                # material/energy.h Boundary of each glass (zeros elsewhere):
                # rarer and denser (17 ratios x 32 views each), then the
                # rarer and denser averages and the rarer-through shares
                "finish_boundary": np.array([f.get("boundary", [0.0] * BOUNDARY_DOUBLES) for f in fs], np.float64).reshape(-1, BOUNDARY_DOUBLES),
            })
        # the patterns (ref_dump.cpp writes them with each material)
        pat_rows, pat_first, pat_result, args, arg_first, stops, stop_first = [], [0], [], [], [0], [], [0]
        for m in ms:
            for srow in m.get("patternSteps", []):
                pat_rows.append(tuple(srow))
            pat_first.append(len(pat_rows))
            pat_result.append(m.get("patternResult", 0))
            args.extend(m.get("patternArguments", []))
            arg_first.append(len(args))
            stops.extend(m["stops"])
            stop_first.append(len(stops) // 3)
        pat_steps = np.zeros(len(pat_rows), STEP_DTYPE)
        if pat_rows:
            arr = np.array(pat_rows, dtype=object)
            for i, k in enumerate(("opcode", "a", "b", "c", "value", "leaf")):
                pat_steps[k] = arr[:, i].astype(pat_steps.dtype[k])
        patterns = {
            "steps": pat_steps, "first": np.array(pat_first, np.uint32), "result": np.array(pat_result, np.uint32),
            "arguments": np.array(args, np.float64), "argument_first": np.array(arg_first, np.uint32),
            "stops": np.array(stops, np.float32).reshape(-1, 3), "stop_first": np.array(stop_first, np.uint32),
            "world": np.array([m.get("world", 0) for m in ms], np.uint8),
        }
        placement = np.array(d["placements"], np.float64).reshape(-1, 12) if "placements" in d else None
        ls = d["lights"]
        lights = {
            "kind": np.array([l["kind"] for l in ls], np.uint8),
            "at": np.array([l["at"] for l in ls], np.float64).reshape(-1, 3),
            "direction": np.array([l["direction"] for l in ls], np.float64).reshape(-1, 3),
            "along": np.array([l["along"] for l in ls], np.float64).reshape(-1, 3),
            "across": np.array([l["across"] for l in ls], np.float64).reshape(-1, 3),
            "radius": np.array([l["radius"] for l in ls], np.float32),
            "angle": np.array([l["angle"] for l in ls], np.float32),
            "power": np.array([l["power"] for l in ls], np.float64).reshape(-1, 3),
        }
        return Scene(steps, np.array(first, np.uint32), np.array(result, np.uint32), np.array(d["leaves"], np.uint32),
                     mats, lights, d["sky"], d["camera"], d["render"],
                     np.array(d["region"]["lower"], np.float64), np.array(d["region"]["size"], np.float64), placement, patterns)
