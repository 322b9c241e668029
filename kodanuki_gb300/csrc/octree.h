// Host build of the cut octree and its flattening into the device layout.
#pragma once

#include "kdn.h"
#include "world.h"

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace kdn {

// A program as the reference keeps one (sdf/program.h:62 Program): steps in
// SSA order and the result, plus the object it was cut from.
struct Prog {
	std::vector<kdn_step> steps;
	uint32_t result = 0;
	uint32_t object = 0;
};
using ProgPtr = std::shared_ptr<const Prog>;

struct Cell {
	uint8_t occupancy   = Empty;
	uint32_t level      = 0;
	uint32_t place[3]   = { 0, 0, 0 };
	int64_t firstChild  = -1;
	std::vector<ProgPtr> programs; // kept programs (cut.cpp CellPrograms)
};

struct Octree {
	double lower[3] = { 0, 0, 0 };
	double size[3]  = { 0, 0, 0 };
	std::vector<Cell> cells; // children of a cell contiguous, root first
};

struct BuildOptions {
	int min_depth        = 6;
	int max_depth        = 10;
	uint32_t split_steps = 96;
	size_t max_cells     = size_t(1) << 26;
};

struct FlatWorld {
	std::vector<int32_t> nodes;
	std::vector<GpuLeaf> leaves;
	std::vector<GpuProgram> programs; // one run per leaf
	std::vector<GpuStep> steps;
	std::vector<SsaOps> ssa;
	std::vector<MarchStep> march; // the march form (world.h MarchStep)
};

// Returns an empty string, or what went wrong.
std::string buildOctree(const std::vector<ProgPtr>& objects, const double lower[3], const double size[3], const BuildOptions& options, Octree& tree);
std::string flattenOctree(const Octree& tree, FlatWorld& flat);
// The grid of `level` over a flattened octree (world.h GridCell).
std::vector<GridCell> gridOf(const FlatWorld& flat, uint32_t level);
// The walls of that grid per axis (3 x (2^level + 1)): the descent's
// midpoints in FP32 over [lower, lower + size].
std::vector<float> gridWallsOf(const float lower[3], const float size[3], uint32_t level);

} // namespace kdn
