// kdn_world_march: the march form of a cell's kept programs, run on the host
// by the same interpreter the trace kernel runs (program.cuh).
#include "context.h"
#include "locate.cuh"
#include "program.cuh"

#include <vector>

using kdn::Context;

extern "C" kdn_status kdn_world_march(kdn_ctx* handle, uint64_t i, const float* points, uint32_t n, float* values, size_t capacity, uint32_t* programs) {
	if (handle == nullptr || programs == nullptr || (n > 0 && (points == nullptr || values == nullptr))) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	if (ctx->source != nullptr) ctx = ctx->source; // a sharing context reads its scene's world
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (!ctx->built) return ctx->fail(KDN_NOT_READY, "kdn_world_march: no world built");
	if (ctx->flat.nodes.empty()) return ctx->fail(KDN_NOT_READY, "kdn_world_march: no device layout: " + ctx->flatError);
	const int64_t c = ctx->preorderCell(i);
	if (c < 0) return ctx->fail(KDN_BAD_ARG, "kdn_world_march: no such cell");
	const int32_t node = ctx->flat.nodes[size_t(c)];
	if (node >= 0) {
		*programs = 0; // an inner cell keeps no programs
		return KDN_OK;
	}
	const kdn::GpuLeaf& leaf = ctx->flat.leaves[size_t(~node)];
	*programs                = leaf.count;
	if (size_t(leaf.count) * n > capacity) return ctx->fail(KDN_BAD_ARG, "kdn_world_march: values too small");
	std::vector<float> slots(kdn::kMaxSlots);
	kdn::setConstants(slots.data(), 1);
	for (uint32_t k = 0; k < leaf.count; ++k) {
		const kdn::GpuProgram& g = ctx->flat.programs[leaf.first + k];
		const kdn::MarchStep* code = ctx->flat.march.data() + g.march;
		for (uint32_t j = 0; j < n; ++j) values[size_t(k) * n + j] = kdn::evalSlots(code, g.marchCount, g.marchSlot, slots.data(), 1, points + 3 * size_t(j));
	}
	return KDN_OK;
}

// kdn_world_locate: the leaf of each point by the trace kernel's locate()
// (grid, then descent) and by the descent from the root, on the host.
extern "C" kdn_status kdn_world_locate(kdn_ctx* handle, const float* points, uint32_t n, uint32_t* by_grid, uint32_t* by_descent) {
	if (handle == nullptr || (n > 0 && (points == nullptr || by_grid == nullptr || by_descent == nullptr))) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	if (ctx->source != nullptr) ctx = ctx->source; // a sharing context reads its scene's world
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (!ctx->built) return ctx->fail(KDN_NOT_READY, "kdn_world_locate: no world built");
	if (ctx->flat.nodes.empty()) return ctx->fail(KDN_NOT_READY, "kdn_world_locate: no device layout: " + ctx->flatError);
	kdn::DeviceWorld w {};
	w.nodes     = ctx->flat.nodes.data();
	w.grid      = ctx->gridCells.data();
	w.gridWalls = ctx->walls.data();
	w.gridLevel = kdn::kGridLevel;
	for (int a = 0; a < 3; ++a) {
		w.lower[a]     = ctx->lowerF[a];
		w.size[a]      = ctx->sizeF[a];
		w.gridScale[a] = float(double(1u << kdn::kGridLevel) / double(w.size[a]));
	}
	for (uint32_t j = 0; j < n; ++j) {
		by_grid[j]    = kdn::locate(w, points + 3 * size_t(j)).leaf;
		by_descent[j] = kdn::descendFromRoot(w, points + 3 * size_t(j));
	}
	return KDN_OK;
}
