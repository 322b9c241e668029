// kdn_world_march: the march form of a cell's kept programs, run on the host
// by the same interpreter the trace kernel runs (program.cuh).
#include "context.h"
#include "program.cuh"

#include <vector>

using kdn::Context;

extern "C" kdn_status kdn_world_march(kdn_ctx* handle, uint64_t i, const float* points, uint32_t n, float* values, size_t capacity, uint32_t* programs) {
	if (handle == nullptr || programs == nullptr || (n > 0 && (points == nullptr || values == nullptr))) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
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
