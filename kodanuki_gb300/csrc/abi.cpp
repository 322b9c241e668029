// The C ABI of libkdn_gb300 (include/kdn.h): context, blocks, world build
// and the geometry entry points.  The frame entry points are in render.cpp.
#include "context.h"

#include <cstring>
#include <new>

using kdn::Context;

namespace {

const char* const kStatusText[] = {
	"ok", "bad argument", "out of memory", "device loop reached its limit", "CUDA error", "not ready", "no usable CUDA device",
};

struct BlockSpec {
	const char* name;
	size_t size;
	bool single;
};

const BlockSpec kBlocks[] = {
	{ "scene.steps", sizeof(kdn_step), false },
	{ "scene.programs", sizeof(kdn_program_ref), false },
	{ "scene.leaves", sizeof(uint32_t), false },
	{ "looks.materials", sizeof(kdn_material), false },
	{ "transport.finishes", sizeof(kdn_finish), false },
	{ "lighting.lights", sizeof(kdn_light), false },
	{ "lighting.sky", sizeof(kdn_sky), true },
	{ "shot.camera", sizeof(kdn_camera), true },
	{ "geometry.region", sizeof(kdn_region), true },
	{ "looks.patterns", sizeof(kdn_pattern), false },
	{ "looks.pattern_steps", sizeof(kdn_step), false },
	{ "looks.pattern_arguments", sizeof(double), false },
	{ "looks.stops", sizeof(float), false },
	{ "looks.placements", sizeof(kdn_placement), false },
	{ "transport.boundaries", sizeof(kdn_boundary), false },
};
static_assert(sizeof(kdn_boundary) == 9112, "kdn_boundary is 9112 bytes");
static_assert(sizeof(kdn_pattern) == 32, "kdn_pattern is 32 bytes");
static_assert(sizeof(kdn_placement) == 96, "kdn_placement is 96 bytes");

static_assert(sizeof(kdn_step) == 32, "kdn_step is the reference's 32-byte Step");
static_assert(sizeof(kdn_ray) == 36, "kdn_ray is the reference's 36-byte Ray");
static_assert(sizeof(kdn_hit) == 56, "kdn_hit is the reference's 56-byte Hit");
static_assert(sizeof(kdn_program_ref) == 12, "kdn_program_ref is 12 bytes");
static_assert(sizeof(kdn_material) == 72, "kdn_material is 72 bytes");
static_assert(sizeof(kdn_light) == 136, "kdn_light is 136 bytes");
static_assert(sizeof(kdn_finish) == 352, "kdn_finish is 352 bytes");
static_assert(sizeof(kdn_sky) == 136, "kdn_sky is 136 bytes");
static_assert(sizeof(kdn_camera) == 96, "kdn_camera is 96 bytes");
static_assert(sizeof(kdn_region) == 48, "kdn_region is 48 bytes");

thread_local std::string openError;

} // namespace

namespace kdn {

void setThreadError(const std::string& message) { openError = message; }

} // namespace kdn

extern "C" {

const char* kdn_status_string(kdn_status status) {
	const int s = int(status);
	return s >= 0 && s < int(sizeof(kStatusText) / sizeof(kStatusText[0])) ? kStatusText[s] : "unknown status";
}

const char* kdn_last_error(const kdn_ctx* ctx) {
	if (ctx == nullptr) return openError.c_str();
	return reinterpret_cast<const Context*>(ctx)->error.c_str();
}

kdn_status kdn_open(int device, kdn_ctx** out) {
	if (out == nullptr) {
		openError = "kdn_open: null output";
		return KDN_BAD_ARG;
	}
	*out = nullptr;
	if (device == KDN_HOST_ONLY) {
		Context* ctx = new (std::nothrow) Context();
		if (ctx == nullptr) return KDN_OOM;
		ctx->device = -1;
		*out        = reinterpret_cast<kdn_ctx*>(ctx);
		return KDN_OK;
	}
	int count = 0;
	if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
		cudaGetLastError();
		openError = "kdn_open: no CUDA device";
		return KDN_NO_DEVICE;
	}
	if (device < 0 || device >= count) {
		openError = "kdn_open: device index out of range";
		return KDN_BAD_ARG;
	}
	Context* ctx = new (std::nothrow) Context();
	if (ctx == nullptr) return KDN_OOM;
	ctx->device      = device;
	const kdn_status s = ctx->open();
	if (s != KDN_OK) {
		openError = ctx->error;
		delete ctx;
		return s;
	}
	*out = reinterpret_cast<kdn_ctx*>(ctx);
	return KDN_OK;
}

kdn_status kdn_open_sharing(kdn_ctx* scene, int priority, kdn_ctx** out) {
	if (scene == nullptr || out == nullptr) return KDN_BAD_ARG;
	*out          = nullptr;
	Context* from = reinterpret_cast<Context*>(scene);
	std::lock_guard<std::mutex> guard(from->lock);
	if (!from->built) return from->fail(KDN_NOT_READY, "kdn_open_sharing: the scene has no world built (kdn_build)");
	if (from->source != nullptr) return from->fail(KDN_BAD_ARG, "kdn_open_sharing: the scene itself shares another context's world");
	Context* ctx = new (std::nothrow) Context();
	if (ctx == nullptr) return KDN_OOM;
	ctx->device   = from->device;
	ctx->priority = priority;
	if (ctx->device >= 0) {
		int least = 0, greatest = 0;
		cudaDeviceGetStreamPriorityRange(&least, &greatest);
		ctx->priority = std::min(std::max(priority, greatest), least);
		const kdn_status s = ctx->open();
		if (s != KDN_OK) {
			from->error = ctx->error;
			ctx->release();
			delete ctx;
			return s;
		}
	}
	ctx->share(from);
	*out = reinterpret_cast<kdn_ctx*>(ctx);
	return KDN_OK;
}

kdn_status kdn_set_frame_budget(kdn_ctx* handle, uint64_t bytes) {
	if (handle == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	ctx->frameBudget = bytes;
	return KDN_OK;
}

kdn_status kdn_set_march_budget(kdn_ctx* handle, uint32_t steps) {
	if (handle == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	ctx->marchBudget = steps >= kdn::kMarchSteps ? 0u : steps;
	return KDN_OK;
}

kdn_status kdn_set_guide(kdn_ctx* handle, kdn_guide* guide, float share, uint32_t flags) {
	if (handle == nullptr || (guide != nullptr && !(share > 0.0f && share < 1.0f)) || (flags & ~(KDN_GUIDE_SAMPLE | KDN_GUIDE_TRAIN)) != 0) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (guide != nullptr && kdn::guideDevice(guide) != ctx->device) return ctx->fail(KDN_BAD_ARG, "kdn_set_guide: the guide lives on another device");
	ctx->guide      = guide;
	ctx->guideShare = share;
	ctx->guideFlags = guide != nullptr ? flags : 0u;
	return KDN_OK;
}

kdn_status kdn_set_sm_limit(kdn_ctx* handle, int sms) {
	if (handle == nullptr || sms < 0) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->device >= 0) ctx->smCount = sms == 0 ? ctx->deviceSms : std::min(sms, ctx->deviceSms);
	return KDN_OK;
}

kdn_status kdn_close(kdn_ctx* handle) {
	if (handle == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	if (ctx->sharers.load() > 0) return ctx->fail(KDN_BAD_ARG, "kdn_close: other contexts still draw this one's world (close them first)");
	{
		std::lock_guard<std::mutex> guard(ctx->lock);
		ctx->release();
	}
	delete ctx;
	return KDN_OK;
}

kdn_status kdn_upload_block(kdn_ctx* handle, const char* name, const void* data, size_t count, size_t size) {
	if (handle == nullptr || name == nullptr || (data == nullptr && count > 0)) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	for (const BlockSpec& spec : kBlocks) {
		if (std::strcmp(spec.name, name) != 0) continue;
		if (size != spec.size) return ctx->fail(KDN_BAD_ARG, std::string("block ") + name + ": element size " + std::to_string(size) + ", expected " + std::to_string(spec.size));
		if (spec.single && count != 1) return ctx->fail(KDN_BAD_ARG, std::string("block ") + name + " holds exactly one element");
		std::vector<uint8_t>& block = ctx->blocks[name];
		block.assign(static_cast<const uint8_t*>(data), static_cast<const uint8_t*>(data) + count * size);
		if (std::strncmp(name, "scene.", 6) == 0 || std::strncmp(name, "geometry.", 9) == 0) ctx->built = false;
		ctx->sceneChanged = true;
		return KDN_OK;
	}
	return ctx->fail(KDN_BAD_ARG, std::string("unknown block name ") + name);
}

kdn_status kdn_build(kdn_ctx* handle, const kdn_build_options* options) {
	if (handle == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->sharers.load() > 0) return ctx->fail(KDN_BAD_ARG, "kdn_build: other contexts draw this one's world (close them first)");
	if (ctx->source != nullptr) return ctx->fail(KDN_BAD_ARG, "kdn_build: this context draws another's world");
	kdn::BuildOptions o;
	if (options != nullptr) {
		if (options->min_depth < 0 || options->max_depth < options->min_depth || options->max_depth > 24) return ctx->fail(KDN_BAD_ARG, "kdn_build: depths out of range");
		o.min_depth   = options->min_depth;
		o.max_depth   = options->max_depth;
		o.split_steps = options->split_steps;
	}
	return ctx->build(o);
}

kdn_status kdn_world_stats(kdn_ctx* handle, uint64_t out[4]) {
	if (handle == nullptr || out == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	if (ctx->source != nullptr) ctx = ctx->source; // a sharing context reads its scene's world
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (!ctx->built) return ctx->fail(KDN_NOT_READY, "kdn_world_stats: no world built");
	out[0] = ctx->octree.cells.size();
	out[1] = ctx->flat.leaves.size();
	out[2] = ctx->flat.programs.size();
	out[3] = ctx->flat.steps.size();
	return KDN_OK;
}

kdn_status kdn_world_cell(kdn_ctx* handle, uint64_t i, uint32_t head[6], uint32_t* objects, uint32_t* results, uint32_t* counts, kdn_step* steps, size_t capacity) {
	if (handle == nullptr || head == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	if (ctx->source != nullptr) ctx = ctx->source; // a sharing context reads its scene's world
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (!ctx->built) return ctx->fail(KDN_NOT_READY, "kdn_world_cell: no world built");
	const int64_t at = ctx->preorderCell(i);
	if (at < 0) return ctx->fail(KDN_BAD_ARG, "kdn_world_cell: cell index out of range");
	const kdn::Cell& c = ctx->octree.cells[size_t(at)];
	head[0] = c.level;
	head[1] = c.place[0];
	head[2] = c.place[1];
	head[3] = c.place[2];
	head[4] = c.occupancy;
	head[5] = uint32_t(c.programs.size());
	size_t used = 0;
	for (size_t k = 0; k < c.programs.size(); ++k) {
		const kdn::Prog& p = *c.programs[k];
		if (objects) objects[k] = p.object;
		if (results) results[k] = p.result;
		if (counts) counts[k] = uint32_t(p.steps.size());
		if (steps) {
			if (used + p.steps.size() > capacity) return ctx->fail(KDN_BAD_ARG, "kdn_world_cell: step buffer too small");
			std::memcpy(steps + used, p.steps.data(), p.steps.size() * sizeof(kdn_step));
		}
		used += p.steps.size();
	}
	return KDN_OK;
}

kdn_status kdn_extend_device(kdn_ctx* handle, const kdn_ray* rays, uint32_t n, kdn_hit* hits, void* stream) {
	if (handle == nullptr || (n > 0 && (rays == nullptr || hits == nullptr))) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->device < 0) return ctx->fail(KDN_NO_DEVICE, "kdn_extend_device: a host-only context has no device");
	return ctx->extend(rays, n, hits, stream ? static_cast<cudaStream_t>(stream) : ctx->stream);
}

kdn_status kdn_extend(kdn_ctx* handle, const kdn_ray* rays, uint32_t n, kdn_hit* hits) {
	if (handle == nullptr || (n > 0 && (rays == nullptr || hits == nullptr))) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->device < 0) return ctx->fail(KDN_NO_DEVICE, "kdn_extend: a host-only context has no device");
	if (n == 0) return KDN_OK;
	kdn_status s = ctx->ensure(ctx->extendRays, size_t(n) * sizeof(kdn_ray));
	if (s != KDN_OK) return s;
	s = ctx->ensure(ctx->extendHits, size_t(n) * sizeof(kdn_hit));
	if (s != KDN_OK) return s;
	if (!ctx->check(cudaMemcpyAsync(ctx->extendRays.ptr, rays, size_t(n) * sizeof(kdn_ray), cudaMemcpyHostToDevice, ctx->stream), "copy rays")) return KDN_CUDA_ERROR;
	s = ctx->extend(static_cast<const kdn_ray*>(ctx->extendRays.ptr), n, static_cast<kdn_hit*>(ctx->extendHits.ptr), ctx->stream);
	if (s != KDN_OK) return s;
	if (!ctx->check(cudaMemcpyAsync(hits, ctx->extendHits.ptr, size_t(n) * sizeof(kdn_hit), cudaMemcpyDeviceToHost, ctx->stream), "copy hits")) return KDN_CUDA_ERROR;
	if (!ctx->check(cudaStreamSynchronize(ctx->stream), "synchronise")) return KDN_CUDA_ERROR;
	return KDN_OK;
}

kdn_status kdn_flush_l2(kdn_ctx* handle) {
	if (handle == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->device < 0) return ctx->fail(KDN_NO_DEVICE, "kdn_flush_l2: a host-only context has no device");
	return ctx->flushL2();
}

} // extern "C"
