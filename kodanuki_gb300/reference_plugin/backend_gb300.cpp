// backend/gb300: the binding a maintainer of the reference renderer adds to
// its source tree (source/plugins/backend/gb300/) so that the renderer's
// ExtendRays step runs on this library's GB300 sphere trace.  It fills the
// reference's Backend point (core/plugin.h:333-357, core/worker.h:41 Crew)
// the way backend/cpu does (plugins/backend/cpu/plugin.cpp:13-36), and its
// ExtendRays follows execution/single (plugins/execution/single/plugin.cpp:
// 28-36): every slot of the worker's pool that waits on a ray
// (core/batch.h:360 waitsOnRay) gets its first hit and is marked answered;
// the other steps go to the fallback (core/step.cpp:47 ranKernel).
//
// The world: the scene's object programs (sdf/scene.cpp:290 objectPrograms),
// each leaf's material and the region the reference's tree is built over
// (plugins/geometry/tree/build.cpp:405 sceneRegion) are uploaded as this
// library's blocks (include/kdn.h) and built into the cut octree once per
// scene; a frame of another scene builds it again.  The device's hits are
// the reference's Hit byte for byte; like the reference's sphere-traced
// hits (sphere_trace.cpp:150 sphereHit) they carry no tree cell.
//
// Errors print and exit (the reference's rule 19).  With the environment
// variable KDN_GB300_HOST_ONLY=1 the plugin opens a context without a
// device: it uploads and builds the world (so a machine without a GPU can
// check the binding) and, owning no kernel there, hands every step to the
// fallback, as the reference's own contract test's backend does
// (target/tests/generic.cpp:213-247).
#include "core/batch.h"
#include "core/block.h"
#include "core/geometry.h"
#include "core/plugin.h"
#include "core/render.h"
#include "core/step.h"
#include "core/worker.h"
#include "plugins/geometry/tree/build.h"
#include "sdf/program.h"
#include "sdf/scene.h"

#include "kdn.h"

#include <array>
#include <atomic>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace kodanuki {

static_assert(sizeof(Ray) == sizeof(kdn_ray) && offsetof(Ray, far) == offsetof(kdn_ray, far) && offsetof(Ray, within) == offsetof(kdn_ray, within),
              "kdn_ray is core/batch.h Ray byte for byte");
static_assert(sizeof(Hit) == sizeof(kdn_hit) && offsetof(Hit, cell) == offsetof(kdn_hit, cell) && offsetof(Hit, leafKind) == offsetof(kdn_hit, leaf_kind),
              "kdn_hit is core/batch.h Hit byte for byte");
static_assert(sizeof(Step) == sizeof(kdn_step), "kdn_step is sdf/program.h Step byte for byte");

namespace {

struct Gb300State {
	kdn_ctx* context = nullptr;
	bool device      = false;
	std::mutex opening;
	std::uint64_t built = 0; // the digest of the scene the world was built for (0: none)
	std::atomic<std::uint64_t> steps { 0 };
	std::atomic<int> blocks { 0 };
	std::array<std::atomic<std::uint64_t>, rayKindCount> rays {};
};

// The plugin's state, reached only through this accessor (reference rule 54).
Gb300State& gb300() {
	static Gb300State state;
	return state;
}

void gb300Check(kdn_status status, const char* what) {
	if (status != KDN_OK) {
		std::fprintf(stderr, "backend/gb300: %s: %s: %s\n", what, kdn_status_string(status), kdn_last_error(gb300().context));
		std::exit(1);
	}
}

// 64-bit FNV-1a over the object programs' steps and the leaves' materials:
// a frame of an unchanged scene keeps the built world.
std::uint64_t sceneDigest(const Scene& scene) {
	std::uint64_t h = 0xCBF29CE484222325ull;
	const auto mix  = [&](const void* data, std::size_t bytes) {
		const auto* p = static_cast<const unsigned char*>(data);
		for (std::size_t i = 0; i < bytes; ++i) h = (h ^ p[i]) * 0x100000001B3ull;
	};
	for (const Program& program : scene.objectPrograms) {
		mix(program.steps.data(), program.steps.size() * sizeof(Step));
		mix(&program.result, sizeof program.result);
	}
	for (const Leaf& leaf : scene.leaves) mix(&leaf.material, sizeof leaf.material);
	return h == 0 ? 1 : h;
}

void uploadWorld(const Renderer& renderer) {
	const Scene& scene = renderer.file.scene;
	std::vector<kdn_step> steps;
	std::vector<kdn_program_ref> programs;
	for (const Program& program : scene.objectPrograms) {
		programs.push_back(kdn_program_ref { std::uint32_t(steps.size()), std::uint32_t(program.steps.size()), program.result });
		for (const Step& step : program.steps) {
			kdn_step s;
			std::memcpy(&s, &step, sizeof s);
			steps.push_back(s);
		}
	}
	std::vector<std::uint32_t> leaves;
	for (const Leaf& leaf : scene.leaves) leaves.push_back(leaf.material);
	const Region region = sceneRegion(scene, renderer.file.shot, renderer.options.choices.threads);
	kdn_region box {};
	for (int a = 0; a < 3; ++a) {
		box.lower[a] = region.lower[a];
		box.size[a]  = region.size[a];
	}
	kdn_ctx* ctx = gb300().context;
	gb300Check(kdn_upload_block(ctx, "scene.steps", steps.data(), steps.size(), sizeof(kdn_step)), "scene.steps");
	gb300Check(kdn_upload_block(ctx, "scene.programs", programs.data(), programs.size(), sizeof(kdn_program_ref)), "scene.programs");
	gb300Check(kdn_upload_block(ctx, "scene.leaves", leaves.data(), leaves.size(), sizeof(std::uint32_t)), "scene.leaves");
	gb300Check(kdn_upload_block(ctx, "geometry.region", &box, 1, sizeof box), "geometry.region");
	// --depth caps the octree as it caps the reference's tree (core/options.cpp:346)
	const int depth               = renderer.options.choices.depth;
	const kdn_build_options build = { depth > 0 ? std::min(depth, 6) : 6, depth > 0 ? depth : 11, 64, 0 };
	gb300Check(kdn_build(ctx, &build), "kdn_build");
}

// The frame's blocks that hold data (core/block.cpp:16 frameBlocks): the
// transport's finishes, lamps and sky, and the Geometry plugin's arrays.
int heldBlocks(const Renderer& renderer) {
	int held = 0;
	for (const Block& block : frameBlocks(renderer)) held += block.count > 0 && block.data != nullptr && block.size > 0 && block.name.find('.') != std::string::npos ? 1 : 0;
	return held;
}

Crew gb300Workers(const Renderer& renderer) {
	Gb300State& g = gb300();
	{
		std::lock_guard<std::mutex> guard(g.opening);
		if (g.context == nullptr) {
			const char* hostOnly = std::getenv("KDN_GB300_HOST_ONLY");
			g.device             = !(hostOnly != nullptr && std::strcmp(hostOnly, "1") == 0);
			gb300Check(kdn_open(g.device ? 0 : KDN_HOST_ONLY, &g.context), "kdn_open");
		}
		const std::uint64_t digest = sceneDigest(renderer.file.scene);
		if (digest != g.built) {
			uploadWorld(renderer);
			g.built = digest;
		}
		g.blocks = std::max(g.blocks.load(), heldBlocks(renderer));
	}
	return Crew {
		.workers  = renderer.options.choices.threads,
		.capacity = poolCapacity,
	};
}

bool gb300Ran(const Renderer&, Worker& worker, const Plugin&, LoopStep step) {
	Gb300State& g = gb300();
	g.steps += 1;
	if (step != LoopStep::ExtendRays || !g.device) return false;
	Pool& pool = worker.pool;
	thread_local std::vector<kdn_ray> rays;
	thread_local std::vector<kdn_hit> hits;
	thread_local std::vector<std::uint32_t> slots;
	rays.clear();
	slots.clear();
	for (std::size_t slot = 0; slot < std::size_t(pool.capacity); ++slot) {
		if (!waitsOnRay(pool.phases[slot])) continue;
		kdn_ray r;
		std::memcpy(&r, &pool.rays[slot], sizeof r);
		rays.push_back(r);
		slots.push_back(std::uint32_t(slot));
	}
	hits.resize(rays.size());
	gb300Check(kdn_extend(g.context, rays.data(), std::uint32_t(rays.size()), hits.data()), "kdn_extend");
	std::array<std::uint64_t, rayKindCount> extended = {};
	for (std::size_t k = 0; k < slots.size(); ++k) {
		const std::uint32_t slot = slots[k];
		hits[k].cell             = noLeaf; // no tree cell, as a sphere-traced hit
		std::memcpy(&pool.hits[slot], &hits[k], sizeof(Hit));
		pool.answered[slot] = 1;
		extended[std::size_t(pool.kinds[slot])] += 1;
	}
	for (std::size_t kind = 0; kind < extended.size(); ++kind) g.rays[kind].fetch_add(extended[kind], std::memory_order_relaxed);
	return true;
}

std::vector<Counter> gb300Published(const Renderer&) {
	std::vector<Counter> counters;
	for (std::size_t kind = 0; kind < std::size_t(rayKindCount); ++kind) {
		counters.push_back(Counter { .name = "rays." + rayKindName(RayKind(kind)), .value = double(gb300().rays[kind].load()) });
	}
	return counters;
}

} // namespace

// What the binding saw: the steps it was asked for, the most frame blocks
// holding data, whether it traces on a device, and the cells of the world
// it built.
void gb300Seen(std::uint64_t* steps, int* blocks, int* device, std::uint64_t* cells) {
	*steps  = gb300().steps.load();
	*blocks = gb300().blocks.load();
	*device = gb300().device ? 1 : 0;
	std::uint64_t stats[4] = {};
	*cells = gb300().context != nullptr && kdn_world_stats(gb300().context, stats) == KDN_OK ? stats[0] : 0;
}

Plugin backendGb300Plugin() {
	Hooks hooks       = noHooks();
	hooks.openWorkers = gb300Workers;
	hooks.ranStep     = gb300Ran;
	hooks.published   = gb300Published;
	return Plugin {
		.name   = "backend/gb300",
		.point  = Point::Backend,
		.effect = Effect::Exact,
		.hooks  = hooks,
		.reads  = Reads::Nothing,
		.after  = {},
	};
}

} // namespace kodanuki
