// Context: device set-up, blocks to world, and the geometry entry points.
#include "context.h"

#include <cstring>

namespace kdn {

kdn_status Context::open() {
	if (!check(cudaSetDevice(device), "cudaSetDevice")) return KDN_NO_DEVICE;
	cudaDeviceProp prop;
	if (!check(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties")) return KDN_NO_DEVICE;
	smCount   = prop.multiProcessorCount;
	deviceSms = prop.multiProcessorCount;
	if (!check(setTraceAttributes(), "the trace kernel is not built for this device")) return KDN_NO_DEVICE;
	if (!check(cudaStreamCreateWithPriority(&stream, cudaStreamNonBlocking, priority), "cudaStreamCreate")) return KDN_CUDA_ERROR;
	kdn_status s = ensure(counters, 8 * sizeof(unsigned long long));
	if (s != KDN_OK) return s;
	return ensure(fetch, 256);
}

// Draw frames of `from`'s built world: its world buffers are borrowed (not
// copied, not freed here), its blocks copied; the frame buffers, streams and
// counters are this context's own.
kdn_status Context::share(Context* from) {
	blocks = from->blocks;
	world  = from->world;
	for (auto pair : { std::make_pair(&leafMaterial, &from->leafMaterial), std::make_pair(&objectMaterial, &from->objectMaterial) }) {
		*pair.first          = *pair.second;
		pair.first->borrowed = true;
	}
	built        = from->built;
	sceneChanged = false;
	source       = from;
	from->sharers.fetch_add(1);
	return KDN_OK;
}

static void freeBuffer(DeviceBuffer& b) {
	if (b.ptr && !b.borrowed) cudaFree(b.ptr);
	b.ptr      = nullptr;
	b.bytes    = 0;
	b.borrowed = false;
}

void Context::release() {
	if (source) source->sharers.fetch_sub(1);
	source = nullptr;
	if (device < 0) return;
	cudaSetDevice(device);
	if (stream) cudaStreamSynchronize(stream);
	releaseFrame();
	for (DeviceBuffer* b : { &nodes, &leaves, &programs, &steps, &march, &ssa, &leafMaterial, &objectMaterial, &grid, &gridWalls, &extendRays, &extendHits, &extendStates, &counters, &l2, &denoiseScratch, &denoiseIo, &fetch, &upscale.samples, &upscale.axes, &sobolTables }) freeBuffer(*b);
	if (stream) cudaStreamDestroy(stream);
	stream = nullptr;
}

kdn_status Context::fail(kdn_status status, const std::string& message) {
	error = message;
	return status;
}

bool Context::check(cudaError_t e, const char* what) {
	if (e == cudaSuccess) return true;
	error = std::string(what) + ": " + cudaGetErrorString(e);
	return false;
}

kdn_status Context::ensure(DeviceBuffer& buffer, size_t bytes) {
	if (buffer.bytes >= bytes && buffer.ptr) return KDN_OK;
	freeBuffer(buffer);
	if (bytes == 0) bytes = 16;
	const cudaError_t e = cudaMalloc(&buffer.ptr, bytes);
	if (e != cudaSuccess) {
		cudaGetLastError();
		buffer.ptr = nullptr;
		return fail(e == cudaErrorMemoryAllocation ? KDN_OOM : KDN_CUDA_ERROR, std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes: " + cudaGetErrorString(e));
	}
	buffer.bytes = bytes;
	return KDN_OK;
}

kdn_status Context::upload(DeviceBuffer& buffer, const void* data, size_t bytes) {
	const kdn_status s = ensure(buffer, bytes);
	if (s != KDN_OK) return s;
	if (bytes && !check(cudaMemcpyAsync(buffer.ptr, data, bytes, cudaMemcpyHostToDevice, stream), "upload")) return KDN_CUDA_ERROR;
	return KDN_OK;
}

kdn_status Context::build(const BuildOptions& options) {
	if (device >= 0 && !check(cudaSetDevice(device), "cudaSetDevice")) return KDN_CUDA_ERROR;
	if (!has("scene.steps") || !has("scene.programs") || !has("geometry.region")) return fail(KDN_NOT_READY, "kdn_build: the scene.steps, scene.programs and geometry.region blocks are needed");
	const std::vector<kdn_step> all          = block<kdn_step>("scene.steps");
	const std::vector<kdn_program_ref> refs  = block<kdn_program_ref>("scene.programs");
	const std::vector<kdn_region> regions    = block<kdn_region>("geometry.region");
	const std::vector<uint32_t> leafMaterials = block<uint32_t>("scene.leaves");
	std::vector<ProgPtr> objects;
	std::vector<uint32_t> firstLeafMaterial;
	for (uint32_t i = 0; i < refs.size(); ++i) {
		const kdn_program_ref& r = refs[i];
		if (uint64_t(r.first) + r.count > all.size() || r.count == 0 || r.result >= r.count) return fail(KDN_BAD_ARG, "kdn_build: program " + std::to_string(i) + " runs past scene.steps");
		auto p    = std::make_shared<Prog>();
		p->steps.assign(all.begin() + r.first, all.begin() + r.first + r.count);
		p->result = r.result;
		p->object = i;
		uint32_t material = 0xFFFFFFFFu;
		for (const kdn_step& s : p->steps) {
			if (s.opcode >= OpCount) return fail(KDN_BAD_ARG, "kdn_build: unknown opcode in program " + std::to_string(i));
			const int reads = s.opcode == OpSelect || s.opcode == OpSmin ? 3 : (s.opcode <= OpNormalZ ? 0 : (s.opcode == OpNegate || (s.opcode >= OpSqrt && s.opcode <= OpSign) || s.opcode == OpNot ? 1 : 2));
			const uint32_t at = uint32_t(&s - p->steps.data());
			if ((reads > 0 && s.a >= at) || (reads > 1 && s.b >= at) || (reads > 2 && s.c >= at)) return fail(KDN_BAD_ARG, "kdn_build: a step reads a later step in program " + std::to_string(i));
			if (material == 0xFFFFFFFFu && s.leaf < leafMaterials.size()) material = leafMaterials[s.leaf];
		}
		firstLeafMaterial.push_back(material);
		objects.push_back(p);
	}
	std::string message = buildOctree(objects, regions[0].lower, regions[0].size, options, octree);
	if (!message.empty()) return fail(KDN_BAD_ARG, "kdn_build: " + message);
	// the device layout and its limits (kMaxSsa, kMaxSlots): a device needs
	// it; a host-only context keeps it where the limits allow, for checks
	flat = FlatWorld();
	flatError.clear();
	message = flattenOctree(octree, flat);
	if (!message.empty()) {
		if (device >= 0) return fail(KDN_BAD_ARG, "kdn_build: " + message);
		flat      = FlatWorld();
		flatError = message;
	}
	// the grid over the flat octree, for locating points
	gridCells.clear();
	walls.clear();
	for (int a = 0; a < 3; ++a) {
		lowerF[a] = float(regions[0].lower[a]);
		sizeF[a]  = float(regions[0].size[a]);
	}
	if (!flat.nodes.empty()) {
		gridCells = gridOf(flat, kGridLevel);
		walls     = gridWallsOf(lowerF, sizeF, kGridLevel);
	}
	// depth-first order of the cells, for kdn_world_cell
	preorder.clear();
	preorder.reserve(octree.cells.size());
	std::vector<int64_t> stack = { 0 };
	while (!stack.empty()) {
		const int64_t c = stack.back();
		stack.pop_back();
		preorder.push_back(c);
		const int64_t first = octree.cells[size_t(c)].firstChild;
		if (first >= 0) {
			for (int o = 7; o >= 0; --o) stack.push_back(first + o);
		}
	}
	if (device < 0) {
		// a host-only context keeps the world on the host alone
		built = true;
		return KDN_OK;
	}
	kdn_status s;
	if ((s = upload(nodes, flat.nodes.data(), flat.nodes.size() * sizeof(int32_t))) != KDN_OK) return s;
	if ((s = upload(leaves, flat.leaves.data(), flat.leaves.size() * sizeof(GpuLeaf))) != KDN_OK) return s;
	if ((s = upload(programs, flat.programs.data(), flat.programs.size() * sizeof(GpuProgram))) != KDN_OK) return s;
	if ((s = upload(steps, flat.steps.data(), flat.steps.size() * sizeof(GpuStep))) != KDN_OK) return s;
	if ((s = upload(ssa, flat.ssa.data(), flat.ssa.size() * sizeof(SsaOps))) != KDN_OK) return s;
	if ((s = upload(march, flat.march.data(), flat.march.size() * sizeof(MarchStep))) != KDN_OK) return s;
	if ((s = upload(leafMaterial, leafMaterials.data(), leafMaterials.size() * sizeof(uint32_t))) != KDN_OK) return s;
	if ((s = upload(objectMaterial, firstLeafMaterial.data(), firstLeafMaterial.size() * sizeof(uint32_t))) != KDN_OK) return s;
	if ((s = upload(grid, gridCells.data(), gridCells.size() * sizeof(GridCell))) != KDN_OK) return s;
	if ((s = upload(gridWalls, walls.data(), walls.size() * sizeof(float))) != KDN_OK) return s;
	if (!check(cudaStreamSynchronize(stream), "kdn_build upload")) return KDN_CUDA_ERROR;
	world.nodes         = static_cast<const int32_t*>(nodes.ptr);
	world.leaves        = static_cast<const GpuLeaf*>(leaves.ptr);
	world.programs      = static_cast<const GpuProgram*>(programs.ptr);
	world.steps         = static_cast<const GpuStep*>(steps.ptr);
	world.ssa           = static_cast<const SsaOps*>(ssa.ptr);
	world.march         = static_cast<const MarchStep*>(march.ptr);
	world.leaf_material = static_cast<const uint32_t*>(leafMaterial.ptr);
	world.grid          = static_cast<const GridCell*>(grid.ptr);
	world.gridWalls     = static_cast<const float*>(gridWalls.ptr);
	world.gridLevel     = kGridLevel;
	for (int a = 0; a < 3; ++a) {
		world.lower[a] = float(regions[0].lower[a]);
		world.size[a]  = float(regions[0].size[a]);
		world.gridScale[a] = float(double(1u << kGridLevel) / double(world.size[a]));
	}
	world.leaf_count     = uint32_t(flat.leaves.size());
	world.material_count = uint32_t(block<kdn_material>("looks.materials").size());
	world.marchSlots     = 1;
	for (const GpuProgram& g : flat.programs) world.marchSlots = std::max<uint32_t>(world.marchSlots, g.marchSlots);
	built                = true;
	return KDN_OK;
}

int64_t Context::preorderCell(uint64_t i) const {
	return i < preorder.size() ? preorder[size_t(i)] : -1;
}

kdn_status Context::extend(const kdn_ray* rays, uint32_t n, kdn_hit* hits, cudaStream_t on) {
	if (!built) return fail(KDN_NOT_READY, "kdn_extend: no world built (kdn_build)");
	if (!check(cudaSetDevice(device), "cudaSetDevice")) return KDN_CUDA_ERROR;
	if (n == 0) return KDN_OK;
	kdn_status s = ensure(extendStates, size_t(n) * sizeof(HitState));
	if (s != KDN_OK) return s;
	TraceArgs t;
	t.world          = world;
	t.rays           = rays;
	t.n              = n;
	t.states         = static_cast<HitState*>(extendStates.ptr);
	t.objectMaterial = static_cast<const uint32_t*>(objectMaterial.ptr);
	t.maxSteps       = kMarchSteps;
	t.counters       = nullptr;
	t.count          = nullptr;
	t.fetch          = static_cast<uint32_t*>(fetch.ptr);
	if (!check(launchTrace(t, on, smCount), "trace kernel")) return KDN_CUDA_ERROR;
	HitArgs h;
	h.world  = world;
	h.rays   = rays;
	h.states = t.states;
	h.n      = n;
	h.hits   = hits;
	h.count  = nullptr;
	if (!check(launchHits(h, on, smCount), "hit kernel")) return KDN_CUDA_ERROR;
	return KDN_OK;
}

kdn_status Context::flushL2() {
	const size_t bytes = size_t(512) << 20;
	kdn_status s       = ensure(l2, bytes);
	if (s != KDN_OK) return s;
	if (!check(cudaMemsetAsync(l2.ptr, 0x5a, bytes, stream), "L2 flush")) return KDN_CUDA_ERROR;
	return KDN_OK;
}

} // namespace kdn
