// The state behind one kdn_ctx: blocks, the built world, device buffers.
#pragma once

#include "kdn.h"
#include "kernels.h"
#include "octree.h"

#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace kdn {

// A device allocation that grows on demand and is freed with the context.
struct DeviceBuffer {
	void* ptr     = nullptr;
	size_t bytes  = 0;
	bool borrowed = false; // another context's: not freed with this one
};

struct FrameState; // render.cpp

// The upscale member's scratch: the drawn frame's tones and depths, and the
// axes of every phase of a film factor over a shown size (columns of each
// place across, then rows of each place down), kept while the factor and
// size stay.
struct UpscaleScratch {
	DeviceBuffer samples, axes;
	uint32_t factor = 0;
	int32_t width = 0, height = 0;
};

struct Context {
	int device          = 0;
	int smCount         = 0; // SMs the kernels' grids are sized for (kdn_set_sm_limit)
	int deviceSms       = 0; // the device's
	cudaStream_t stream = nullptr;
	int priority        = 0; // of this context's streams (cudaStreamCreateWithPriority)
	// a context that draws frames of another's world (kdn_open_sharing)
	Context* source = nullptr;
	std::atomic<int> sharers { 0 }; // contexts drawing this one's world
	// the most device bytes a frame's path buffers may take (0: half the free memory)
	uint64_t frameBudget = 0;
	// march steps a ray takes in one trace launch of a frame before it is
	// carried to the next (0: no budget; kdn_set_march_budget)
	uint32_t marchBudget = 0;
	std::mutex lock;
	std::string error;
	std::map<std::string, std::vector<uint8_t>> blocks;
	bool built        = false;
	bool sceneChanged = true;
	Octree octree;
	FlatWorld flat;
	std::string flatError; // why a host-only context has no device layout
	std::vector<GridCell> gridCells; // the grid over the flat octree (world.h GridCell)
	std::vector<float> walls;        // its walls per axis
	float lowerF[3] = {}, sizeF[3] = {};
	std::vector<int64_t> preorder; // cell index of each depth-first position
	DeviceWorld world {};
	DeviceBuffer nodes, leaves, programs, steps, march, ssa, leafMaterial, objectMaterial, grid, gridWalls;
	DeviceBuffer extendRays, extendHits, extendStates, counters, l2;
	DeviceBuffer denoiseScratch, denoiseIo, fetch;
	UpscaleScratch upscale; // kdn_upscale_device's
	DeviceBuffer sobolTables; // --use sampler=sobol's byte tables, built at the first frame that asks
	FrameState* frame = nullptr;
	// the learned guide frames use (kdn_set_guide): KDN_GUIDE_SAMPLE, KDN_GUIDE_TRAIN
	kdn_guide* guide    = nullptr;
	float guideShare    = 0.5f;
	uint32_t guideFlags = 0;

	kdn_status open();
	kdn_status share(Context* from);
	void release();
	kdn_status fail(kdn_status status, const std::string& message);
	bool check(cudaError_t e, const char* what);
	kdn_status ensure(DeviceBuffer& buffer, size_t bytes);
	kdn_status upload(DeviceBuffer& buffer, const void* data, size_t bytes);
	template <typename T>
	const std::vector<T> block(const char* name) const {
		std::vector<T> out;
		auto it = blocks.find(name);
		if (it == blocks.end()) return out;
		out.resize(it->second.size() / sizeof(T));
		if (!out.empty()) std::memcpy(out.data(), it->second.data(), out.size() * sizeof(T));
		return out;
	}
	bool has(const char* name) const { return blocks.count(name) != 0; }
	kdn_status build(const BuildOptions& options);
	int64_t preorderCell(uint64_t i) const;
	kdn_status extend(const kdn_ray* rays, uint32_t n, kdn_hit* hits, cudaStream_t on);
	kdn_status flushL2();
	void releaseFrame();
};

// guide.cu: the device a learned guide lives on
int guideDevice(const kdn_guide* guide);

// denoise_abi.cpp: the upscale member over device buffers (kdn_upscale_device
// and a frame's chain), with the scratch of its caller.
kdn_status upscaleOnDevice(Context* ctx, UpscaleScratch& scratch, const kdn_upscale_frame* frame, const kdn_upscale_buffers* io, cudaStream_t stream);

// denoise_abi.cpp: the denoiser over device buffers with the context's scratch.
kdn_status denoiseOnDevice(Context* ctx, const kdn_denoise_frame* frame, const float* colour, const float* moment, const float* length, const uint16_t* distance,
                           const uint16_t* normal, const uint16_t* albedo, const uint32_t* leaf, float* out, cudaStream_t stream);

} // namespace kdn
