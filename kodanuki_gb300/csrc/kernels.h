// Launch interfaces of the backend's CUDA kernels (host side).
#pragma once

#include "kdn.h"
#include "world.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

namespace kdn {

// Where a ray's march ended: kind 0 none, 1 surface at distance, 2 a crossing
// into a solid of another material (read past the point); first/index name
// the kept program that is least there.
struct HitState {
	uint32_t kind;
	float distance;
	uint32_t first;
	uint32_t index;
	uint32_t steps;
};

struct TraceArgs {
	DeviceWorld world;
	const kdn_ray* rays;
	uint32_t n;
	HitState* states;
	const uint32_t* objectMaterial; // material of each object's first leaf
	uint32_t maxSteps;
	unsigned long long* counters;   // [0] march steps, [1] program steps, [2] longest march, [3] capped rays, [4] rays
	const uint32_t* count;          // if set, the number of rays is read here on the device
	uint32_t* fetch;                // the next ray to take; launchTrace zeroes it
	// a second run of rays in the same arrays, from index `second` on, its
	// count read on the device (null: none); traced in the same launch
	const uint32_t* secondCount = nullptr;
	uint32_t second             = 0;
};

struct HitArgs {
	DeviceWorld world;
	const kdn_ray* rays;
	const HitState* states;
	uint32_t n;
	kdn_hit* hits;
	const uint32_t* count;          // if set, the number of rays is read here on the device
};

cudaError_t setTraceAttributes();
cudaError_t launchTrace(const TraceArgs& args, cudaStream_t stream, int smCount);
cudaError_t launchHits(const HitArgs& args, cudaStream_t stream, int smCount);

} // namespace kdn
