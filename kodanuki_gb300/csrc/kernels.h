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
// the kept program that is least there.  Kind kCarried: the ray used up its
// march budget for this launch and goes on in a later one from distance,
// after steps march steps (its resume data, TraceArgs::carry).
constexpr uint32_t kCarried = 3;
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
	// Carried rays (null: none).  A ray whose pad_[0] has bit 0 set resumes
	// its march where carry[ray] says (x: distance bits, y: march steps so
	// far) instead of at the region's edge; with budget > 0 a ray that has
	// taken budget march steps in this launch stops as kCarried.  The march
	// is deterministic, so a carried ray ends where it would have in one launch.
	const uint2* carry = nullptr;
	uint32_t budget    = 0;
	// where set, a count that must be zero (path rays left after a frame's
	// last round): added to counters[6], which the host checks
	const uint32_t* left = nullptr;
};

// kdn_hit.kind of a carried ray: distance is where its march stands, cell
// its march steps so far.
constexpr uint8_t kHitCarried = 0xFE;
// kdn_ray.pad_[0] bit 0: the ray resumes a carried march.
constexpr uint8_t kRayResumes = 1;

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
