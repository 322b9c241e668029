// The learned guide behind kdn_guide: what the frame loop (render.cpp)
// launches of it.
#pragma once

#include "frame.h"
#include "kdn.h"

#include <cuda_runtime.h>

namespace kdn {

constexpr int kGuideLobes        = 8;
constexpr int kGuideLobeFloats   = 5 * kGuideLobes;
constexpr int kGuideDepth        = 3;  // vertices 0, 1, 2 of a path are guided and recorded
constexpr int kGuideSampleFloats = 10; // point, normal, direction, weight

// One vertex of a path that a training frame records: where it stood, its
// faced normal, the direction it left by, the throughput that reached it
// (the lanes' sum) and the radiance the path held when the next vertex was
// reached (the lanes' sum; NaN until then).  A record with a NaN direction
// is empty.
struct GuideRecord {
	float point[3];
	float normal[3];
	float direction[3];
	float reached;
	float before;
	float pad;
};

// The frame loop's view of a guide for one bounce's queue.
struct GuideQueue {
	const kdn_hit* hits;
	const kdn_ray* rays;
	const uint32_t* count;
	Looks looks;
	uint32_t materialCount;
	float* lobes; // count x kGuideLobeFloats, written where the hit is guidable
};

// a material the guide samples for: matte and plastic
__host__ __device__ __forceinline__ bool guidable(uint32_t kind) { return kind == 0 || kind == 1; }

// inference over a bounce's queue (no launch where the guide is not ready)
cudaError_t guideQueryQueue(kdn_guide* guide, const GuideQueue& queue, uint32_t capacity, cudaStream_t stream, int smCount);
// the records of a chunk's paths into the guide's training samples
cudaError_t guideGather(kdn_guide* guide, const GuideRecord* records, const float4* radiance, uint32_t paths, uint64_t framePaths, uint32_t salt, cudaStream_t stream, int smCount);
// one training pass over the samples gathered so far (reads their count:
// synchronises the stream), then clears them
kdn_status guideTrainGathered(kdn_guide* guide, cudaStream_t stream);
// the device the guide lives on
int guideDevice(const kdn_guide* guide);

} // namespace kdn
