// The temporal member on the device (plugins/reconstruction/temporal/
// temporal.cpp:1001 temporalFrame) at a film factor of 1 with a G-buffer:
// the grid the reference runs before the a-trous denoiser, each pixel's
// light divided by its first surface's albedo.
#pragma once

#include "kdn.h"

#include <cuda_runtime.h>

#include <cstdint>

namespace kdn {

// temporal.cpp:307 temporalCamera, in FP32.
struct TemporalCamera {
	float eye[3], forward[3], corner[3], across[3], down[3], acrossInverse[3], downInverse[3];
	float width, height;
};

// From a lens of 14 doubles (eye, forward, right, up, reach, aspect).
TemporalCamera temporalCameraOf(const double lens[14], int width, int height);

struct TemporalArgs {
	int width, height;
	uint32_t moved, recounted, kept;
	TemporalCamera now, before;
	kdn_temporal_buffers io;
};

cudaError_t launchTemporal(const TemporalArgs& args, cudaStream_t stream);

} // namespace kdn
