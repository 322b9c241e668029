// The temporal member on the device (plugins/reconstruction/temporal/
// temporal.cpp:1001 temporalFrame) with a G-buffer: the drawn grid the
// reference runs before the a-trous denoiser, each pixel's light divided by
// its first surface's albedo.
#pragma once

#include "kdn.h"

#include <cuda_runtime.h>

#include <cstdint>

namespace kdn {

// temporal.cpp:307 temporalCamera, in double as the reference's.
struct TemporalCamera {
	double eye[3], forward[3], corner[3], across[3], down[3], acrossInverse[3], downInverse[3];
	double width, height;
};

// From a lens of 14 doubles (eye, forward, right, up, reach, aspect).
TemporalCamera temporalCameraOf(const double lens[14], int width, int height);

// core/camera.cpp:51 filmCentre: where in a pixel of the drawn grid the
// rays of a frame at film factor `factor` and phase `phase` pass (factor 0
// or 1: the pixel's centre).
void filmCentreOf(uint32_t factor, uint32_t phase, float centre[2]);

struct TemporalArgs {
	int width, height;
	uint32_t moved, recounted, kept;
	TemporalCamera now, before;
	float centre[2], centreBefore[2]; // this frame's film centre and the state before's
	kdn_temporal_buffers io;
};

cudaError_t launchTemporal(const TemporalArgs& args, cudaStream_t stream);

} // namespace kdn
