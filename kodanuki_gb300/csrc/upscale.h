// The upscale and upsample members on the device (plugins/reconstruction/
// upscale/upscale.cpp upscaledFrame, upsample/upsample.cpp upsampledImage):
// a frame drawn at 1/factor of the shown size, one phase of the factor^2
// shown pixels a drawn pixel covers each frame, gathered to the shown size
// against a history of shown pixels, or blown up bilinearly.
#pragma once

#include "kdn.h"

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace kdn {

// upscale.cpp:568 upscaleAxis: for one shown column (or row), the three
// drawn taps around it, their sharp (Gaussian) and fill (Catmull-Rom)
// weights, the drawn neighbour toward the shown pixel and the 3x3 box the
// clamp reads (its centre's index plus one).
struct UpscaleAxis {
	int taps[3];
	float sharp[3];
	float fill[3];
	int toward;
	int box;
	int pad;
};

// The axes of `shown` shown columns (or rows) over `count` drawn ones at a
// film factor, for the phase's place along the axis (phase % factor across,
// phase / factor down), with the reference's own double arithmetic and exp
// on the host.
void upscaleAxes(int factor, int place, int count, int shown, UpscaleAxis* out);

struct UpscaleArgs {
	int width, height;           // shown
	int drawnWidth, drawnHeight; // drawn: shown / factor
	uint32_t kept, settling;
	double now[14], before[14];  // lenses: eye, forward, right, up, reach, aspect
	const float* internal;       // x3, drawn
	const uint16_t* distance;    // FP16 G-buffer distances, drawn, or null (every sample sky)
	const UpscaleAxis* columns;  // shown width
	const UpscaleAxis* rows;     // shown height
	const float4* before_state;  // shown: colour and depth of the state before (read when kept)
	float4* after_state;         // shown
	float* image;                // x3, shown
	float4* samples;             // scratch, drawn: tone and depth
};

cudaError_t launchUpscale(const UpscaleArgs& args, cudaStream_t stream, int smCount);

// plugins/reconstruction/upsample/upsample.cpp upsampledImage: the drawn
// frame (width / factor x height / factor, RGB) bilinearly to width x height.
cudaError_t launchUpsample(int width, int height, int factor, const float* drawn, float* shown, cudaStream_t stream, int smCount);

} // namespace kdn
