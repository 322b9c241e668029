// The device denoiser's launch interface.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace kdn {

struct DenoiseArgs {
	int width, height;
	int demodulated;
	double lens[14];         // eye[3], forward[3], right[3], up[3], reach, aspect: by value, in the kernels' parameters
	const float* colour;     // RGB a pixel
	const float* moment;
	const float* length;
	const uint16_t* distance; // FP16 bits
	const uint16_t* normal;   // FP16 bits, 3 a pixel
	const uint16_t* albedo;   // FP16 bits, 3 a pixel
	const uint32_t* leaf;
	float* out;               // RGB a pixel
	// scratch: guides and two light buffers
	float4* guideA;           // x, y, z, plane offset
	float4* guideB;           // normal, 1 / reach
	float* sky;
	float4* lightA;           // r, g, b, variance
	float4* lightB;
};

// Bytes of scratch one pixel needs (guideA, guideB, sky, lightA, lightB).
constexpr size_t kDenoiseScratchPerPixel = 16 + 16 + 4 + 16 + 16;

cudaError_t launchDenoise(const DenoiseArgs& args, cudaStream_t stream);

} // namespace kdn
