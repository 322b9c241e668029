// kdn_denoise_static: the denoiser for callers that may not allocate device
// memory.
//
// kdn_denoise and kdn_denoise_device keep their scratch (guides and two light
// buffers, 68 bytes a pixel) in buffers the context allocates on first use
// and grows with the frame.  Some callers cannot let a call allocate: a frame
// loop that reserved its whole device-memory budget at start-up and must not
// go past it, or one that must not stall its other streams on the device-wide
// synchronisation cudaMalloc and cudaFree can cause.  This entry point takes
// no context and allocates nothing: its scratch is the file-scope array below,
// a fixed size, held by every GPU that loads the library until the process
// exits.
#include "denoise.h"
#include "kdn.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>

namespace kdn {

void setThreadError(const std::string& message); // abi.cpp: kdn_last_error(NULL)

// The largest frame the static scratch holds: 512 x 512 pixels.  The lens
// travels by value in the kernels' parameters, so the scratch is the
// per-pixel guides and light alone.
constexpr size_t kStaticDenoisePixels = size_t(512) * 512;
constexpr size_t kStaticDenoiseBytes  = kStaticDenoisePixels * kDenoiseScratchPerPixel;

// File-scope device scratch: 17 MiB on every device that loads the library.
static __device__ __align__(256) unsigned char staticDenoiseScratch[kStaticDenoiseBytes];

namespace {

constexpr int kMostDevices = 64;
std::mutex staticLock;
void* staticAddress[kMostDevices] = {};

// The message kdn_last_error(NULL) gives on this thread.
kdn_status failed(kdn_status s, const std::string& message) {
	setThreadError(message);
	return s;
}

// The device address of the scratch on the current device, looked up once
// per device: in host code `staticDenoiseScratch` names a host-side stand-in,
// not device memory, so the kernels get the address cudaGetSymbolAddress gives.
kdn_status scratchAddress(int device, void** out) {
	std::lock_guard<std::mutex> guard(staticLock);
	if (staticAddress[device] == nullptr) {
		void* ptr           = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&ptr, staticDenoiseScratch);
		if (e != cudaSuccess) return failed(KDN_CUDA_ERROR, std::string("kdn_denoise_static: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
		staticAddress[device] = ptr;
	}
	*out = staticAddress[device];
	return KDN_OK;
}

} // namespace

} // namespace kdn

extern "C" {

kdn_status kdn_denoise_static(const kdn_denoise_frame* frame, const float* colour, const float* moment, const float* length, const uint16_t* distance,
                              const uint16_t* normal, const uint16_t* albedo, const uint32_t* leaf, float* out, void* stream) {
	using namespace kdn;
	if (frame == nullptr || !colour || !moment || !length || !distance || !normal || !albedo || !leaf || !out) return failed(KDN_BAD_ARG, "kdn_denoise_static: a null argument");
	if (frame->width <= 0 || frame->height <= 0) return failed(KDN_BAD_ARG, "kdn_denoise_static: the frame size must be positive");
	const size_t n = size_t(frame->width) * size_t(frame->height);
	if (n > kStaticDenoisePixels) {
		return failed(KDN_BAD_ARG, "kdn_denoise_static: " + std::to_string(frame->width) + "x" + std::to_string(frame->height) + " is " + std::to_string(n) +
		                               " pixels, past the 262144 (512x512) its static scratch holds; use kdn_denoise_device");
	}
	if (!(frame->reach > 0) || !(frame->aspect > 0)) return failed(KDN_BAD_ARG, "kdn_denoise_static: the lens needs a positive reach and aspect");
	int device = 0;
	cudaError_t e = cudaGetDevice(&device);
	if (e != cudaSuccess) return failed(KDN_NO_DEVICE, std::string("kdn_denoise_static: cudaGetDevice: ") + cudaGetErrorString(e));
	if (device < 0 || device >= kMostDevices) return failed(KDN_BAD_ARG, "kdn_denoise_static: device ordinal past 63");
	void* base = nullptr;
	const kdn_status s = scratchAddress(device, &base);
	if (s != KDN_OK) return s;
	const cudaStream_t on = static_cast<cudaStream_t>(stream);
	DenoiseArgs a {};
	for (int k = 0; k < 3; ++k) {
		a.lens[k]     = frame->eye[k];
		a.lens[3 + k] = frame->forward[k];
		a.lens[6 + k] = frame->right[k];
		a.lens[9 + k] = frame->up[k];
	}
	a.lens[12] = frame->reach;
	a.lens[13] = frame->aspect;
	// Every kernel writes each pixel's guides and light before any reads
	// them, so nothing in the scratch has to start at zero.
	a.guideA      = static_cast<float4*>(base);
	a.guideB      = a.guideA + n;
	a.lightA      = a.guideB + n;
	a.lightB      = a.lightA + n;
	a.sky         = reinterpret_cast<float*>(a.lightB + n);
	a.width       = frame->width;
	a.height      = frame->height;
	a.demodulated = frame->demodulated ? 1 : 0;
	a.colour      = colour;
	a.moment      = moment;
	a.length      = length;
	a.distance    = distance;
	a.normal      = normal;
	a.albedo      = albedo;
	a.leaf        = leaf;
	a.out         = out;
	e = launchDenoise(a, on);
	if (e != cudaSuccess) return failed(KDN_CUDA_ERROR, std::string("kdn_denoise_static: ") + cudaGetErrorString(e));
	return KDN_OK;
}

} // extern "C"
