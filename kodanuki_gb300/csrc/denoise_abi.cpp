// kdn_denoise / kdn_denoise_device: the denoiser's entry points.
#include "context.h"
#include "denoise.h"

#include <algorithm>
#include <cstring>
#include <vector>

using kdn::Context;

namespace {

constexpr int64_t kMostPixels = int64_t(1) << 26;

kdn_status checkFrame(Context* ctx, const kdn_denoise_frame* f) {
	if (f->width <= 0 || f->height <= 0 || int64_t(f->width) * int64_t(f->height) > kMostPixels) return ctx->fail(KDN_BAD_ARG, "kdn_denoise: frame size out of range");
	if (!(f->reach > 0) || !(f->aspect > 0)) return ctx->fail(KDN_BAD_ARG, "kdn_denoise: the lens needs a positive reach and aspect");
	return KDN_OK;
}

void lensOf(const kdn_denoise_frame* f, double lens[14]) {
	for (int k = 0; k < 3; ++k) {
		lens[k]     = f->eye[k];
		lens[3 + k] = f->forward[k];
		lens[6 + k] = f->right[k];
		lens[9 + k] = f->up[k];
	}
	lens[12] = f->reach;
	lens[13] = f->aspect;
}

// The context's scratch for n pixels, carved from one allocation.
kdn_status scratch(Context* ctx, size_t n, kdn::DenoiseArgs& a) {
	const kdn_status s = ctx->ensure(ctx->denoiseScratch, n * kdn::kDenoiseScratchPerPixel);
	if (s != KDN_OK) return s;
	char* base = static_cast<char*>(ctx->denoiseScratch.ptr);
	a.guideA   = reinterpret_cast<float4*>(base);
	a.guideB = a.guideA + n;
	a.lightA = a.guideB + n;
	a.lightB = a.lightA + n;
	a.sky    = reinterpret_cast<float*>(a.lightB + n);
	return KDN_OK;
}

kdn_status run(Context* ctx, const kdn_denoise_frame* f, kdn::DenoiseArgs& a, cudaStream_t stream) {
	lensOf(f, a.lens);
	a.width       = f->width;
	a.height      = f->height;
	a.demodulated = f->demodulated ? 1 : 0;
	if (!ctx->check(kdn::launchDenoise(a, stream), "denoise kernels")) return KDN_CUDA_ERROR;
	return KDN_OK;
}

} // namespace

namespace kdn {

// The denoiser over device feature buffers with the context's scratch; the
// caller holds the context's lock and has made its device current.
kdn_status denoiseOnDevice(Context* ctx, const kdn_denoise_frame* frame, const float* colour, const float* moment, const float* length, const uint16_t* distance,
                           const uint16_t* normal, const uint16_t* albedo, const uint32_t* leaf, float* out, cudaStream_t stream) {
	kdn_status s = checkFrame(ctx, frame);
	if (s != KDN_OK) return s;
	const size_t n = size_t(frame->width) * size_t(frame->height);
	DenoiseArgs a {};
	if ((s = scratch(ctx, n, a)) != KDN_OK) return s;
	a.colour   = colour;
	a.moment   = moment;
	a.length   = length;
	a.distance = distance;
	a.normal   = normal;
	a.albedo   = albedo;
	a.leaf     = leaf;
	a.out      = out;
	return run(ctx, frame, a, stream);
}

} // namespace kdn

extern "C" {

kdn_status kdn_denoise_device(kdn_ctx* handle, const kdn_denoise_frame* frame, const float* colour, const float* moment, const float* length,
                              const uint16_t* distance, const uint16_t* normal, const uint16_t* albedo, const uint32_t* leaf, float* out, void* stream) {
	if (handle == nullptr || frame == nullptr || !colour || !moment || !length || !distance || !normal || !albedo || !leaf || !out) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->device < 0) return ctx->fail(KDN_NO_DEVICE, "kdn_denoise_device: a host-only context has no device");
	if (!ctx->check(cudaSetDevice(ctx->device), "cudaSetDevice")) return KDN_CUDA_ERROR;
	return kdn::denoiseOnDevice(ctx, frame, colour, moment, length, distance, normal, albedo, leaf, out, stream ? static_cast<cudaStream_t>(stream) : ctx->stream);
}

kdn_status kdn_denoise(kdn_ctx* handle, const kdn_denoise_frame* frame, const float* colour, const float* moment, const float* length,
                       const uint16_t* distance, const uint16_t* normal, const uint16_t* albedo, const uint32_t* leaf, float* out) {
	if (handle == nullptr || frame == nullptr || !colour || !moment || !length || !distance || !normal || !albedo || !leaf || !out) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->device < 0) return ctx->fail(KDN_NO_DEVICE, "kdn_denoise: a host-only context has no device");
	kdn_status s = checkFrame(ctx, frame);
	if (s != KDN_OK) return s;
	if (!ctx->check(cudaSetDevice(ctx->device), "cudaSetDevice")) return KDN_CUDA_ERROR;
	const size_t n = size_t(frame->width) * size_t(frame->height);
	// inputs and output, one device allocation reused between calls
	const size_t bytes[] = { n * 12, n * 4, n * 4, n * 2, n * 6, n * 6, n * 4, n * 12 };
	size_t total         = 0;
	size_t offsets[8];
	for (int k = 0; k < 8; ++k) {
		offsets[k] = total;
		total += (bytes[k] + 255) & ~size_t(255);
	}
	if ((s = ctx->ensure(ctx->denoiseIo, total)) != KDN_OK) return s;
	char* base          = static_cast<char*>(ctx->denoiseIo.ptr);
	const void* hosts[] = { colour, moment, length, distance, normal, albedo, leaf };
	for (int k = 0; k < 7; ++k) {
		if (!ctx->check(cudaMemcpyAsync(base + offsets[k], hosts[k], bytes[k], cudaMemcpyHostToDevice, ctx->stream), "kdn_denoise copy in")) return KDN_CUDA_ERROR;
	}
	kdn::DenoiseArgs a {};
	if ((s = scratch(ctx, n, a)) != KDN_OK) return s;
	a.colour   = reinterpret_cast<const float*>(base + offsets[0]);
	a.moment   = reinterpret_cast<const float*>(base + offsets[1]);
	a.length   = reinterpret_cast<const float*>(base + offsets[2]);
	a.distance = reinterpret_cast<const uint16_t*>(base + offsets[3]);
	a.normal   = reinterpret_cast<const uint16_t*>(base + offsets[4]);
	a.albedo   = reinterpret_cast<const uint16_t*>(base + offsets[5]);
	a.leaf     = reinterpret_cast<const uint32_t*>(base + offsets[6]);
	a.out      = reinterpret_cast<float*>(base + offsets[7]);
	if ((s = run(ctx, frame, a, ctx->stream)) != KDN_OK) return s;
	if (!ctx->check(cudaMemcpyAsync(out, a.out, bytes[7], cudaMemcpyDeviceToHost, ctx->stream), "kdn_denoise copy out")) return KDN_CUDA_ERROR;
	if (!ctx->check(cudaStreamSynchronize(ctx->stream), "kdn_denoise")) return KDN_CUDA_ERROR;
	return KDN_OK;
}

} // extern "C"

#include "temporal.h"
#include "upscale.h"

extern "C" kdn_status kdn_temporal_device(kdn_ctx* handle, const kdn_temporal_frame* frame, const kdn_temporal_buffers* io, void* stream) {
	if (handle == nullptr || frame == nullptr || io == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->device < 0) return ctx->fail(KDN_NO_DEVICE, "kdn_temporal_device: a host-only context has no device");
	if (frame->width <= 0 || frame->height <= 0 || int64_t(frame->width) * int64_t(frame->height) > (int64_t(1) << 26))
		return ctx->fail(KDN_BAD_ARG, "kdn_temporal_device: frame size out of range");
	if (frame->factor > 4 || frame->before_factor > 4 || frame->phase >= std::max(frame->factor, 1u) * std::max(frame->factor, 1u) ||
	    frame->before_phase >= std::max(frame->before_factor, 1u) * std::max(frame->before_factor, 1u))
		return ctx->fail(KDN_BAD_ARG, "kdn_temporal_device: a film factor of 1 to 4 and a phase below its square are needed");
	const bool reads = frame->kept != 0;
	if (!io->light || !io->first_distance || !io->first_normal || !io->first_albedo || !io->first_leaf || !io->centre_distance || !io->centre_normal ||
	    !io->centre_albedo || !io->centre_leaf || !io->colour || !io->moment || !io->length ||
	    (reads && (!io->before_colour || !io->before_moment || !io->before_length || !io->before_distance || !io->before_normal || !io->before_leaf)))
		return ctx->fail(KDN_BAD_ARG, "kdn_temporal_device: a buffer is missing");
	if (!ctx->check(cudaSetDevice(ctx->device), "cudaSetDevice")) return KDN_CUDA_ERROR;
	kdn::TemporalArgs a {};
	a.width     = frame->width;
	a.height    = frame->height;
	a.moved     = frame->moved;
	a.recounted = frame->recounted;
	a.kept      = frame->kept;
	a.now       = kdn::temporalCameraOf(frame->now, frame->width, frame->height);
	a.before    = kdn::temporalCameraOf(frame->before, frame->width, frame->height);
	kdn::filmCentreOf(frame->factor, frame->phase, a.centre);
	kdn::filmCentreOf(frame->before_factor, frame->before_phase, a.centreBefore);
	a.io        = *io;
	if (!ctx->check(kdn::launchTemporal(a, stream ? static_cast<cudaStream_t>(stream) : ctx->stream), "temporal kernel")) return KDN_CUDA_ERROR;
	return KDN_OK;
}

namespace kdn {

kdn_status upscaleOnDevice(Context* ctx, UpscaleScratch& scratch, const kdn_upscale_frame* frame, const kdn_upscale_buffers* io, cudaStream_t stream) {
	const int factor = int(frame->factor);
	const int dw = frame->width / factor, dh = frame->height / factor;
	kdn_status s;
	if ((s = ctx->ensure(scratch.samples, size_t(dw) * size_t(dh) * sizeof(float4))) != KDN_OK) return s;
	if (scratch.factor != frame->factor || scratch.width != frame->width || scratch.height != frame->height) {
		// upscale.cpp:568 upscaleAxis of every place of the factor, on the host
		std::vector<UpscaleAxis> axes(size_t(factor) * size_t(frame->width + frame->height));
		for (int place = 0; place < factor; ++place) {
			upscaleAxes(factor, place, dw, frame->width, axes.data() + size_t(place) * size_t(frame->width));
			upscaleAxes(factor, place, dh, frame->height, axes.data() + size_t(factor) * size_t(frame->width) + size_t(place) * size_t(frame->height));
		}
		scratch.factor = 0;
		if ((s = ctx->ensure(scratch.axes, axes.size() * sizeof(UpscaleAxis))) != KDN_OK) return s;
		if (!ctx->check(cudaMemcpyAsync(scratch.axes.ptr, axes.data(), axes.size() * sizeof(UpscaleAxis), cudaMemcpyHostToDevice, stream), "upscale axes")) return KDN_CUDA_ERROR;
		if (!ctx->check(cudaStreamSynchronize(stream), "upscale axes")) return KDN_CUDA_ERROR;
		scratch.factor = frame->factor;
		scratch.width  = frame->width;
		scratch.height = frame->height;
	}
	const UpscaleAxis* axes = static_cast<const UpscaleAxis*>(scratch.axes.ptr);
	UpscaleArgs a {};
	a.width       = frame->width;
	a.height      = frame->height;
	a.drawnWidth  = dw;
	a.drawnHeight = dh;
	a.kept        = frame->kept;
	a.settling    = frame->settling;
	std::memcpy(a.now, frame->now, sizeof a.now);
	std::memcpy(a.before, frame->before, sizeof a.before);
	a.internal     = io->internal;
	a.distance     = io->distance;
	a.columns      = axes + size_t(frame->phase % frame->factor) * size_t(frame->width);
	a.rows         = axes + size_t(factor) * size_t(frame->width) + size_t(frame->phase / frame->factor) * size_t(frame->height);
	a.before_state = reinterpret_cast<const float4*>(io->before);
	a.after_state  = reinterpret_cast<float4*>(io->after);
	a.image        = io->image;
	a.samples      = static_cast<float4*>(scratch.samples.ptr);
	if (!ctx->check(launchUpscale(a, stream, ctx->smCount), "upscale kernels")) return KDN_CUDA_ERROR;
	return KDN_OK;
}

} // namespace kdn

extern "C" kdn_status kdn_upscale_device(kdn_ctx* handle, const kdn_upscale_frame* frame, const kdn_upscale_buffers* io, void* stream) {
	if (handle == nullptr || frame == nullptr || io == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->device < 0) return ctx->fail(KDN_NO_DEVICE, "kdn_upscale_device: a host-only context has no device");
	if (frame->factor < 2 || frame->factor > 4) return ctx->fail(KDN_BAD_ARG, "kdn_upscale_device: the film factor must be 2, 3 or 4");
	if (frame->phase >= frame->factor * frame->factor) return ctx->fail(KDN_BAD_ARG, "kdn_upscale_device: the phase must be below the factor's square");
	if (frame->width <= 0 || frame->height <= 0 || frame->width % int32_t(frame->factor) != 0 || frame->height % int32_t(frame->factor) != 0 ||
	    int64_t(frame->width) * int64_t(frame->height) > (int64_t(1) << 26))
		return ctx->fail(KDN_BAD_ARG, "kdn_upscale_device: the shown size must be positive, a multiple of the factor and at most 2^26 pixels");
	if (!io->internal || !io->after || !io->image || (frame->kept && !io->before)) return ctx->fail(KDN_BAD_ARG, "kdn_upscale_device: a buffer is missing");
	if (!ctx->check(cudaSetDevice(ctx->device), "cudaSetDevice")) return KDN_CUDA_ERROR;
	return kdn::upscaleOnDevice(ctx, ctx->upscale, frame, io, stream ? static_cast<cudaStream_t>(stream) : ctx->stream);
}

extern "C" kdn_status kdn_upsample_device(kdn_ctx* handle, int32_t width, int32_t height, uint32_t factor, const float* drawn, float* shown, void* stream) {
	if (handle == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->device < 0) return ctx->fail(KDN_NO_DEVICE, "kdn_upsample_device: a host-only context has no device");
	if (factor < 1 || factor > 4) return ctx->fail(KDN_BAD_ARG, "kdn_upsample_device: the film factor must be 1 to 4");
	if (width <= 0 || height <= 0 || width % int32_t(factor) != 0 || height % int32_t(factor) != 0 || int64_t(width) * int64_t(height) > (int64_t(1) << 26))
		return ctx->fail(KDN_BAD_ARG, "kdn_upsample_device: the shown size must be positive, a multiple of the factor and at most 2^26 pixels");
	if (drawn == nullptr || shown == nullptr) return ctx->fail(KDN_BAD_ARG, "kdn_upsample_device: a buffer is missing");
	if (!ctx->check(cudaSetDevice(ctx->device), "cudaSetDevice")) return KDN_CUDA_ERROR;
	if (!ctx->check(kdn::launchUpsample(width, height, int(factor), drawn, shown, stream ? static_cast<cudaStream_t>(stream) : ctx->stream, ctx->smCount), "upsample kernel"))
		return KDN_CUDA_ERROR;
	return KDN_OK;
}
