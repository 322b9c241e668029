// The SVGF-like denoiser on the device (plugins/reconstruction/atrous/
// atrous.cpp:513 denoisedFrame), five kernels over the frame:
//   K-prep     guides (camera-space point, normal, plane offset, 1/reach) and
//              the demodulated light with its history variance (:148);
//   K-var      a 7x7 spatial variance where the history is young (:376);
//   K-atrous   x4: a 3x3 prefilter of the variance, then the 5x5 B3 spline
//              at steps 1, 2, 4, 8 stopped by normal^128, plane distance and
//              luminance over the deviation (:411);
//   K-remod    times the albedo, faded toward the history by its length (:461).
// Features come in as FP16 (distance, normal, albedo) beside FP32 light;
// the arithmetic is FP32 in the reference's order (this file is compiled
// without FMA contraction) and the per-pixel guide set-up is FP64 as the
// reference's is, so the output matches the reference's float for float.
#include "denoise.h"

#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace kdn {

namespace {

constexpr int kBlockX = 16;
constexpr int kBlockY = 8;

__device__ __forceinline__ float quickExp(float x) {
	// atrous.cpp:31: 2^(x log2 e), the mantissa from a fitted quadratic
	const float t     = fmaxf(x, -30.0f) * 1.44269504f;
	const float whole = floorf(t);
	const float f     = t - whole;
	const float power = 1.0f + f * (0.66023f + f * 0.33977f);
	const float value = __int_as_float(__float_as_int(power) + int(whole) * (1 << 23));
	return x > -30.0f ? value : 0.0f;
}

__device__ __forceinline__ float luma(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

__device__ __forceinline__ double divisorOf(double a) { return a < 1e-3 ? 1.0 : a; }

__global__ void prepKernel(const __grid_constant__ DenoiseArgs a) {
	const int x = blockIdx.x * blockDim.x + threadIdx.x;
	const int y = blockIdx.y * blockDim.y + threadIdx.y;
	if (x >= a.width || y >= a.height) return;
	const size_t p = size_t(y) * size_t(a.width) + size_t(x);
	const float distance = __half2float(__ushort_as_half(a.distance[p]));
	const bool sky       = a.leaf[p] == 0xFFFFFFFFu || !isfinite(distance) || !(distance > 0.0f);
	float4 g0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), g1 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	if (!sky) {
		const double nx = __half2float(__ushort_as_half(a.normal[3 * p]));
		const double ny = __half2float(__ushort_as_half(a.normal[3 * p + 1]));
		const double nz = __half2float(__ushort_as_half(a.normal[3 * p + 2]));
		const double* L = a.lens;
		const double sideways = L[12] * L[13];
		double h[3];
		for (int k = 0; k < 3; ++k) {
			const double corner = L[3 + k] - L[6 + k] * sideways + L[9 + k] * L[12];
			const double across = L[6 + k] * (2.0 * sideways / double(a.width));
			const double down   = L[9 + k] * (-2.0 * L[12] / double(a.height));
			h[k]                = corner + across * (double(x) + 0.5) + down * (double(y) + 0.5);
		}
		const double hl = sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
		const double s  = double(distance) / hl;
		const double px = h[0] * s, py = h[1] * s, pz = h[2] * s;
		g0 = make_float4(float(px), float(py), float(pz), float(px * nx + py * ny + pz * nz));
		g1 = make_float4(float(nx), float(ny), float(nz), float(1.0 / (0.02 * double(distance))));
	}
	a.guideA[p] = g0;
	a.guideB[p] = g1;
	a.sky[p]    = sky ? 1.0f : 0.0f;
	double dv[3] = { 1.0, 1.0, 1.0 };
	if (!a.demodulated) {
		for (int c = 0; c < 3; ++c) dv[c] = divisorOf(double(__half2float(__ushort_as_half(a.albedo[3 * p + c]))));
	}
	const double cr = a.colour[3 * p], cg = a.colour[3 * p + 1], cb = a.colour[3 * p + 2];
	const float r = float(cr / dv[0]), g = float(cg / dv[1]), b = float(cb / dv[2]);
	float variance = -1.0f;
	const float length = a.length[p];
	if (length >= 4.0f) {
		const double l      = 0.2126 * cr + 0.7152 * cg + 0.0722 * cb;
		const double scale  = 0.2126 * dv[0] + 0.7152 * dv[1] + 0.0722 * dv[2];
		const double spread = double(a.moment[p]) - l * l;
		variance            = float((spread > 0.0 ? spread : 0.0) / (double(length) * scale * scale));
	}
	a.lightA[p] = make_float4(r, g, b, variance);
}

// The weight of tap q for centre p (atrous.cpp:260-300).
__device__ __forceinline__ float tapWeight(float4 pa, float4 pb, float psky, float plum, float4 qa, float4 qb, float qsky, float qlum, float invPlane, float invDev, float kernel) {
	const float facing = pb.x * qb.x + pb.y * qb.y + pb.z * qb.z + psky * qsky;
	float power        = facing > 0.5f ? facing : 0.0f;
	for (int n = 0; n < 7; ++n) power *= power;
	const float along = qa.x * pb.x + qa.y * pb.y + qa.z * pb.z;
	const float plane = fabsf(along - pa.w) * invPlane;
	const float apart = fabsf(qlum - plum) * invDev;
	return kernel * power * quickExp(-plane - apart);
}

__global__ void varianceKernel(const __grid_constant__ DenoiseArgs a) {
	const int x = blockIdx.x * blockDim.x + threadIdx.x;
	const int y = blockIdx.y * blockDim.y + threadIdx.y;
	if (x >= a.width || y >= a.height) return;
	const size_t p  = size_t(y) * size_t(a.width) + size_t(x);
	const float4 lp = a.lightA[p];
	float4 out      = lp;
	if (lp.w < 0.0f) {
		const float4 pa = a.guideA[p], pb = a.guideB[p];
		const float psky = a.sky[p];
		const float plum = luma(lp.x, lp.y, lp.z);
		float sr = 0.0f, sg = 0.0f, sb = 0.0f, sq = 0.0f, sw = 0.0f;
		for (int j = -3; j <= 3; ++j) {
			const int qy = y + j;
			if (qy < 0 || qy >= a.height) continue;
			for (int i = -3; i <= 3; ++i) {
				const int qx = x + i;
				if (qx < 0 || qx >= a.width) continue;
				const size_t q  = size_t(qy) * size_t(a.width) + size_t(qx);
				const float4 lq = a.lightA[q];
				const float qlum = luma(lq.x, lq.y, lq.z);
				const float w   = tapWeight(pa, pb, psky, plum, a.guideA[q], a.guideB[q], a.sky[q], qlum, pb.w * 1.0f, 0.0f, 1.0f);
				sr += w * lq.x;
				sg += w * lq.y;
				sb += w * lq.z;
				sw += w;
				sq += w * qlum * qlum;
			}
		}
		if (!(sw > 0.0f)) {
			out.w = 0.0f;
		} else {
			const float mean = luma(sr, sg, sb) / sw;
			const float v    = sq / sw - mean * mean;
			out.w            = v > 0.0f ? v : 0.0f;
		}
	}
	a.lightB[p] = out;
}

__constant__ float cSpline[5] = { 1.0f / 16, 1.0f / 4, 3.0f / 8, 1.0f / 4, 1.0f / 16 };
__constant__ float cGauss[3]  = { 0.25f, 0.5f, 0.25f };

__global__ void atrousKernel(const __grid_constant__ DenoiseArgs a, const float4* __restrict__ in, float4* __restrict__ out, int step) {
	const int x = blockIdx.x * blockDim.x + threadIdx.x;
	const int y = blockIdx.y * blockDim.y + threadIdx.y;
	if (x >= a.width || y >= a.height) return;
	const size_t p  = size_t(y) * size_t(a.width) + size_t(x);
	const float4 lp = in[p];
	const float plum = luma(lp.x, lp.y, lp.z);
	// prefilteredDeviation: the 3x3 Gaussian of the variance
	float vs = 0.0f, vw = 0.0f;
	for (int j = 0; j < 3; ++j) {
		const int qy = y + j - 1;
		if (qy < 0 || qy >= a.height) continue;
		for (int i = 0; i < 3; ++i) {
			const int qx = x + i - 1;
			if (qx < 0 || qx >= a.width) continue;
			const float k = cGauss[i] * cGauss[j];
			vs += k * in[size_t(qy) * size_t(a.width) + size_t(qx)].w;
			vw += k;
		}
	}
	const float invDev   = 1.0f / (4.0f * sqrtf(vs / vw) + 1e-4f + 1e-3f * plum);
	const float4 pa      = a.guideA[p], pb = a.guideB[p];
	const float psky     = a.sky[p];
	const float invPlane = pb.w * (1.0f / float(step));
	float sr = 0.0f, sg = 0.0f, sb = 0.0f, sv = 0.0f, sw = 0.0f;
	for (int j = -2; j <= 2; ++j) {
		const int qy = y + j * step;
		if (qy < 0 || qy >= a.height) continue;
		for (int i = -2; i <= 2; ++i) {
			const int qx = x + i * step;
			if (qx < 0 || qx >= a.width) continue;
			const size_t q  = size_t(qy) * size_t(a.width) + size_t(qx);
			const float4 lq = in[q];
			const float w   = tapWeight(pa, pb, psky, plum, a.guideA[q], a.guideB[q], a.sky[q], luma(lq.x, lq.y, lq.z), invPlane, invDev, cSpline[i + 2] * cSpline[j + 2]);
			sr += w * lq.x;
			sg += w * lq.y;
			sb += w * lq.z;
			sv += w * w * lq.w;
			sw += w;
		}
	}
	float4 o = lp;
	if (sw > 0.0f) {
		const float scale = 1.0f / sw;
		o = make_float4(sr * scale, sg * scale, sb * scale, sv * scale * scale);
	}
	out[p] = o;
}

__global__ void remodulateKernel(const __grid_constant__ DenoiseArgs a, const float4* __restrict__ light) {
	const int x = blockIdx.x * blockDim.x + threadIdx.x;
	const int y = blockIdx.y * blockDim.y + threadIdx.y;
	if (x >= a.width || y >= a.height) return;
	const size_t p = size_t(y) * size_t(a.width) + size_t(x);
	const float4 l = light[p];
	const double share = 1.0 / (1.0 + double(a.length[p]) / 8.0);
	const float f[3]   = { l.x, l.y, l.z };
	for (int c = 0; c < 3; ++c) {
		const double dv   = divisorOf(double(__half2float(__ushort_as_half(a.albedo[3 * p + c]))));
		const double held = a.demodulated ? double(a.colour[3 * p + c]) * dv : double(a.colour[3 * p + c]);
		a.out[3 * p + c]  = float(double(f[c]) * dv * share + held * (1.0 - share));
	}
}

} // namespace

cudaError_t launchDenoise(const DenoiseArgs& args, cudaStream_t stream) {
	const dim3 block(kBlockX, kBlockY);
	const dim3 grid((args.width + kBlockX - 1) / kBlockX, (args.height + kBlockY - 1) / kBlockY);
	prepKernel<<<grid, block, 0, stream>>>(args);
	varianceKernel<<<grid, block, 0, stream>>>(args);
	// the spatial variance lives in lightB; the passes ping-pong B -> A -> B ...
	const float4* in = args.lightB;
	float4* out      = args.lightA;
	for (int pass = 0; pass < 4; ++pass) {
		atrousKernel<<<grid, block, 0, stream>>>(args, in, out, 1 << pass);
		const float4* t = in;
		in              = out;
		out             = const_cast<float4*>(t);
	}
	remodulateKernel<<<grid, block, 0, stream>>>(args, in);
	return cudaGetLastError();
}

} // namespace kdn
