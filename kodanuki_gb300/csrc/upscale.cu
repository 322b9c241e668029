// The upscale member on the device (plugins/reconstruction/upscale/
// upscale.cpp:611 upscaledFrame), one thread a shown pixel, with the
// reference's own number types and order of operations (tones in float,
// positions, lenses and history colours in double; compiled without FMA
// contraction) so that it answers as the reference does to the bit.
//
// A first kernel turns each drawn pixel into its tone (:179 toneOf: luma,
// orange, green of the colour tone-mapped by 1 / (1 + max)) and depth (the
// G-buffer's distance, sky where there is none); the second, for each shown
// pixel, gathers the 3x3 drawn samples around it with the axes' sharp and
// fill weights (:317 upscaleGather), the box's mean, deviation and range
// (:273 upscaleStatsAt), finds where its nearest surface was seen by the
// frame before (:357 seenFrom), keeps the history where the depth there
// matches (:418 sameDepth), reads it by five bilinear taps (:476 historyAt),
// clamps it to the box (:481 clampedHistory) and blends (:497 blendedTone).
// The state it leaves a shown pixel is its colour (float values, as the
// reference's untonedColour makes them) and the box's closest depth.
#include "upscale.h"

#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>

namespace kdn {

namespace {

// upscale.cpp:17-34
constexpr float kCeiling = 60000.0f, kFloor = 1e-4f;
constexpr float kAlpha = 0.5f, kAlphaSettle = 1.0f, kAlphaFast = 1.0f, kAlphaLeast = 1e-5f, kAlphaMoving = 0.15f;
constexpr double kFast = 8.0, kStill = 1.0;
constexpr float kClampMoving = 1.25f, kClampStill = 6.0f, kStillMargin = 1.0f;
constexpr float kDepthShare = 0.03f, kSpreadShare = 0.25f, kLeastWeight = 1e-6f;
constexpr int kBlock = 256;

struct Tone {
	float l, o, g;
};
__device__ __forceinline__ Tone operator+(Tone a, Tone b) { return { a.l + b.l, a.o + b.o, a.g + b.g }; }
__device__ __forceinline__ Tone operator-(Tone a, Tone b) { return { a.l - b.l, a.o - b.o, a.g - b.g }; }
__device__ __forceinline__ Tone operator*(Tone a, float s) { return { a.l * s, a.o * s, a.g * s }; }
// std::min / std::max as the reference calls them: (b < a) ? b : a, (a < b) ? b : a
__device__ __forceinline__ float least(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float most(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ Tone least(Tone a, Tone b) { return { least(a.l, b.l), least(a.o, b.o), least(a.g, b.g) }; }
__device__ __forceinline__ Tone most(Tone a, Tone b) { return { most(a.l, b.l), most(a.o, b.o), most(a.g, b.g) }; }
__device__ __forceinline__ Tone squared(Tone a) { return { a.l * a.l, a.o * a.o, a.g * a.g }; }
__device__ __forceinline__ Tone root(Tone a) { return { sqrtf(most(a.l, 0.0f)), sqrtf(most(a.o, 0.0f)), sqrtf(most(a.g, 0.0f)) }; }
__device__ __forceinline__ Tone clamped(Tone a, Tone low, Tone high) { return least(most(a, low), high); }
__device__ __forceinline__ Tone mixed(Tone a, Tone b, float share) { return a + (b - a) * share; }
__device__ __forceinline__ Tone spread(Tone a, float s) { return { a.l + s, a.o + s, a.g + s }; }

// :179 toneOf of a colour of doubles
__device__ __forceinline__ Tone toneOf(double red, double green, double blue) {
	const float r0 = least(float(red), kCeiling), g0 = least(float(green), kCeiling), b0 = least(float(blue), kCeiling);
	const float scale = 1.0f / (1.0f + most(r0, most(g0, b0)));
	const float r = r0 * scale, g = g0 * scale, b = b0 * scale;
	return { 0.25f * r + 0.5f * g + 0.25f * b, 0.5f * r - 0.5f * b, -0.25f * r + 0.5f * g - 0.25f * b };
}

__device__ __forceinline__ Tone toneAt(const float4* samples, size_t k) {
	const float4 s = samples[k];
	return { s.x, s.y, s.z };
}

__global__ void __launch_bounds__(kBlock) samplesKernel(const float* internal, const uint16_t* distance, int n, float4* samples) {
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		const Tone t = toneOf(double(internal[3 * k]), double(internal[3 * k + 1]), double(internal[3 * k + 2]));
		float depth  = INFINITY;
		if (distance != nullptr) {
			const float d = __half2float(__ushort_as_half(distance[k]));
			depth         = isfinite(d) ? d : INFINITY;
		}
		samples[k] = make_float4(t.l, t.o, t.g, depth);
	}
}

struct D3 {
	double x, y, z;
};
__device__ __forceinline__ D3 lensPart(const double* l, int k) { return { l[3 * k], l[3 * k + 1], l[3 * k + 2] }; }
__device__ __forceinline__ double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

struct Seen {
	bool inside;
	double x, y;
	float depth;
};

// :357 seenFrom
__device__ __forceinline__ Seen seenFrom(const double* before, int width, int height, D3 along, float depth) {
	const double ahead = dot(along, lensPart(before, 1));
	if (!(ahead > 1e-9)) return { false, 0.0, 0.0, 0.0f };
	const double u = dot(along, lensPart(before, 2)) / (ahead * before[12] * before[13]);
	const double v = dot(along, lensPart(before, 3)) / (ahead * before[12]);
	const double x = (u + 1) * 0.5 * double(width);
	const double y = (1 - v) * 0.5 * double(height);
	if (!(x >= 0 && x < double(width) && y >= 0 && y < double(height))) return { false, 0.0, 0.0, 0.0f };
	return { true, x, y, depth };
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (hi < v ? hi : v); }

struct History {
	const float4* state;
	int width, height;
	__device__ float4 at(int x, int y) const { return state[size_t(clampi(y, 0, height - 1)) * size_t(width) + size_t(clampi(x, 0, width - 1))]; }
};

// :428 historyShare, :432 historyIndex
__device__ __forceinline__ double historyShare(double at) { return at - 0.5 - floor(at - 0.5); }
__device__ __forceinline__ int historyIndex(double at) { return int(floor(at - 0.5)); }

// :436 historyAcross, :442 historyDown, scaled by a tap's weight
__device__ __forceinline__ D3 across(const History& h, double x, int y, double weight) {
	const double share = historyShare(x);
	const int column   = historyIndex(x);
	const float4 a = h.at(column, y), b = h.at(column + 1, y);
	return { (double(a.x) * (1 - share) + double(b.x) * share) * weight, (double(a.y) * (1 - share) + double(b.y) * share) * weight,
		     (double(a.z) * (1 - share) + double(b.z) * share) * weight };
}

__device__ __forceinline__ D3 down(const History& h, int x, double y, double weight) {
	const double share = historyShare(y);
	const int row      = historyIndex(y);
	const float4 a = h.at(x, row), b = h.at(x, row + 1);
	return { (double(a.x) * (1 - share) + double(b.x) * share) * weight, (double(a.y) * (1 - share) + double(b.y) * share) * weight,
		     (double(a.z) * (1 - share) + double(b.z) * share) * weight };
}

struct Taps {
	int before;
	double middle;
	int after;
	double middleWeight, beforeWeight, afterWeight;
};

// :460 upscaleTaps
__device__ __forceinline__ Taps tapsAt(double at) {
	const double centre = floor(at - 0.5) + 0.5;
	const double f      = at - centre;
	const double w0     = f * (-0.5 + f * (1 - 0.5 * f));
	const double w1     = 1 + f * f * (-2.5 + 1.5 * f);
	const double w2     = f * (0.5 + f * (2 - 1.5 * f));
	const double w3     = f * f * (-0.5 + 0.5 * f);
	return { int(centre - 1.5), centre + w2 / (w1 + w2), int(centre + 1.5), w1 + w2, w0, w3 };
}

// :476 historyAt
__device__ __forceinline__ D3 historyAt(const History& h, const Seen& s) {
	const Taps ax = tapsAt(s.x), dy = tapsAt(s.y);
	const D3 top    = across(h, ax.middle, dy.before, ax.middleWeight * dy.beforeWeight);
	const D3 left   = down(h, ax.before, dy.middle, ax.beforeWeight * dy.middleWeight);
	// :448 bilinearHistory
	const double share = historyShare(dy.middle);
	const int row      = historyIndex(dy.middle);
	const D3 upper = across(h, ax.middle, row, 1.0), lower = across(h, ax.middle, row + 1, 1.0);
	const double wm = ax.middleWeight * dy.middleWeight;
	const D3 middle = { (upper.x * (1 - share) + lower.x * share) * wm, (upper.y * (1 - share) + lower.y * share) * wm, (upper.z * (1 - share) + lower.z * share) * wm };
	const D3 right  = down(h, ax.after, dy.middle, ax.afterWeight * dy.middleWeight);
	const D3 bottom = across(h, ax.middle, dy.after, ax.middleWeight * dy.afterWeight);
	const double ends  = dy.beforeWeight + dy.middleWeight + dy.afterWeight;
	const double total = ax.middleWeight * ends + dy.middleWeight * (ax.beforeWeight + ax.afterWeight);
	const double scale = 1 / total;
	const double r = (top.x + left.x + middle.x + right.x + bottom.x) * scale;
	const double g = (top.y + left.y + middle.y + right.y + bottom.y) * scale;
	const double b = (top.z + left.z + middle.z + right.z + bottom.z) * scale;
	return { r < 0.0 ? 0.0 : r, g < 0.0 ? 0.0 : g, b < 0.0 ? 0.0 : b };
}

// :409 depthMatches
__device__ __forceinline__ bool depthMatches(float last, float depth, float slack) {
	if (!(depth < INFINITY)) return !(last < INFINITY);
	return fabsf(last - depth) <= kDepthShare * depth + slack;
}

__global__ void __launch_bounds__(kBlock) upscaleKernel(const __grid_constant__ UpscaleArgs a) {
	const int n = a.width * a.height;
	const History history { a.before_state, a.width, a.height };
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		const int x = k % a.width, y = k / a.width;
		const UpscaleAxis& column = a.columns[x];
		const UpscaleAxis& row    = a.rows[y];
		// :273 upscaleStatsAt of the box around the nearest sample (clamped
		// taps: the gather's own 3x3), then :317 upscaleGather
		const float big = 3.402823466e+38f;
		Tone sum = { 0, 0, 0 }, squares = { 0, 0, 0 }, low = { big, big, big }, high = { -big, -big, -big };
		float closest = INFINITY, farthest = 0.0f;
		const int bx = column.box - 1, by = row.box - 1;
		for (int dy = -1; dy <= 1; ++dy) {
			for (int dx = -1; dx <= 1; ++dx) {
				const float4 s = a.samples[size_t(clampi(by + dy, 0, a.drawnHeight - 1)) * size_t(a.drawnWidth) + size_t(clampi(bx + dx, 0, a.drawnWidth - 1))];
				const Tone t   = { s.x, s.y, s.z };
				sum            = sum + t;
				squares        = squares + squared(t);
				low            = least(low, t);
				high           = most(high, t);
				closest        = least(closest, s.w);
				if (s.w < INFINITY) farthest = most(farthest, s.w);
			}
		}
		const Tone mean      = sum * (1.0f / 9);
		const Tone deviation = root(squares * (1.0f / 9) - squared(mean));
		Tone sharp = { 0, 0, 0 }, fill = { 0, 0, 0 };
		float sharpWeight = 0.0f, fillWeight = 0.0f;
		for (int dy = 0; dy < 3; ++dy) {
			for (int dx = 0; dx < 3; ++dx) {
				const Tone t       = toneAt(a.samples, size_t(row.taps[dy]) * size_t(a.drawnWidth) + size_t(column.taps[dx]));
				const float near   = column.sharp[dx] * row.sharp[dy];
				const float spread = column.fill[dx] * row.fill[dy];
				sharp              = sharp + t * near;
				fill               = fill + t * spread;
				sharpWeight += near;
				fillWeight += spread;
			}
		}
		fill = clamped(fill * (1.0f / fillWeight), low, high);
		// :515 upscaledTone
		Tone out = fill;
		if (a.kept) {
			// :342 upscaleHeading through the shown pixel's centre, :381 seenBefore
			const double u = 2 * (double(x) + 0.5) / double(a.width) - 1;
			const double v = 1 - 2 * (double(y) + 0.5) / double(a.height);
			const D3 forward = lensPart(a.now, 1), right = lensPart(a.now, 2), up = lensPart(a.now, 3);
			const double sideways = u * a.now[12] * a.now[13], upward = v * a.now[12];
			D3 direction = { forward.x + right.x * sideways + up.x * upward, forward.y + right.y * sideways + up.y * upward,
				             forward.z + right.z * sideways + up.z * upward };
			const double size = sqrt(dot(direction, direction));
			if (size > 0) direction = { direction.x / size, direction.y / size, direction.z / size };
			Seen seen;
			if (!(closest < INFINITY)) {
				seen = seenFrom(a.before, a.width, a.height, direction, INFINITY);
			} else {
				const D3 eye = lensPart(a.now, 0), then = lensPart(a.before, 0);
				const double c = double(closest);
				const D3 along = { eye.x + direction.x * c - then.x, eye.y + direction.y * c - then.y, eye.z + direction.z * c - then.z };
				seen = seenFrom(a.before, a.width, a.height, along, float(sqrt(dot(along, along))));
			}
			// :511 upscaleSlack, :418 sameDepth
			const float slack = least(farthest - closest, kSpreadShare * closest);
			bool same         = false;
			if (seen.inside) {
				const int hx = int(floor(seen.x - 0.5)), hy = int(floor(seen.y - 0.5));
				for (int dy = 0; dy <= 1 && !same; ++dy) {
					for (int dx = 0; dx <= 1 && !same; ++dx) same = depthMatches(history.at(hx + dx, hy + dy).w, seen.depth, slack);
				}
			}
			if (same) {
				// :497 blendedTone
				const double mx = seen.x - (double(x) + 0.5), my = seen.y - (double(y) + 0.5);
				const double moved  = sqrt(mx * mx + my * my);
				const D3 held       = historyAt(history, seen);
				const Tone toned    = toneOf(held.x, held.y, held.z);
				const float motion  = float(moved / kStill < 1.0 ? moved / kStill : 1.0);
				// :481 clampedHistory
				const float width   = kClampStill + (kClampMoving - kClampStill) * motion;
				const float margin  = kStillMargin * (1 - motion);
				const Tone lowClamp  = spread(mean - deviation * width, -margin);
				const Tone highClamp = spread(mean + deviation * width, margin);
				Tone last;
				if (!(motion > 0)) {
					last = clamped(toned, lowClamp, highClamp);
				} else {
					// :469 nearestBox
					const int cx = column.taps[1], cy = row.taps[1];
					const Tone p = toneAt(a.samples, size_t(cy) * size_t(a.drawnWidth) + size_t(cx));
					const Tone q = toneAt(a.samples, size_t(cy) * size_t(a.drawnWidth) + size_t(column.toward));
					const Tone r = toneAt(a.samples, size_t(row.toward) * size_t(a.drawnWidth) + size_t(cx));
					const Tone e = toneAt(a.samples, size_t(row.toward) * size_t(a.drawnWidth) + size_t(column.toward));
					const Tone boxLow  = least(least(p, q), least(r, e));
					const Tone boxHigh = most(most(p, q), most(r, e));
					last = clamped(toned, mixed(lowClamp, most(lowClamp, boxLow), motion), mixed(highClamp, least(highClamp, boxHigh), motion));
				}
				const float speed = float(moved / kFast < 1.0 ? moved / kFast : 1.0);
				const float base  = a.settling ? kAlphaSettle : kAlpha;
				float alpha       = (base + (kAlphaFast - base) * speed) * sharpWeight;
				alpha             = alpha < kAlphaLeast ? kAlphaLeast : (1.0f < alpha ? 1.0f : alpha);
				const Tone sharpTone = sharp * (1.0f / most(sharpWeight, kLeastWeight));
				out = mixed(mixed(last, sharpTone, alpha), fill, kAlphaMoving * speed);
			}
		}
		// :190 untonedColour
		const float r = most(out.l + out.o - out.g, 0.0f);
		const float g = most(out.l + out.g, 0.0f);
		const float b = most(out.l - out.o - out.g, 0.0f);
		const float scale = 1.0f / most(1.0f - most(r, most(g, b)), kFloor);
		const float cr = r * scale, cg = g * scale, cb = b * scale;
		a.after_state[k]  = make_float4(cr, cg, cb, closest);
		a.image[3 * k]     = cr;
		a.image[3 * k + 1] = cg;
		a.image[3 * k + 2] = cb;
	}
}

// plugins/reconstruction/upsample/upsample.cpp:15 upsampleTap: the two
// drawn pixels either side of a shown pixel's centre and the share of the
// second, clamped to the drawn frame
struct UpsampleTap {
	int first, second;
	float share;
};

__device__ __forceinline__ UpsampleTap upsampleTap(int shown, int factor, int drawn) {
	const double centre  = (double(shown) + 0.5) / double(factor) - 0.5;
	const double clamped = centre < 0.0 ? 0.0 : (double(drawn - 1) < centre ? double(drawn - 1) : centre);
	const int first      = int(clamped);
	return { first, first + 1 < drawn - 1 ? first + 1 : drawn - 1, float(clamped - double(first)) };
}

// upsample.cpp:63 upsampledImage, :41 blendedChannel: bilinear in float
__global__ void __launch_bounds__(kBlock) upsampleKernel(int width, int height, int factor, const float* drawn, float* shown) {
	const int n = width * height, dw = width / factor, dh = height / factor;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		const int x = k % width, y = k / width;
		const UpsampleTap row = upsampleTap(y, factor, dh), column = upsampleTap(x, factor, dw);
		const float* upper    = drawn + size_t(row.first) * size_t(dw) * 3;
		const float* lower    = drawn + size_t(row.second) * size_t(dw) * 3;
		for (int c = 0; c < 3; ++c) {
			const float a = upper[3 * column.first + c], b = upper[3 * column.second + c];
			const float d = lower[3 * column.first + c], e = lower[3 * column.second + c];
			const float top    = a + (b - a) * column.share;
			const float bottom = d + (e - d) * column.share;
			shown[size_t(k) * 3 + c] = top + (bottom - top) * row.share;
		}
	}
}

double catmullRom(double t) {
	const double a = std::fabs(t);
	if (a < 1) return (1.5 * a - 2.5) * a * a + 1;
	if (a < 2) return ((-0.5 * a + 2.5) * a - 4) * a + 2;
	return 0;
}

} // namespace

void upscaleAxes(int factor, int place, int count, int shown, UpscaleAxis* out) {
	// :665 upscaleJitter
	const double jitter = (double(place) + 0.5) / double(factor) - 0.5;
	for (int s = 0; s < shown; ++s) {
		const double internal = (double(s) + 0.5) / double(factor);
		const int nearest     = int(std::floor(internal - jitter));
		const double first    = double(nearest) + 0.5 + jitter - internal;
		UpscaleAxis& a        = out[s];
		for (int d = 0; d < 3; ++d) {
			const int at        = std::min(std::max(nearest + d - 1, 0), count - 1);
			const double offset = (double(at) + 0.5 + jitter - internal) * double(factor);
			a.taps[d]           = at;
			a.sharp[d]          = float(std::exp(-8.0 * offset * offset));
			a.fill[d]           = float(catmullRom(first + double(d - 1)));
		}
		// :564 towardSpot
		const double centre = double(a.taps[1]) + 0.5 + jitter - internal;
		const int toward    = centre > 0 ? -1 : (centre < 0 ? 1 : 0);
		a.toward            = std::min(std::max(a.taps[1] + toward, 0), count - 1);
		a.box               = nearest + 1;
		a.pad               = 0;
	}
}

cudaError_t launchUpscale(const UpscaleArgs& args, cudaStream_t stream, int smCount) {
	const int drawn = args.drawnWidth * args.drawnHeight, shown = args.width * args.height;
	const int most  = smCount * 8;
	samplesKernel<<<std::min((drawn + kBlock - 1) / kBlock, most), kBlock, 0, stream>>>(args.internal, args.distance, drawn, args.samples);
	upscaleKernel<<<std::min((shown + kBlock - 1) / kBlock, most), kBlock, 0, stream>>>(args);
	return cudaGetLastError();
}

cudaError_t launchUpsample(int width, int height, int factor, const float* drawn, float* shown, cudaStream_t stream, int smCount) {
	const int n = width * height;
	upsampleKernel<<<std::min((n + kBlock - 1) / kBlock, smCount * 8), kBlock, 0, stream>>>(width, height, factor, drawn, shown);
	return cudaGetLastError();
}

} // namespace kdn
