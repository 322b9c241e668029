// The temporal member on the device, one thread a pixel, in FP32
// (plugins/reconstruction/temporal/temporal.cpp, at a film factor of 1 with
// a G-buffer).  Per pixel:
//   - the 3x3 neighbourhood of this frame's demodulated light (:903
//     neighbourhoodOf): mean, deviation;
//   - whether the pixel's sample met the G-buffer's surface (:244
//     aimedSurface);
//   - the history: the pixel's own on a still camera (:570 stillHistory),
//     else the frame before's pixels around where the G-buffer's point was
//     seen, bilinear over those whose surface lies on this pixel's plane
//     (:584 surfacedHistory, :495 fetchedHistory);
//   - the blend (:796 freshBlend, :836 heldBlend with :810 heldColour's
//     clamp while the history is young or the camera moves);
//   - the shown light, the blend times the G-buffer's albedo (:220).
// The state it leaves is the colour, moment and length; what a pixel shows
// is the G-buffer's surface, which the frame keeps.
#include "temporal.h"

#include <cuda_fp16.h>

#include <cmath>

namespace kdn {

namespace {

constexpr float kMovingCap = 32.0f, kStillCap = 256.0f, kYoungLength = 8.0f;
constexpr float kMovingSpread = 1.25f, kStillSpread = 6.0f;
constexpr float kDepthShare = 0.03f, kNormalCosine = 0.9f, kAlbedoFloor = 1e-3f;
constexpr uint32_t kSky = 0xFFFFFFFFu;

struct V {
	float x, y, z;
};
__device__ __forceinline__ V v3(const float* a) { return { a[0], a[1], a[2] }; }
__device__ __forceinline__ V operator+(V a, V b) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
__device__ __forceinline__ V operator-(V a, V b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
__device__ __forceinline__ V operator*(V a, float s) { return { a.x * s, a.y * s, a.z * s }; }
__device__ __forceinline__ float dotV(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ __forceinline__ float half(const uint16_t* p, size_t i) { return __half2float(__ushort_as_half(p[i])); }

struct Surf {
	float distance;
	V normal;
	uint32_t leaf;
};

__device__ __forceinline__ Surf surfAt(const uint16_t* distance, const uint16_t* normal, const uint32_t* leaf, size_t k) {
	return { half(distance, k), { half(normal, 3 * k), half(normal, 3 * k + 1), half(normal, 3 * k + 2) }, leaf[k] };
}

__device__ __forceinline__ bool skyOf(const Surf& s) { return s.leaf == kSky || !isfinite(s.distance); }

struct Plane {
	uint32_t leaf;
	V point, normal;
	float reach;
};

__device__ __forceinline__ V filmHeading(const TemporalCamera& c, float x, float y) { return v3(c.corner) + v3(c.across) * x + v3(c.down) * y; }

// :358 planeThrough
__device__ __forceinline__ Plane planeThrough(const Surf& s, V eye, V heading, float reach) {
	if (skyOf(s)) return { kSky, { 0, 0, 0 }, { 0, 0, 0 }, 0.0f };
	return { s.leaf, eye + heading * (s.distance / sqrtf(dotV(heading, heading))), s.normal, reach * s.distance };
}

__device__ __forceinline__ bool sameLeaf(uint32_t a, uint32_t b, bool recounted) { return recounted ? ((a == kSky) == (b == kSky)) : a == b; }

// :397 onPlane
__device__ __forceinline__ bool onPlane(const Plane& p, const Plane& other, bool recounted) {
	if (!sameLeaf(other.leaf, p.leaf, recounted)) return false;
	if (p.leaf == kSky) return true;
	if (dotV(other.normal, p.normal) < kNormalCosine) return false;
	return fabsf(dotV(other.point - p.point, p.normal)) <= p.reach;
}

__device__ __forceinline__ float divisorOf(float albedo) { return albedo < kAlbedoFloor ? 1.0f : albedo; }

// :224 sampleLight: the light divided by the sample's albedo
__device__ __forceinline__ V sampleLight(const kdn_temporal_buffers& io, size_t k) {
	return { io.light[3 * k] / divisorOf(half(io.first_albedo, 3 * k)), io.light[3 * k + 1] / divisorOf(half(io.first_albedo, 3 * k + 1)),
		     io.light[3 * k + 2] / divisorOf(half(io.first_albedo, 3 * k + 2)) };
}

__device__ __forceinline__ float luminance(V c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

__device__ __forceinline__ size_t clampedPixel(int x, int y, int w, int h) {
	x = x < 0 ? 0 : (x > w - 1 ? w - 1 : x);
	y = y < 0 ? 0 : (y > h - 1 ? h - 1 : y);
	return size_t(y) * size_t(w) + size_t(x);
}

__device__ __forceinline__ bool sampleOnPlane(const TemporalArgs& a, const Plane& p, size_t k) {
	const int x = int(k % size_t(a.width)), y = int(k / size_t(a.width));
	const Surf s = surfAt(a.io.first_distance, a.io.first_normal, a.io.first_leaf, k);
	return onPlane(p, planeThrough(s, v3(a.now.eye), filmHeading(a.now, float(x) + 0.5f, float(y) + 0.5f), kDepthShare), false);
}

__global__ void temporalKernel(TemporalArgs a) {
	const int n = a.width * a.height;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
		const int x = k % a.width, y = k / a.width;
		const kdn_temporal_buffers& io = a.io;
		// the 3x3 neighbourhood of this frame's light
		V sum = { 0, 0, 0 }, squares = { 0, 0, 0 };
		for (int dy = -1; dy <= 1; ++dy) {
			for (int dx = -1; dx <= 1; ++dx) {
				const V c = sampleLight(io, clampedPixel(x + dx, y + dy, a.width, a.height));
				sum       = sum + c;
				squares   = squares + V { c.x * c.x, c.y * c.y, c.z * c.z };
			}
		}
		const V mean = sum * (1.0f / 9.0f);
		const V deviation = { sqrtf(fmaxf(squares.x / 9.0f - mean.x * mean.x, 0.0f)), sqrtf(fmaxf(squares.y / 9.0f - mean.y * mean.y, 0.0f)),
			                  sqrtf(fmaxf(squares.z / 9.0f - mean.z * mean.z, 0.0f)) };
		const Surf first  = surfAt(io.first_distance, io.first_normal, io.first_leaf, k);
		const Surf centre = surfAt(io.centre_distance, io.centre_normal, io.centre_leaf, k);
		const bool aimed  = (skyOf(first) ? kSky : first.leaf) == (skyOf(centre) ? kSky : centre.leaf);
		const V heading   = filmHeading(a.now, float(x) + 0.5f, float(y) + 0.5f);
		const Plane plane = planeThrough(centre, v3(a.now.eye), heading, kDepthShare);
		// the history
		bool found = false;
		V history  = { 0, 0, 0 };
		float historyMoment = 0.0f, historyLength = 0.0f;
		if (a.kept) {
			if (!a.moved) {
				const float length = io.before_length[k];
				if (length > 0.0f) {
					found         = true;
					history       = v3(io.before_colour + 3 * k);
					historyMoment = io.before_moment[k];
					historyLength = length;
				}
			} else {
				const V along     = plane.leaf == kSky ? heading : plane.point - v3(a.before.eye);
				const float ahead = dotV(along, v3(a.before.forward));
				if (ahead > 0.0f) {
					const float scale = 1.0f / ahead;
					const float px    = dotV(along, v3(a.before.acrossInverse)) * scale + 0.5f * a.before.width;
					const float py    = dotV(along, v3(a.before.downInverse)) * scale + 0.5f * a.before.height;
					if (px >= 0.0f && px < a.before.width && py >= 0.0f && py < a.before.height) {
						const float ax = px - 0.5f, ay = py - 0.5f;
						const int lx = int(floorf(ax)), ly = int(floorf(ay));
						const float tx = ax - float(lx), ty = ay - float(ly);
						V colour = { 0, 0, 0 };
						float moment = 0.0f, length = 0.0f, weight = 0.0f;
						for (int j = 0; j < 2; ++j) {
							for (int i = 0; i < 2; ++i) {
								const int cx = lx + i, cy = ly + j;
								const float w = (i == 0 ? 1.0f - tx : tx) * (j == 0 ? 1.0f - ty : ty);
								if (!(w > 0.0f && cx >= 0 && cx < a.width && cy >= 0 && cy < a.height)) continue;
								const size_t c = size_t(cy) * size_t(a.width) + size_t(cx);
								const float lastLength = io.before_length[c];
								if (!(lastLength > 0.0f)) continue;
								const Surf last = surfAt(io.before_distance, io.before_normal, io.before_leaf, c);
								const Plane lastPlane = planeThrough(last, v3(a.before.eye), filmHeading(a.before, float(cx) + 0.5f, float(cy) + 0.5f), 0.0f);
								if (!onPlane(plane, lastPlane, a.recounted != 0)) continue;
								colour = colour + v3(io.before_colour + 3 * c) * w;
								moment += io.before_moment[c] * w;
								length += lastLength * w;
								weight += w;
							}
						}
						if (weight > 0.0f) {
							found         = true;
							history       = colour * (1.0f / weight);
							historyMoment = moment / weight;
							historyLength = length / weight;
						}
					}
				}
			}
		}
		V colour;
		float moment, length;
		if (!found) {
			// :796 freshBlend; not aimed: :754 jointFilled
			if (aimed || sampleOnPlane(a, plane, size_t(k))) {
				colour = sampleLight(io, size_t(k));
			} else {
				V fill = { 0, 0, 0 };
				float weight = 0.0f;
				for (int dy = -1; dy <= 1; ++dy) {
					for (int dx = -1; dx <= 1; ++dx) {
						const size_t j = clampedPixel(x + dx, y + dy, a.width, a.height);
						if (!sampleOnPlane(a, plane, j)) continue;
						fill = fill + sampleLight(io, j);
						weight += 1.0f;
					}
				}
				colour = weight > 0.0f ? fill * (1.0f / weight) : sampleLight(io, size_t(k));
			}
			const float l = luminance(colour);
			moment        = l * l;
			length        = aimed ? 1.0f : 0.0f;
		} else {
			// :836 heldBlend
			const float cap  = a.moved ? kMovingCap : kStillCap;
			const float held = fminf(historyLength, cap);
			V keep           = history;
			if (a.moved || historyLength < kYoungLength) {
				const float spread = a.moved ? kMovingSpread : kStillSpread;
				keep = { fminf(fmaxf(history.x, mean.x - spread * deviation.x), mean.x + spread * deviation.x),
					     fminf(fmaxf(history.y, mean.y - spread * deviation.y), mean.y + spread * deviation.y),
					     fminf(fmaxf(history.z, mean.z - spread * deviation.z), mean.z + spread * deviation.z) };
			}
			if (!aimed) {
				colour = keep;
				moment = historyMoment;
				length = held;
			} else {
				const V sample    = sampleLight(io, size_t(k));
				const float l     = luminance(sample);
				const float alpha = fmaxf(1.0f / (held + 1.0f), 1.0f / cap);
				colour            = keep * (1.0f - alpha) + sample * alpha;
				moment            = historyMoment * (1.0f - alpha) + l * l * alpha;
				length            = fminf(held + 1.0f, cap);
			}
		}
		io.colour[3 * k]     = colour.x;
		io.colour[3 * k + 1] = colour.y;
		io.colour[3 * k + 2] = colour.z;
		io.moment[k]         = moment;
		io.length[k]         = length;
		if (io.image) {
			io.image[3 * k]     = colour.x * divisorOf(half(io.centre_albedo, 3 * k));
			io.image[3 * k + 1] = colour.y * divisorOf(half(io.centre_albedo, 3 * k + 1));
			io.image[3 * k + 2] = colour.z * divisorOf(half(io.centre_albedo, 3 * k + 2));
		}
	}
}

} // namespace

TemporalCamera temporalCameraOf(const double l[14], int width, int height) {
	const double sideways = l[12] * l[13], reach = l[12];
	double across[3], down[3], corner[3];
	double aa = 0, dd = 0;
	for (int a = 0; a < 3; ++a) {
		across[a] = l[6 + a] * (2 * sideways / double(width));
		down[a]   = l[9 + a] * (-2 * reach / double(height));
		corner[a] = l[3 + a] - l[6 + a] * sideways + l[9 + a] * reach;
		aa += across[a] * across[a];
		dd += down[a] * down[a];
	}
	TemporalCamera c {};
	for (int a = 0; a < 3; ++a) {
		c.eye[a]           = float(l[a]);
		c.forward[a]       = float(l[3 + a]);
		c.corner[a]        = float(corner[a]);
		c.across[a]        = float(across[a]);
		c.down[a]          = float(down[a]);
		c.acrossInverse[a] = float(across[a] / aa);
		c.downInverse[a]   = float(down[a] / dd);
	}
	c.width  = float(width);
	c.height = float(height);
	return c;
}

cudaError_t launchTemporal(const TemporalArgs& args, cudaStream_t stream) {
	const int n = args.width * args.height;
	if (n <= 0) return cudaSuccess;
	temporalKernel<<<(n + 255) / 256, 256, 0, stream>>>(args);
	return cudaGetLastError();
}

} // namespace kdn
