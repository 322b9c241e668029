// The temporal member on the device, one thread a pixel: the geometry
// (headings, planes, where a point was seen before, the bilinear weights)
// in double as the reference computes it, the light in FP32
// (plugins/reconstruction/temporal/temporal.cpp, with a G-buffer, on the
// drawn grid: at a film factor above 1 a grid pixel's rays pass through the
// centre of the shown pixel its phase aims at, core/camera.cpp:51
// filmCentre, this frame's and the state before's).  Per pixel:
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
constexpr double kDepthShare = 0.03, kNormalCosine = 0.9;
constexpr float kAlbedoFloor = 1e-3f;
constexpr uint32_t kSky = 0xFFFFFFFFu;

struct V {
	float x, y, z;
};
__device__ __forceinline__ V v3(const float* a) { return { a[0], a[1], a[2] }; }
__device__ __forceinline__ V operator+(V a, V b) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
__device__ __forceinline__ V operator-(V a, V b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
__device__ __forceinline__ V operator*(V a, float s) { return { a.x * s, a.y * s, a.z * s }; }

// the geometry's vectors, in double
struct D {
	double x, y, z;
};
__device__ __forceinline__ D d3(const double* a) { return { a[0], a[1], a[2] }; }
__device__ __forceinline__ D operator+(D a, D b) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
__device__ __forceinline__ D operator-(D a, D b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
__device__ __forceinline__ D operator*(D a, double s) { return { a.x * s, a.y * s, a.z * s }; }
__device__ __forceinline__ double dotD(D a, D b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ __forceinline__ float half(const uint16_t* p, size_t i) { return __half2float(__ushort_as_half(p[i])); }

struct Surf {
	float distance;
	D normal;
	uint32_t leaf;
};

__device__ __forceinline__ Surf surfAt(const uint16_t* distance, const uint16_t* normal, const uint32_t* leaf, size_t k) {
	return { half(distance, k), { double(half(normal, 3 * k)), double(half(normal, 3 * k + 1)), double(half(normal, 3 * k + 2)) }, leaf[k] };
}

__device__ __forceinline__ bool skyOf(const Surf& s) { return s.leaf == kSky || !isfinite(s.distance); }

struct Plane {
	uint32_t leaf;
	D point, normal;
	double reach;
};

// :324 filmHeading
__device__ __forceinline__ D filmHeading(const TemporalCamera& c, double x, double y) { return d3(c.corner) + d3(c.across) * x + d3(c.down) * y; }

// :358 planeThrough over :345 surfacePointAlong
__device__ __forceinline__ Plane planeThrough(const Surf& s, D eye, D heading, double share) {
	if (skyOf(s)) return { kSky, { 0, 0, 0 }, { 0, 0, 0 }, 0.0 };
	const double distance = double(s.distance);
	return { s.leaf, eye + heading * (distance / sqrt(dotD(heading, heading))), s.normal, share * distance };
}

__device__ __forceinline__ bool sameLeaf(uint32_t a, uint32_t b, bool recounted) { return recounted ? ((a == kSky) == (b == kSky)) : a == b; }

// :397 onPlane
__device__ __forceinline__ bool onPlane(const Plane& p, const Plane& other, bool recounted) {
	if (!sameLeaf(other.leaf, p.leaf, recounted)) return false;
	if (p.leaf == kSky) return true;
	if (dotD(other.normal, p.normal) < kNormalCosine) return false;
	return fabs(dotD(other.point - p.point, p.normal)) <= p.reach;
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
	return onPlane(p, planeThrough(s, d3(a.now.eye), filmHeading(a.now, double(x) + double(a.centre[0]), double(y) + double(a.centre[1])), kDepthShare), false);
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
		const D heading   = filmHeading(a.now, double(x) + double(a.centre[0]), double(y) + double(a.centre[1]));
		const Plane plane = planeThrough(centre, d3(a.now.eye), heading, kDepthShare);
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
				// :584 surfacedHistory, :418 placeBefore, :495 fetchedHistory
				const D along      = plane.leaf == kSky ? heading : plane.point - d3(a.before.eye);
				const double ahead = dotD(along, d3(a.before.forward));
				if (ahead > 0) {
					const double scale = 1 / ahead;
					const double px    = dotD(along, d3(a.before.acrossInverse)) * scale + 0.5 * a.before.width;
					const double py    = dotD(along, d3(a.before.downInverse)) * scale + 0.5 * a.before.height;
					if (px >= 0 && px < a.before.width && py >= 0 && py < a.before.height) {
						const double ax = px - double(a.centreBefore[0]), ay = py - double(a.centreBefore[1]);
						const int lx = int(floor(ax)), ly = int(floor(ay));
						const double tx = ax - double(lx), ty = ay - double(ly);
						D colour = { 0, 0, 0 };
						double moment = 0.0, weight = 0.0;
						float length  = 0.0f;
						for (int j = 0; j < 2; ++j) {
							for (int i = 0; i < 2; ++i) {
								const int cx = lx + i, cy = ly + j;
								const double w = (i == 0 ? 1 - tx : tx) * (j == 0 ? 1 - ty : ty);
								if (!(w > 0 && cx >= 0 && cx < a.width && cy >= 0 && cy < a.height)) continue;
								const size_t c = size_t(cy) * size_t(a.width) + size_t(cx);
								const float lastLength = io.before_length[c];
								if (!(lastLength > 0.0f)) continue;
								const Surf last = surfAt(io.before_distance, io.before_normal, io.before_leaf, c);
								const Plane lastPlane = planeThrough(last, d3(a.before.eye),
								                                     filmHeading(a.before, double(cx) + double(a.centreBefore[0]), double(cy) + double(a.centreBefore[1])), 0.0);
								if (!onPlane(plane, lastPlane, a.recounted != 0)) continue;
								const float* lc = io.before_colour + 3 * c;
								colour = colour + D { double(lc[0]), double(lc[1]), double(lc[2]) } * w;
								moment += double(io.before_moment[c]) * w;
								length += float(double(lastLength) * w);
								weight += w;
							}
						}
						if (weight > 0) {
							// :470 summedHistory
							found         = true;
							history       = { float(colour.x * (1 / weight)), float(colour.y * (1 / weight)), float(colour.z * (1 / weight)) };
							historyMoment = float(moment / weight);
							historyLength = float(double(length) / weight);
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

void filmCentreOf(uint32_t factor, uint32_t phase, float centre[2]) {
	const uint32_t f = factor > 1 ? factor : 1;
	centre[0]        = float((double(f > 1 ? phase % f : 0) + 0.5) / double(f));
	centre[1]        = float((double(f > 1 ? phase / f : 0) + 0.5) / double(f));
}

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
	const double acrossScale = 1 / aa, downScale = 1 / dd;
	for (int a = 0; a < 3; ++a) {
		c.eye[a]           = l[a];
		c.forward[a]       = l[3 + a];
		c.corner[a]        = corner[a];
		c.across[a]        = across[a];
		c.down[a]          = down[a];
		c.acrossInverse[a] = across[a] * acrossScale;
		c.downInverse[a]   = down[a] * downScale;
	}
	c.width  = double(width);
	c.height = double(height);
	return c;
}

cudaError_t launchTemporal(const TemporalArgs& args, cudaStream_t stream) {
	const int n = args.width * args.height;
	if (n <= 0) return cudaSuccess;
	temporalKernel<<<(n + 255) / 256, 256, 0, stream>>>(args);
	return cudaGetLastError();
}

} // namespace kdn
