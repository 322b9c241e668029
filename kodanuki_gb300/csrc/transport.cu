// The path-transport kernels, wavefront form: K-cam, K-shade (arrive, meet
// with MIS, aim with a one-sample reservoir, BSDF sample, roulette), K-line
// (add the lit shadow lines) and K-fold (spectral to RGB, per-pixel sums).
//
// The estimator follows the reference's plain strategy set (Meet + Aim,
// plugins/transport/paths/strategy.cpp:119) with the power heuristic
// (weight.cpp:27 weightOf, :95 meetDensities, :107 aimDensities):
//  - camera legs see only the sky (light.cpp:132 seenByCamera);
//  - every lamp is offered at a vertex and one offer, drawn by its lane mean,
//    is traced (trace.cpp:896 aimedFrom, :830 offered);
//  - at the surface cap the aim takes the whole weight (weight.cpp:107);
//  - roulette from depth 4 with survival at most 0.95 (trace.cpp:1051);
//  - rays leave a vertex lifted by 4e-3 plus twice the hit's looseness
//    along the side they leave by (path.cpp:48 leavingRay, trace.cpp:466).
// Throughput and radiance are four hero-wavelength lanes in FP32 (the
// reference carries them in double).
#include "frame.h"
#include "guide_mix.cuh"
#include "materials.cuh"
#include "program.cuh"
#include "atmosphere.h"
#include "skymap.h"
#include "sobol.h"

#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace kdn {

// The frame's constants travel with each launch as a kernel parameter
// (__grid_constant__, read through the constant bank), so frames of
// several contexts can run at once without one's constants overwriting
// another's.

namespace {

constexpr int kBlock = 128;
constexpr float kBias = 4e-3f;

enum Draw : int { PixelX = 0, PixelY, LensU, LensV, LightU, LightV, DirectionU, DirectionV, Lobe, Side, Survival, Pick };

__device__ __forceinline__ float unitFrom(uint64_t bits53) {
	const float u = __ull2float_rn(bits53) * 0x1p-53f;
	return fminf(u, 0x1.fffffep-1f);
}

// plugins/transport/paths/path.cpp:22 dimensionOf for the per-event draws.
__device__ __forceinline__ uint64_t dimensionOf(int event, int draw) {
	return draw < LightU ? uint64_t(draw) : uint64_t(4 + event * 8 + (draw - LightU));
}

// plugins/transport/paths/sampler.cpp:16 numberAt: a hashed number, or with
// the Sobol tables the scrambled Sobol sequence's for the first 28
// dimensions (a pixel's sample index and its group are the same at one
// sample a split)
__device__ __forceinline__ float number(const uint32_t* sobol, uint64_t stream, uint32_t index, int event, int draw) {
	const uint64_t dimension = dimensionOf(event, draw);
	if (sobol != nullptr && dimension < kSobolDimensions) return fminf(float(sobolBits(sobol, stream, index, uint32_t(dimension))) * 0x1p-32f, 0x1.fffffep-1f);
	return unitFrom(hashedBits(stream, index, dimension));
}

// the hashed number of a dimension past the per-event draws: path.cpp:22
// dimensionOf's plain draws, five an event from 2^20 (MixturePart,
// MixtureLump, AimPart, AimJitterU, AimJitterV)
constexpr uint64_t kPlainFirst = uint64_t(1) << 20;
// ... and path.cpp:13 collisionFirst: the Collision draw, one an event from 2^22
constexpr uint64_t kCollisionFirst = uint64_t(1) << 22;
enum PlainDraw : int { AimPart = 2, AimJitterU = 3, AimJitterV = 4 };
__device__ __forceinline__ float plainNumber(uint64_t stream, uint32_t index, int event, int draw) {
	return unitFrom(hashedBits(stream, index, kPlainFirst + uint64_t(event) * 5u + uint64_t(draw)));
}

// material.cpp:1051 phaseCosine, :1059 phaseScatter: a direction drawn
// from Henyey-Greenstein's phase of g = lean about the heading, exactly
// (its weight is 1 and its density the phase's value)
__device__ __forceinline__ float phaseValue(float lean, float cosine) {
	const float denominator = fmaxf(1.0f + lean * lean - 2.0f * lean * cosine, 0.0f);
	return (1.0f - lean * lean) / (4.0f * 3.14159265358979f * denominator * sqrtf(denominator));
}

__device__ float3 phaseDirection(float lean, float3 heading, float u, float v) {
	float cosine = 1.0f - 2.0f * u;
	if (fabsf(lean) > 1e-3f) {
		const float term = (1.0f - lean * lean) / (1.0f - lean + 2.0f * lean * u);
		cosine           = fminf(fmaxf((1.0f + lean * lean - term * term) / (2.0f * lean), -1.0f), 1.0f);
	}
	const float reach = sqrtf(fmaxf(1.0f - cosine * cosine, 0.0f));
	const float angle = 2.0f * 3.14159265358979f * v;
	return frameAround(heading).toWorld(make_float3(reach * cosf(angle), reach * sinf(angle), cosine));
}

// plugins/transport/paths/trace.cpp:66 pixelNumbers
__device__ __forceinline__ uint64_t streamOf(const FrameConstants& cFrame, uint32_t x, uint32_t y) {
	return cFrame.seedMix ^ mixedBits((uint64_t(x) << 32) | uint64_t(y));
}

__device__ __forceinline__ float3 f3(const float* v) { return make_float3(v[0], v[1], v[2]); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 crossOf(float3 a, float3 b) { return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
__device__ __forceinline__ float lengthOf(float3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ float3 normalizedOf(float3 a) { return a * (1.0f / lengthOf(a)); }
__device__ __forceinline__ float4 mul4(float4 a, float4 b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
__device__ __forceinline__ float4 scale4(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
__device__ __forceinline__ float4 add4(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float mean4(float4 a) { return 0.25f * (a.x + a.y + a.z + a.w); }
__device__ __forceinline__ float max4(float4 a) { return fmaxf(fmaxf(a.x, a.y), fmaxf(a.z, a.w)); }

// ---- spectra (math/colour.cpp, math/spectrum.cpp) ----

__device__ __forceinline__ float tableAt(const float* curve, float nm) {
	const float slot  = (nm - 380.0f) / 5.0f;
	int below         = int(slot);
	below             = below < 0 ? 0 : (below > kTableSize - 2 ? kTableSize - 2 : below);
	const float blend = fminf(fmaxf(slot - float(below), 0.0f), 1.0f);
	return curve[below] + blend * (curve[below + 1] - curve[below]);
}

// math/colour.cpp:213 colourOf
__device__ float3 colourOf(const FrameConstants& cFrame, float4 nm, float4 density, float4 spectrum) {
	const float lanes[4] = { nm.x, nm.y, nm.z, nm.w };
	const float dens[4]  = { density.x, density.y, density.z, density.w };
	const float spec[4]  = { spectrum.x, spectrum.y, spectrum.z, spectrum.w };
	float x = 0.0f, y = 0.0f, z = 0.0f;
	for (int k = 0; k < 4; ++k) {
		if (dens[k] <= 0.0f) continue;
		const float w = spec[k] / dens[k];
		x += tableAt(cFrame.spectral.cie[0], lanes[k]) * w;
		y += tableAt(cFrame.spectral.cie[1], lanes[k]) * w;
		z += tableAt(cFrame.spectral.cie[2], lanes[k]) * w;
	}
	x *= 0.25f;
	y *= 0.25f;
	z *= 0.25f;
	const float r = 3.2406f * x - 1.5372f * y - 0.4986f * z;
	const float g = -0.9689f * x + 1.8758f * y + 0.0415f * z;
	const float b = 0.0557f * x - 0.2040f * y + 1.0570f * z;
	return make_float3(r / cFrame.spectral.white[0], g / cFrame.spectral.white[1], b / cFrame.spectral.white[2]);
}

// ---- lamps (plugins/transport/paths/light/light.cpp) ----

struct Aim {
	bool found;
	float3 toward;
	float distance;
	float3 arriving; // RGB radiance over the density of the direction
	float density;
};

// A spherical rectangle seen from a point: solid-angle sampling of a
// rectangular light (Urena, Fajardo and King, "An Area-Preserving
// Parametrization for Spherical Rectangles", EGSR 2013).
struct Rectangle {
	float3 x, y, z;
	float z0, x0, x1, y0, y1, b0, b1, k, angle;
};

__device__ Rectangle rectangleFrom(const DeviceLamp& l, float3 origin) {
	Rectangle r;
	const float3 offset = f3(l.at) - origin;
	const float3 raw    = f3(l.raw);
	r.z                 = dot3(offset, raw) > 0.0f ? raw * -1.0f : raw;
	r.x                 = f3(l.ex);
	r.y                 = f3(l.ey);
	r.z0                = dot3(offset, r.z);
	r.x0                = dot3(offset, r.x);
	r.y0                = dot3(offset, r.y);
	r.x1                = r.x0 + l.alongLength;
	r.y1                = r.y0 + l.acrossLength;
	// normals of the four planes through the origin and each edge, by their z parts
	const float sides[4]   = { r.z0 * r.x1 - r.x0 * r.z0, r.y0 * r.z0 - r.z0 * r.y1, r.z0 * r.x0 - r.x1 * r.z0, r.y1 * r.z0 - r.z0 * r.y0 };
	const float heights[4] = { r.x0 * r.y0 - r.y0 * r.x1, r.x1 * r.y1 - r.y0 * r.x1, r.x1 * r.y1 - r.y1 * r.x0, r.x0 * r.y0 - r.y1 * r.x0 };
	float upright[4];
	for (int s = 0; s < 4; ++s) {
		const float size = sqrtf(sides[s] * sides[s] + heights[s] * heights[s]);
		upright[s]       = size > 0.0f ? heights[s] / size : heights[s];
	}
	const float g0 = acosf(fminf(fmaxf(-(upright[0] * upright[1]), -1.0f), 1.0f));
	const float g1 = acosf(fminf(fmaxf(-(upright[1] * upright[2]), -1.0f), 1.0f));
	const float g2 = acosf(fminf(fmaxf(-(upright[2] * upright[3]), -1.0f), 1.0f));
	const float g3 = acosf(fminf(fmaxf(-(upright[3] * upright[0]), -1.0f), 1.0f));
	r.b0           = upright[0];
	r.b1           = upright[2];
	r.k            = 2.0f * 3.14159265358979f - g2 - g3;
	r.angle        = g0 + g1 - r.k;
	return r;
}

__device__ float3 rectanglePoint(const Rectangle& r, float3 origin, float u, float v) {
	const float au  = u * r.angle + r.k;
	const float fu  = (cosf(au) * r.b0 - r.b1) / sinf(au);
	const float cu  = fminf(fmaxf(copysignf(1.0f / sqrtf(fu * fu + r.b0 * r.b0), fu), -1.0f), 1.0f);
	const float xu  = fminf(fmaxf(-(cu * r.z0) / sqrtf(fmaxf(1.0f - cu * cu, 1e-14f)), r.x0), r.x1);
	const float d   = sqrtf(xu * xu + r.z0 * r.z0);
	const float h0  = r.y0 / sqrtf(d * d + r.y0 * r.y0);
	const float h1  = r.y1 / sqrtf(d * d + r.y1 * r.y1);
	const float hv  = h0 + v * (h1 - h0);
	const float hv2 = hv * hv;
	const float yv  = hv2 < 1.0f - 1e-6f ? (hv * d) / sqrtf(1.0f - hv2) : r.y1;
	return origin + r.x * xu + r.y * yv + r.z * r.z0;
}

__device__ __forceinline__ float coneDensity(float cosine) {
	const float cone = 2.0f * 3.14159265358979f * (1.0f - cosine);
	return cone > 1e-12f ? 1.0f / cone : 0.0f;
}

// sky_layers.cpp:273 moonLit: the share of a moon's disc the first sun
// lights where a direction meets it, eased (in double: the disc is small)
__device__ __noinline__ float moonShare(const FrameConstants& c, const DeviceLamp& l, float3 toward) {
	const double d[3]   = { double(toward.x), double(toward.y), double(toward.z) };
	const double along  = d[0] * l.disc[0] + d[1] * l.disc[1] + d[2] * l.disc[2];
	const double aside  = fmax(1.0 - along * along, 0.0);
	const double reach  = along - sqrt(fmax(l.discRadius * l.discRadius - aside, 0.0));
	double facing       = 0.0;
	for (int a = 0; a < 3; ++a) facing += (d[a] * reach - l.disc[a]) / l.discRadius * c.sunDirection[a];
	const double lit    = fmin(fmax(facing / 0.1 + 0.5, 0.0), 1.0);
	return float(lit * lit * (3.0 - 2.0 * lit));
}

__device__ __forceinline__ float moonLit(const FrameConstants& c, const DeviceLamp& l, float3 toward) {
	return l.kind == 5 && c.hasSun ? moonShare(c, l, toward) : 1.0f;
}

// aimLight (light.cpp:372) for a point light, a directional light, a sun
// or a moon (out of line: most scenes light by quads and spheres).
__device__ __noinline__ Aim aimOther(const DeviceLamp& l, float3 from, float u, float v) {
	Aim a;
	a.found = false;
	if (l.kind == 0) { // point (light.cpp:349 aimPoint): singular, density 0
		const float3 off = f3(l.at) - from;
		const float dist = lengthOf(off);
		if (dist < 1e-9f) return a;
		a.found    = true;
		a.toward   = off * (1.0f / dist);
		a.distance = dist;
		a.arriving = f3(l.power) * (1.0f / (dist * dist));
		a.density  = 0.0f;
		return a;
	}
	if (l.kind == 1) { // directional (light.cpp:362): singular, from afar
		a.found    = true;
		a.toward   = f3(l.direction);
		a.distance = __int_as_float(0x7f800000);
		a.arriving = f3(l.power);
		a.density  = 0.0f;
		return a;
	}
	if (l.kind == 4 || l.kind == 5) { // sun or moon (light.cpp:334 aimSun): evenly in the disc's cone
		if (!(l.oneLess > 0.0f)) return a;
		const float drop   = u * l.oneLess; // 1 - the height in the cone
		const float ring   = sqrtf(fmaxf(drop * (2.0f - drop), 0.0f));
		const float angle  = 2.0f * 3.14159265358979f * v;
		const Frame f      = frameAround(f3(l.direction));
		a.found    = true;
		a.toward   = f.toWorld(make_float3(ring * cosf(angle), ring * sinf(angle), 1.0f - drop));
		a.distance = __int_as_float(0x7f800000);
		a.density  = 1.0f / (2.0f * 3.14159265358979f * l.oneLess);
		a.arriving = f3(l.radiance) * (2.0f * 3.14159265358979f * l.oneLess);
		return a;
	}
	return a;
}

// aimLight (light.cpp:372) for a quad or a sphere lamp.
__device__ __forceinline__ Aim aimArea(const DeviceLamp& l, float3 from, float u, float v) {
	Aim a;
	a.found = false;
	if (l.kind == 3) { // quad
		if (l.area < 1e-12f || dot3(f3(l.facing), from - f3(l.at)) <= 0.0f) return a;
		float3 spot;
		float density;
		if (l.square) {
			const Rectangle r = rectangleFrom(l, from);
			if (!(r.angle > 1e-7f)) return a;
			spot    = rectanglePoint(r, from, u, v);
			density = 1.0f / r.angle;
			const float3 off = spot - from;
			const float dist = lengthOf(off);
			if (dist < 1e-9f) return a;
			a.found    = true;
			a.toward   = off * (1.0f / dist);
			a.distance = dist;
			a.density  = density;
			a.arriving = f3(l.radiance) * r.angle;
			return a;
		}
		spot             = f3(l.at) + f3(l.along) * u + f3(l.across) * v;
		const float3 off = spot - from;
		const float dist = lengthOf(off);
		if (dist < 1e-9f) return a;
		a.toward         = off * (1.0f / dist);
		const float tilt = -dot3(f3(l.facing), a.toward);
		a.found          = true;
		a.distance       = dist;
		if (tilt <= 0.0f) {
			a.arriving = make_float3(0.0f, 0.0f, 0.0f);
			a.density  = 0.0f;
			return a;
		}
		a.arriving = f3(l.radiance) * (tilt * l.area / (dist * dist));
		a.density  = dist * dist / (tilt * l.area);
		return a;
	}
	if (l.kind == 2) { // sphere
		const float3 off  = f3(l.at) - from;
		const float dist  = lengthOf(off);
		if (dist < 1e-9f || dist <= l.radius) return a;
		const float3 axis = off * (1.0f / dist);
		const float side  = l.radius / dist;
		const float cosine = sqrtf(fmaxf(1.0f - side * side, 0.0f));
		const float height = 1.0f - u * (1.0f - cosine);
		const float ring   = sqrtf(fmaxf(1.0f - height * height, 0.0f));
		const float angle  = 2.0f * 3.14159265358979f * v;
		const Frame f      = frameAround(axis);
		const float3 toward = f.toWorld(make_float3(ring * cosf(angle), ring * sinf(angle), height));
		const float h      = dot3(toward, axis);
		const float r2     = sqrtf(fmaxf(1.0f - h * h, 0.0f));
		const float reach  = dist * h - sqrtf(fmaxf(l.radius * l.radius - dist * dist * r2 * r2, 0.0f));
		a.found    = true;
		a.toward   = toward;
		a.distance = fmaxf(reach, 0.0f);
		a.arriving = f3(l.power) * (2.0f * (1.0f - cosine) / (l.radius * l.radius));
		a.density  = coneDensity(cosine);
		return a;
	}
	return a;
}

// aimLight (light.cpp:372) for every kind of lamp.
__device__ __forceinline__ Aim aimLamp(const DeviceLamp& l, float3 from, float u, float v) {
	return l.kind == 2 || l.kind == 3 ? aimArea(l, from, u, v) : aimOther(l, from, u, v);
}

// Whether a unit direction lies in a far disc's cone: 1 - cos(apart) <=
// 1 - cos(half), as half the squared distance between the unit vectors
__device__ __forceinline__ bool inDisc(const DeviceLamp& l, float3 toward) {
	const float3 apart = toward - f3(l.direction);
	return l.oneLess > 0.0f && 0.5f * dot3(apart, apart) <= l.oneLess;
}

// aimDensity (light.cpp:463): the density aiming gives a direction, for a
// quad or a sphere lamp ...
__device__ __forceinline__ float areaDensityOf(const DeviceLamp& l, float3 from, float3 toward, float distance) {
	if (l.kind == 3) {
		if (l.area < 1e-12f || dot3(f3(l.facing), from - f3(l.at)) <= 0.0f) return 0.0f;
		if (l.square) {
			const Rectangle r = rectangleFrom(l, from);
			return r.angle > 1e-7f ? 1.0f / r.angle : 0.0f;
		}
		const float tilt = -dot3(f3(l.facing), toward);
		if (tilt <= 0.0f || distance <= 0.0f) return 0.0f;
		return distance * distance / (tilt * l.area);
	}
	if (l.kind == 2) {
		const float away = lengthOf(f3(l.at) - from);
		if (away <= l.radius || l.radius <= 0.0f) return 0.0f;
		const float side = l.radius / away;
		return coneDensity(sqrtf(fmaxf(1.0f - side * side, 0.0f)));
	}
	return 0.0f;
}

// ... and for every kind (a point or a directional light is singular: 0)
__device__ __forceinline__ float aimDensityOf(const DeviceLamp& l, float3 from, float3 toward, float distance) {
	if (l.kind == 4 || l.kind == 5) return inDisc(l, toward) ? 1.0f / (2.0f * 3.14159265358979f * l.oneLess) : 0.0f;
	return areaDensityOf(l, from, toward, distance);
}

// meetLight (light.cpp:498) for a quad or a sphere lamp: where a ray meets
// it before limit ...
__device__ __forceinline__ bool meetArea(const DeviceLamp& l, float3 origin, float3 dir, float limit, float& reach) {
	if (l.kind == 3) {
		const float3 facing = f3(l.cross);
		const float leaning = dot3(facing, dir);
		if (l.area < 1e-12f || leaning >= -1e-12f) return false;
		reach = dot3(facing, f3(l.at) - origin) / leaning;
		if (reach <= 1e-9f || reach >= limit) return false;
		const float3 spot   = origin + dir * reach - f3(l.at);
		const float squared = l.area * l.area;
		const float u       = dot3(crossOf(spot, f3(l.across)), facing) / squared;
		const float v       = dot3(crossOf(f3(l.along), spot), facing) / squared;
		return !(u < 0.0f || u > 1.0f || v < 0.0f || v > 1.0f);
	}
	if (l.kind == 2) {
		if (l.radius <= 0.0f) return false;
		const float3 off  = origin - f3(l.at);
		const float along = dot3(off, dir);
		const float under = along * along - (dot3(off, off) - l.radius * l.radius);
		if (under <= 0.0f) return false;
		const float root  = sqrtf(under);
		const float first = -along - root;
		reach             = first <= 1e-9f ? -along + root : first;
		return !(reach <= 1e-9f || reach >= limit);
	}
	return false;
}

// ... and for every kind (a point or a directional light is never met; a
// sun or a moon only by a ray that escaped, light.cpp:478 meetSun)
__device__ __forceinline__ bool meetLamp(const DeviceLamp& l, float3 origin, float3 dir, float limit, float& reach) {
	if (l.kind == 4 || l.kind == 5) {
		reach = __int_as_float(0x7f800000);
		return limit >= 3.0e38f && inDisc(l, dir);
	}
	return meetArea(l, origin, dir, limit, reach);
}

// light.cpp:575 gradientColour
__device__ float3 skyColour(const FrameConstants& cFrame, float3 dir);

// sky_map.cpp:138 chartedDirection, :144 chartAim: a direction drawn from the
// sky's chart (or, a tenth of the time, uniformly), its density and the
// sky's radiance there over it
__device__ Aim aimSky(const FrameConstants& cFrame, float u, float v, float part, float jitterU, float jitterV) {
	const double* chart = cFrame.skyChart;
	float height, turn;
	if (double(part) < kChartEven) {
		height = 1.0f - 2.0f * u;
		turn   = 2.0f * 3.14159265358979f * v;
	} else {
		const int row    = chartFound(chart, kChartRows, double(u));
		const int column = chartFound(chart + kChartRows + 1 + row * kChartCells, kChartColumns, double(v));
		height           = -1.0f + (float(row) + jitterU) * (2.0f / kChartRows);
		turn             = (float(column) + jitterV) * (2.0f * 3.14159265358979f / kChartColumns);
	}
	const float across = sqrtf(fmaxf(1.0f - height * height, 0.0f));
	float3 toward      = make_float3(across * cosf(turn), across * sinf(turn), height);
	const float size   = sqrtf(toward.x * toward.x + toward.y * toward.y + toward.z * toward.z);
	toward             = make_float3(toward.x / size, toward.y / size, toward.z / size);
	Aim a;
	a.toward         = toward;
	a.distance       = __int_as_float(0x7f800000);
	a.density        = float(chartDensity(chart, toward.x, toward.y, toward.z));
	a.found          = a.density > 0.0f;
	const float3 sky = skyColour(cFrame, toward);
	a.arriving       = a.found ? make_float3(sky.x / a.density, sky.y / a.density, sky.z / a.density) : make_float3(0.0f, 0.0f, 0.0f);
	return a;
}

__device__ float3 skyColour(const FrameConstants& cFrame, float3 dir) {
	const float height = dir.z;
	const float3 far   = height >= 0.0f ? f3(cFrame.zenith) : f3(cFrame.ground);
	const float share  = sqrtf(fabsf(height));
	return f3(cFrame.horizon) * (1.0f - share) + far * share;
}

// math/spectrum.cpp:83 tablePlace, :88 spectrumTableAt: a 33-place table
// over 380..700 nm read at each lane's wavelength
__device__ __forceinline__ float tablePlaceOf(float nm) { return fminf(fmaxf((nm - 380.0f) / 320.0f, 0.0f), 1.0f) * 32.0f; }

__device__ float4 tableSpectrum(const float* table, float4 nm) {
	const float w[4] = { nm.x, nm.y, nm.z, nm.w };
	float out[4];
	for (int k = 0; k < 4; ++k) {
		const float place = tablePlaceOf(w[k]);
		const int low     = min(int(place), 31);
		out[k]            = table[low] + (table[low + 1] - table[low]) * (place - float(low));
	}
	return make_float4(out[0], out[1], out[2], out[3]);
}

// atmosphere.cpp:206 airTableAt: trilinear in (row, column, colour)
__device__ float airTableAt(const float* table, float row, float column, float colour) {
	const int r = min(int(row), kAirHeights - 2), b = min(int(column), kAirBearings - 2), l = min(int(colour), kAirColours - 2);
	const float fr = fminf(fmaxf(row - float(r), 0.0f), 1.0f), fb = fminf(fmaxf(column - float(b), 0.0f), 1.0f), fl = fminf(fmaxf(colour - float(l), 0.0f), 1.0f);
	const float* t = table + (r * kAirBearings + b) * kAirColours + l;
	const float lo = (1.0f - fb) * ((1.0f - fl) * t[0] + fl * t[1]) + fb * ((1.0f - fl) * t[kAirColours] + fl * t[kAirColours + 1]);
	t += kAirBearings * kAirColours;
	const float hi = (1.0f - fb) * ((1.0f - fl) * t[0] + fl * t[1]) + fb * ((1.0f - fl) * t[kAirColours] + fl * t[kAirColours + 1]);
	return (1.0f - fr) * lo + fr * hi;
}

// atmosphere.cpp:312 airSeen: what the air shows along a direction (the
// ground lit by the sun and the sky below the horizon), per lane
__device__ __noinline__ float4 airSeen(const FrameConstants& c, float3 dir, float4 nm) {
	const float4 sunlight = spectrumOf(c.sunlight[0], c.sunlight[1], c.sunlight[2], nm);
	const float rise      = fminf(fmaxf(dot3(dir, f3(c.airUp)), -1.0f), 1.0f);
	const float height    = asinf(rise);
	if (height < 0.0f) {
		return scale4(mul4(mul4(spectrumOf(c.airGround[0], c.airGround[1], c.airGround[2], nm), tableSpectrum(c.airLanding, nm)), sunlight), 1.0f / 3.14159265358979f);
	}
	const float bearing = fabsf(atan2f(dot3(dir, f3(c.airAside)), dot3(dir, f3(c.airLevel))));
	const float row     = sqrtf(fmaxf(height, 0.0f) / (0.5f * 3.14159265358979f)) * float(kAirHeights - 1);
	const float column  = bearing / 3.14159265358979f * float(kAirBearings - 1);
	const float cosine  = dot3(dir, f3(c.airSun));
	// the air's phase (Rayleigh) and the haze's (Cornette-Shanks, g = 0.76)
	const float airPhase   = 3.0f / (16.0f * 3.14159265358979f) * (1.0f + cosine * cosine);
	const float g          = 0.76f;
	const float base       = fmaxf(1.0f + g * g - 2.0f * g * cosine, 1e-12f);
	const float hazePhase  = 3.0f / (8.0f * 3.14159265358979f) * (1.0f - g * g) * (1.0f + cosine * cosine) / ((2.0f + g * g) * base * sqrtf(base));
	const float w[4]       = { nm.x, nm.y, nm.z, nm.w };
	float out[4];
	for (int k = 0; k < 4; ++k) {
		const float colour = tablePlaceOf(w[k]);
		out[k] = airPhase * airTableAt(c.airTables, row, column, colour) + hazePhase * airTableAt(c.airTables + kAirTable, row, column, colour);
	}
	return mul4(make_float4(out[0], out[1], out[2], out[3]), sunlight);
}

// sky_layers.cpp:33 smoothShare
__device__ __forceinline__ float smoothShare(float from, float to, float value) {
	const float s = fminf(fmaxf((value - from) / (to - from), 0.0f), 1.0f);
	return s * s * (3.0f - 2.0f * s);
}

// sky_layers.cpp:181 glowSeen: the glow about the first sun, falling by e
// over `spread` radians from it, faded as the sun sinks 8 degrees below the
// horizon and over the horizon, 0.02 either side
__device__ __noinline__ float4 glowSeen(const FrameConstants& c, float3 dir, float4 nm) {
	const float above   = smoothShare(-0.02f, 0.02f, dir.z);
	const float apart   = acosf(fminf(fmaxf(float(double(dir.x) * c.sunDirection[0] + double(dir.y) * c.sunDirection[1] + double(dir.z) * c.sunDirection[2]), -1.0f), 1.0f));
	const float fade    = smoothShare(-8.0f * 3.14159265358979f / 180.0f, 0.0f, c.sunElevation);
	const float falling = expf(-apart / fmaxf(c.glowSpread, 1e-6f)) * fade * above;
	return spectrumOf(c.glow[0] * falling, c.glow[1] * falling, c.glow[2] * falling, nm);
}

// sky_layers.cpp:240 starlight: one star a cell of a grid on each cube face
// (about `count` over the sphere), placed, sized and coloured by hashes of
// its cell's key; in double (the discs are small)
__device__ __noinline__ float4 starsSeen(const FrameConstants& c, float3 toward, float4 nm) {
	const double d[3] = { toward.x, toward.y, toward.z };
	const double ax = fabs(d[0]), ay = fabs(d[1]), az = fabs(d[2]);
	uint64_t face;
	double out[3] = { 0, 0, 0 }, right[3] = { 0, 0, 0 }, up[3] = { 0, 0, 0 };
	if (ax >= ay && ax >= az) {
		const double sign = d[0] >= 0 ? 1.0 : -1.0;
		face = d[0] >= 0 ? 0u : 1u, out[0] = sign, right[1] = sign, up[2] = 1;
	} else if (ay >= az) {
		const double sign = d[1] >= 0 ? 1.0 : -1.0;
		face = d[1] >= 0 ? 2u : 3u, out[1] = sign, right[2] = sign, up[0] = 1;
	} else {
		const double sign = d[2] >= 0 ? 1.0 : -1.0;
		face = d[2] >= 0 ? 4u : 5u, out[2] = sign, right[0] = sign, up[1] = 1;
	}
	const double outward = d[0] * out[0] + d[1] * out[1] + d[2] * out[2];
	const double u = (d[0] * right[0] + d[1] * right[1] + d[2] * right[2]) / outward;
	const double v = (d[0] * up[0] + d[1] * up[1] + d[2] * up[2]) / outward;
	const int cells  = max(1, int(ceil(sqrt(double(c.starCount) / 6.0))));
	const int column = min(max(int((u * 0.5 + 0.5) * cells), 0), cells - 1);
	const int row    = min(max(int((v * 0.5 + 0.5) * cells), 0), cells - 1);
	uint64_t key     = (face * 65536u + uint64_t(row)) * 65536u + uint64_t(column);
	double draw[4];
	for (int k = 0; k < 4; ++k) {
		key     = mixedBits(key + 0x9E3779B97F4A7C15ULL);
		draw[k] = double(key >> 11) * 0x1p-53;
	}
	const double across = (column + 0.2 + 0.6 * draw[0]) / cells * 2.0 - 1.0;
	const double down   = (row + 0.2 + 0.6 * draw[1]) / cells * 2.0 - 1.0;
	double star[3], size = 0;
	for (int a = 0; a < 3; ++a) {
		star[a] = out[a] + right[a] * across + up[a] * down;
		size += star[a] * star[a];
	}
	size = sqrt(size);
	if ((d[0] * star[0] + d[1] * star[1] + d[2] * star[2]) / size < cos(0.5 * double(c.starAngle))) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	const double bright = double(c.starStrength) * pow(draw[2], 6.0) * double(c.starNight);
	const double w      = draw[3];
	return spectrumOf(float((0.75 * (1 - w) + 1.0 * w) * bright), float((0.85 * (1 - w) + 0.82 * w) * bright), float((1.0 * (1 - w) + 0.62 * w) * bright), nm);
}

// feature.cpp:30 skyAt: the sky's radiance along a direction, per lane: the
// gradient, or the air of a physical sky, and the glow about the sun
__device__ __forceinline__ float4 skySpectrum(const FrameConstants& c, float3 dir, float4 nm) {
	float4 sky;
	if (c.airTables != nullptr) {
		sky = airSeen(c, dir, nm);
	} else {
		const float3 rgb = skyColour(c, dir);
		sky              = spectrumOf(rgb.x, rgb.y, rgb.z, nm);
	}
	if (c.glows) sky = add4(sky, glowSeen(c, dir, nm));
	if (c.stars && dir.z > 0.0f) sky = add4(sky, starsSeen(c, dir, nm));
	return sky;
}

// feature.cpp:133 lampTint: what of a lamp's light the air lets through
// (the first sun under a physical sky), per lane
__device__ __forceinline__ float4 lampTint(const FrameConstants& c, uint32_t lamp, float4 nm) {
	return c.airTables != nullptr && lamp == c.sunLamp ? tableSpectrum(c.airPassed, nm) : make_float4(1.0f, 1.0f, 1.0f, 1.0f);
}

__device__ __forceinline__ kdn_ray makeRay(float3 o, float3 d, float far, uint32_t medium) {
	kdn_ray r;
	r.origin[0]    = o.x;
	r.origin[1]    = o.y;
	r.origin[2]    = o.z;
	r.direction[0] = d.x;
	r.direction[1] = d.y;
	r.direction[2] = d.z;
	r.far          = far;
	r.inside       = medium != kNoMaterial ? 1 : 0;
	r.pad_[0] = r.pad_[1] = r.pad_[2] = 0;
	r.within       = medium;
	return r;
}

// Append to a queue, one atomic per warp.
__device__ __forceinline__ uint32_t warpSlot(uint32_t* count, bool want) {
	const unsigned active = __activemask();
	const unsigned mask   = __ballot_sync(active, want);
	if (mask == 0) return 0xFFFFFFFFu;
	const int lane   = threadIdx.x & 31;
	const int leader = __ffs(mask) - 1;
	uint32_t base    = 0;
	if (lane == leader) base = atomicAdd(count, uint32_t(__popc(mask)));
	base = __shfl_sync(active, base, leader);
	return want ? base + uint32_t(__popc(mask & ((1u << lane) - 1u))) : 0xFFFFFFFFu;
}

// ---- K-cam: camera rays and hero wavelengths (trace.cpp:116 startedPathIn) ----
__global__ void __launch_bounds__(kBlock) cameraKernel(const __grid_constant__ FrameConstants cFrame, PathBuffers P, QueueBuffers Q, uint32_t firstPixel, uint32_t n) {
	if (blockIdx.x == 0 && threadIdx.x == 0) *Q.count = n;
	for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
		const uint32_t pixel  = firstPixel + p / cFrame.spp;
		const uint32_t sample = cFrame.firstSample + p % cFrame.spp;
		// core/pixels.cpp:5 groupSample: with a split the samples of a group
		// share the first vertex's draws (path.cpp:37 sharedDraw)
		const uint32_t group  = sample / cFrame.split;
		const uint32_t x      = pixel % uint32_t(cFrame.width);
		const uint32_t y      = pixel / uint32_t(cFrame.width);
		const uint64_t stream = streamOf(cFrame, x, y);
		// math/colour.cpp:236 sampledWavelengths of the pixel's golden-ratio share
		const double start  = double(hashedBits(stream, ~uint64_t(0), 0)) * 0x1p-53;
		const double turned = double(group) * 0.6180339887498949 + start;
		const double share  = turned - floor(turned);
		float nm[4], dens[4];
		for (int lane = 0; lane < 4; ++lane) {
			const double raw    = share + 0.25 * lane;
			const double t      = raw >= 1.0 ? raw - 1.0 : raw;
			const double place  = t * kCuts;
			const int index     = int(place) < kCuts - 1 ? int(place) : kCuts - 1;
			const double width  = cFrame.spectral.cuts[index + 1] - cFrame.spectral.cuts[index];
			const double value  = cFrame.spectral.cuts[index] + (place - index) * width;
			nm[lane]            = float(fmin(value, 699.9999999999999));
			dens[lane]          = float(1.0 / (kCuts * width));
		}
		// trace.cpp:105 filmDraw, :93 phasedDraw at a film factor above 1
		float px, py;
		if (cFrame.factor > 1) {
			const float factor = float(cFrame.factor);
			px = float(x) + (float(cFrame.phase % cFrame.factor) + number(cFrame.sobol, stream, group, 0, PixelX)) / factor;
			py = float(y) + (float(cFrame.phase / cFrame.factor) + number(cFrame.sobol, stream, group, 0, PixelY)) / factor;
		} else {
			px = float(x) + number(cFrame.sobol, stream, group, 0, PixelX);
			py = float(y) + number(cFrame.sobol, stream, group, 0, PixelY);
		}
		const float u  = 2.0f * px / float(cFrame.width) - 1.0f;
		const float v  = 1.0f - 2.0f * py / float(cFrame.height);
		float3 heading = normalizedOf(f3(cFrame.forward) + f3(cFrame.right) * (u * cFrame.reach * cFrame.aspect) + f3(cFrame.up) * (v * cFrame.reach));
		float3 origin  = f3(cFrame.eye);
		if (cFrame.aperture > 0.0f) {
			// plugins/transport/paths/camera.cpp:14 cameraRay: from a point of
			// the lens (math/random.cpp:48 concentricDisc of the LensU/LensV
			// pair) toward where the pinhole ray meets the plane in focus
			const float ahead = cFrame.focus / fmaxf(dot3(heading, f3(cFrame.forward)), 1e-9f);
			const float3 sharp = origin + heading * ahead;
			const float a      = 2.0f * number(cFrame.sobol, stream, group, 0, LensU) - 1.0f;
			const float b      = 2.0f * number(cFrame.sobol, stream, group, 0, LensV) - 1.0f;
			float du = 0.0f, dv = 0.0f;
			if (a != 0.0f || b != 0.0f) {
				const bool wide    = fabsf(a) > fabsf(b);
				const float radius = wide ? a : b;
				const float angle  = wide ? 0.78539816f * (b / a) : 1.5707963f - 0.78539816f * (a / b);
				du                 = radius * cosf(angle);
				dv                 = radius * sinf(angle);
			}
			origin  = origin + f3(cFrame.right) * (du * cFrame.aperture) + f3(cFrame.up) * (dv * cFrame.aperture);
			heading = normalizedOf(sharp - origin);
		}
		P.pixel[p]      = pixel;
		P.sample[p]     = sample;
		P.throughput[p] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
		P.radiance[p]   = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		P.nanometres[p] = make_float4(nm[0], nm[1], nm[2], nm[3]);
		P.density[p]    = make_float4(dens[0], dens[1], dens[2], dens[3]);
		P.drawn[p]      = 0.0f;
		P.state[p]      = 1u << 8;
		P.from[p]       = make_float4(origin.x, origin.y, origin.z, 0.0f);
		if (P.held != nullptr) {
			for (uint32_t k = 0; k < kOwnLines; ++k) P.held[size_t(p) * kOwnLines + k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		}
		if (P.collided != nullptr) P.collided[p] = 0u;
		Q.paths[p]      = p;
		Q.rays[p]       = makeRay(origin, heading, __int_as_float(0x7f800000), kNoMaterial);
	}
}

__device__ __forceinline__ const DeviceMaterial& materialOfLeaf(uint32_t leaf, const Looks& L) {
	const uint32_t m = leaf < L.leafCount ? L.leafMaterial[leaf] : 0u;
	return L.materials[m < L.materialCount ? m : 0u];
}

// sdf/program.cpp evaluate over a pattern program's steps, with the point
// and the normal as inputs (its arguments are folded to constants).
__device__ float patternValue(const PatternStep* steps, uint32_t count, uint32_t result, const float p[3], const float n[3]) {
	float r[kPatternSteps];
	r[0] = 0.0f;
	for (uint32_t i = 0; i < count && i < kPatternSteps; ++i) {
		const PatternStep s = steps[i];
		float v;
		if (s.op == OpNormalX) v = n[0];
		else if (s.op == OpNormalY) v = n[1];
		else if (s.op == OpNormalZ) v = n[2];
		else v = stepValue(s.op, r[s.a], r[s.b], r[s.c], s.value, p);
		r[i] = v;
	}
	return r[result < kPatternSteps ? result : 0u];
}

// material.cpp:314 albedoAt over :299 patternAt and :281 rampAt: a flat
// colour, or the ramp (its stops spread evenly over 0..1) at the pattern's
// value at the point and the normal facing the ray, in the painted leaf's
// space (material.cpp:292 placedVector) unless read in world space.
__device__ float3 colourAt(const DeviceMaterial& m, uint32_t leaf, float3 point, float3 normal, const Looks& L) {
	if (m.patternCount == 0) return make_float3(m.albedo[0], m.albedo[1], m.albedo[2]);
	float3 p = point, n = normal;
	if (!m.world && leaf < L.placementCount) {
		const float* pl = L.placements + 12 * size_t(leaf);
		const float3 d  = point - make_float3(pl[9], pl[10], pl[11]);
		p               = make_float3(pl[0] * d.x + pl[1] * d.y + pl[2] * d.z, pl[3] * d.x + pl[4] * d.y + pl[5] * d.z, pl[6] * d.x + pl[7] * d.y + pl[8] * d.z);
		const float3 t  = make_float3(pl[0] * normal.x + pl[1] * normal.y + pl[2] * normal.z, pl[3] * normal.x + pl[4] * normal.y + pl[5] * normal.z,
		                              pl[6] * normal.x + pl[7] * normal.y + pl[8] * normal.z);
		const float size = sqrtf(dot3(t, t));
		n                = size > 0.0f ? t * (1.0f / size) : t;
	}
	const float pp[3] = { p.x, p.y, p.z }, nn[3] = { n.x, n.y, n.z };
	const float value = patternValue(L.patternSteps + m.patternFirst, m.patternCount, m.patternResult, pp, nn);
	const float* stops = L.stops + 3 * size_t(m.stopFirst);
	if (m.stopCount <= 1) return make_float3(stops[0], stops[1], stops[2]);
	const float place    = fminf(fmaxf(value, 0.0f), 1.0f) * float(m.stopCount - 1);
	const uint32_t lower = min(uint32_t(place), m.stopCount - 2);
	const float share    = place - float(lower);
	const float* a       = stops + 3 * lower;
	return make_float3(a[0] * (1.0f - share) + a[3] * share, a[1] * (1.0f - share) + a[4] * share, a[2] * (1.0f - share) + a[5] * share);
}

// material.cpp:345 bsdfAt: the leaf's albedo, mixed with the other leaf's by
// the hit's share where a blend joins two leaves.
__device__ __forceinline__ float3 albedoAt(const kdn_hit& hit, float3 normal, const Looks& L) {
	const float3 point = make_float3(hit.point[0], hit.point[1], hit.point[2]);
	float3 a           = colourAt(materialOfLeaf(hit.leaf, L), hit.leaf, point, normal, L);
	if (hit.other != kNoLeaf && hit.share > 0.0f) {
		const float3 o = colourAt(materialOfLeaf(hit.other, L), hit.other, point, normal, L);
		const float s  = hit.share;
		a = make_float3(a.x * (1.0f - s) + o.x * s, a.y * (1.0f - s) + o.y * s, a.z * (1.0f - s) + o.z * s);
	}
	return a;
}

// ---- the surfaces pass: one ray through each pixel's film centre (core/surfaces.cpp:39 surfaceRay) ----
__global__ void __launch_bounds__(kBlock) surfaceRaysKernel(const __grid_constant__ FrameConstants cFrame, QueueBuffers Q, uint32_t firstPixel, uint32_t n) {
	if (blockIdx.x == 0 && threadIdx.x == 0) *Q.count = n;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const uint32_t pixel = firstPixel + i;
		const uint32_t x     = pixel % uint32_t(cFrame.width);
		const uint32_t y     = pixel / uint32_t(cFrame.width);
		const float u        = 2.0f * (float(x) + cFrame.centre[0]) / float(cFrame.width) - 1.0f;
		const float v        = 1.0f - 2.0f * (float(y) + cFrame.centre[1]) / float(cFrame.height);
		const float3 heading = normalizedOf(f3(cFrame.forward) + f3(cFrame.right) * (u * cFrame.reach * cFrame.aspect) + f3(cFrame.up) * (v * cFrame.reach));
		Q.paths[i]           = pixel;
		Q.rays[i]            = makeRay(f3(cFrame.eye), heading, __int_as_float(0x7f800000), kNoMaterial);
	}
}

// trace.cpp:1640 cameraSurface over trace.cpp:1445 vertexSurface: distance
// from the eye, the normal facing the ray, the albedo and the leaf; a missed
// ray keeps batch.cpp:46 missedSurface (infinite distance, no leaf).  Stored
// as the denoiser's FP16 features.
__global__ void __launch_bounds__(kBlock) surfacesKernel(SurfaceArgs A) {
	const uint32_t n = *A.rays.count;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const kdn_hit hit    = A.hits[i];
		const kdn_ray ray    = A.rays.rays[i];
		const uint32_t px    = A.rays.paths[i];
		const bool found     = hit.kind != 0;
		float3 normal        = make_float3(0.0f, 0.0f, 0.0f);
		float3 albedo        = make_float3(0.0f, 0.0f, 0.0f);
		float distance       = __int_as_float(0x7f800000);
		if (found) {
			const float3 heading = make_float3(ray.direction[0], ray.direction[1], ray.direction[2]);
			normal               = make_float3(hit.normal[0], hit.normal[1], hit.normal[2]);
			if (dot3(normal, heading) >= 0.0f) normal = normal * -1.0f;
			albedo = albedoAt(hit, normal, A.looks);
			const float dx = hit.point[0] - ray.origin[0], dy = hit.point[1] - ray.origin[1], dz = hit.point[2] - ray.origin[2];
			distance       = sqrtf(dx * dx + dy * dy + dz * dz);
		}
		A.distance[px]       = __half_as_ushort(__float2half_rn(distance));
		A.leaf[px]           = found ? hit.leaf : kNoLeaf;
		A.normal[3 * px]     = __half_as_ushort(__float2half_rn(normal.x));
		A.normal[3 * px + 1] = __half_as_ushort(__float2half_rn(normal.y));
		A.normal[3 * px + 2] = __half_as_ushort(__float2half_rn(normal.z));
		A.albedo[3 * px]     = __half_as_ushort(__float2half_rn(albedo.x));
		A.albedo[3 * px + 1] = __half_as_ushort(__float2half_rn(albedo.y));
		A.albedo[3 * px + 2] = __half_as_ushort(__float2half_rn(albedo.z));
	}
}

// An own line of --use sampler=each_lamp_first (out of line: few frames
// draw with it): the line and the slot it answers into (1 + its rank).
__device__ __noinline__ void ownLine(const ShadowBuffers& S, uint32_t lineCapacity, uint32_t p, uint32_t rank, float3 from, float3 toward, float distance,
                                     float4 offer) {
	kdn_ray own    = makeRay(from, toward, distance, kNoMaterial);
	own.pad_[1]    = uint8_t(rank + 1);
	const uint32_t slot = warpSlot(S.count, true);
	if (slot < lineCapacity) {
		S.rays[slot]         = own;
		S.paths[slot]        = p;
		S.contribution[slot] = offer;
	}
}

// ---- K-shade ----
// Films, Extras: built for each, so that a frame without thin films, or
// without any of the rarer parts (scattering bodies, lamps other than quads
// and spheres, a physical sky or a glow, the sky map, own lines, a split),
// runs a kernel with no code for them (FrameConstants::films and ::extras
// pick one)
template <bool Films, bool Extras>
__global__ void __launch_bounds__(kBlock, 3) shadeKernel(const __grid_constant__ FrameConstants cFrame, ShadeArgs A) {
	const uint32_t n = *A.in.count;
	for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
		const uint32_t q = base + threadIdx.x;
		bool live        = q < n;
		bool onward      = false;
		bool lined       = false;
		kdn_ray next {};
		kdn_ray line {};
		float4 lineRadiance = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		uint32_t p = 0;
		// a ray whose march was carried, or a path whose shadow line is still
		// marching, waits a launch: its ray goes on from where its march stands
		bool resumes   = false;
		uint2 carryOut = make_uint2(0u, 0u);
		if (live) {
			p = A.in.paths[q];
			const uint8_t kind = A.hits[q].kind;
			if (kind == kHitCarried || (A.paths.state[p] & kLinesPending)) {
				const HitState h = A.states[q];
				// a landed march resumes a step before its landing and lands again
				const bool landed = h.kind == 1u || h.kind == 2u;
				next              = A.in.rays[q];
				next.pad_[0] |= kRayResumes;
				carryOut = make_uint2(__float_as_uint(h.distance), landed ? h.steps - 1u : h.steps);
				onward = resumes = true;
				live             = false;
			}
		}
		if (live) {
			const kdn_hit hit   = A.hits[q];
			const kdn_ray ray   = A.in.rays[q];
			const uint32_t st   = A.paths.state[p];
			// the surfaces stood on, the collisions inside scattering bodies,
			// and the path's depth (every vertex: the events its numbers follow)
			const int surfaceDepth    = int(st & 0xFFu);
			const uint32_t collisions = Extras && A.paths.collided != nullptr ? A.paths.collided[p] : 0u;
			const int depth           = surfaceDepth + int(collisions);
			const bool camera   = (st >> 8) & 1u;
			uint32_t medium     = (st >> 16) == 0 ? kNoMaterial : (st >> 16) - 1u;
			float4 T            = A.paths.throughput[p];
			float4 R            = A.paths.radiance[p];
			// the first vertex's own lines, all answered by now
			if (Extras && depth == 1 && A.paths.held != nullptr) {
				for (uint32_t k = 0; k < kOwnLines; ++k) {
					R                                        = add4(R, A.paths.held[size_t(p) * kOwnLines + k]);
					A.paths.held[size_t(p) * kOwnLines + k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
				}
			}
			const float4 nm     = A.paths.nanometres[p];
			const float drawnDensity = A.paths.drawn[p];
			// a training frame: the radiance held on reaching this vertex is
			// what the vertex before held once its own aim was answered
			if (A.records != nullptr && depth >= 1 && depth <= kGuideDepth) A.records[size_t(p) * kGuideDepth + depth - 1].before = R.x + R.y + R.z + R.w;
			const float3 heading = make_float3(ray.direction[0], ray.direction[1], ray.direction[2]);
			const float3 origin  = make_float3(ray.origin[0], ray.origin[1], ray.origin[2]);
			const bool found     = hit.kind != 0;
			// trace.cpp:179 keptOnLeg, absorption.cpp:28 keptThrough: what
			// the leg's body keeps over a distance, exp(-absorption x
			// distance) a lane; whole outside any body or where no glass absorbs
			const bool absorbing = medium != kNoMaterial && cFrame.absorbs != 0;
			float4 thickness     = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
			if (absorbing) {
				const DeviceMaterial& body = A.looks.materials[medium < cFrame.materialCount ? medium : 0u];
				thickness                  = spectrumOf(body.absorb[0], body.absorb[1], body.absorb[2], nm);
			}
			// trace.cpp:250 stopOf: a leg inside a scattering body collides
			// where a free flight drawn as -ln(1 - u) / scatter ends before its
			// hit (scattering.cpp:61 scatteredAlong; u the event's Collision
			// draw, trace.cpp:198 collisionNumber)
			bool collided    = false;
			float collidedAt = 0.0f;
			float flight     = __int_as_float(0x7f800000);
			if (Extras && cFrame.scatters && medium != kNoMaterial) {
				const DeviceMaterial& body = A.looks.materials[medium < cFrame.materialCount ? medium : 0u];
				if (body.scatter > 0.0f) {
					const uint32_t px    = A.paths.pixel[p];
					const uint64_t drawn = hashedBits(streamOf(cFrame, px % uint32_t(cFrame.width), px / uint32_t(cFrame.width)), A.paths.sample[p], kCollisionFirst + uint64_t(depth));
					const double far     = -log(1.0 - double(drawn) * 0x1p-53) / double(body.scatter);
					flight               = float(far);
					const float3 leg     = make_float3(hit.point[0] - A.paths.from[p].x, hit.point[1] - A.paths.from[p].y, hit.point[2] - A.paths.from[p].z);
					if (found && far < double(sqrtf(dot3(leg, leg)))) {
						collided   = true;
						collidedAt = flight;
					}
				}
			}
			// trace.cpp:218 keptAlong of the walked leg; a scattering body's
			// absorption reaches only as far as the drawn flight
			// (feature.cpp:358 mediumAlong over collisionAlong's `at`)
			const auto keptOver = [&](float distance) {
				const float reach = fminf(distance, flight);
				return absorbing ? make_float4(expf(-thickness.x * reach), expf(-thickness.y * reach), expf(-thickness.z * reach), expf(-thickness.w * reach))
				                 : make_float4(1.0f, 1.0f, 1.0f, 1.0f);
			};
			// meet: lamps along the leg (not for camera legs) and the sky past it
			if (!camera) {
				const float limit = collided ? collidedAt : (found ? hit.distance : 3.0e38f);
				const float3 from = make_float3(A.paths.from[p].x, A.paths.from[p].y, A.paths.from[p].z);
				for (uint32_t k = 0; k < cFrame.lampCount; ++k) {
					const DeviceLamp& l = cFrame.lamps[k];
					float reach;
					if (Extras ? !meetLamp(l, origin, heading, limit, reach) : !meetArea(l, origin, heading, limit, reach)) continue;
					float w = 1.0f;
					if (drawnDensity > 0.0f) {
						// weight.cpp:15 sharedAim: the first vertex's aim counts once a group
						const float pa = Extras ? aimDensityOf(l, from, heading, reach) / (depth == 1 ? float(cFrame.split) : 1.0f) : areaDensityOf(l, from, heading, reach);
						w              = drawnDensity * drawnDensity / (drawnDensity * drawnDensity + pa * pa);
					}
					float4 lit = mul4(mul4(T, keptOver(reach)), spectrumOf(l.radiance[0], l.radiance[1], l.radiance[2], nm));
					if (Extras) {
						lit = mul4(lit, lampTint(cFrame, k, nm));
						w *= moonLit(cFrame, l, heading);
					}
					R = add4(R, scale4(lit, w));
				}
			}
			// the record's first surface of the pixel's last sample
			// (trace.cpp:1469 recordedStand, :1445 vertexSurface; missed: batch.cpp:46)
			if (camera && A.firstLeaf != nullptr && A.paths.sample[p] + 1u == cFrame.firstSample + cFrame.spp) {
				const uint32_t px = A.paths.pixel[p];
				float3 n          = make_float3(0.0f, 0.0f, 0.0f);
				float3 albedo     = make_float3(0.0f, 0.0f, 0.0f);
				float distance    = __int_as_float(0x7f800000);
				if (found) {
					n = make_float3(hit.normal[0], hit.normal[1], hit.normal[2]);
					if (dot3(n, heading) >= 0.0f) n = n * -1.0f;
					albedo         = albedoAt(hit, n, A.looks);
					const float3 d = make_float3(hit.point[0], hit.point[1], hit.point[2]) - origin;
					distance       = sqrtf(dot3(d, d));
				}
				A.firstDistance[px]       = __half_as_ushort(__float2half_rn(distance));
				A.firstLeaf[px]           = found ? hit.leaf : kNoLeaf;
				A.firstNormal[3 * px]     = __half_as_ushort(__float2half_rn(n.x));
				A.firstNormal[3 * px + 1] = __half_as_ushort(__float2half_rn(n.y));
				A.firstNormal[3 * px + 2] = __half_as_ushort(__float2half_rn(n.z));
				A.firstAlbedo[3 * px]     = __half_as_ushort(__float2half_rn(albedo.x));
				A.firstAlbedo[3 * px + 1] = __half_as_ushort(__float2half_rn(albedo.y));
				A.firstAlbedo[3 * px + 2] = __half_as_ushort(__float2half_rn(albedo.z));
			}
			if (!found) {
				// the sky met, weighed against aiming at it by its chart
				// (trace.cpp:294 meetAimDensity, sampler.cpp:344 aimDensityAt)
				float4 sky;
				if (Extras) {
					sky = skySpectrum(cFrame, heading, nm);
				} else {
					const float3 rgb = skyColour(cFrame, heading);
					sky              = spectrumOf(rgb.x, rgb.y, rgb.z, nm);
				}
				float w          = 1.0f;
				if (Extras && drawnDensity > 0.0f && cFrame.skyChart != nullptr) {
					const float pa = float(chartDensity(cFrame.skyChart, heading.x, heading.y, heading.z)) / (depth == 1 ? float(cFrame.split) : 1.0f);
					w              = drawnDensity * drawnDensity / (drawnDensity * drawnDensity + pa * pa);
				}
				R = add4(R, scale4(mul4(mul4(T, keptOver(__int_as_float(0x7f800000))), sky), w));
			} else if (Extras && collided) {
				// trace.cpp:502 collidedOn: the phase vertex (trace.cpp:474
				// phaseVertex) at the collision, what the leg's body kept up
				// to it; a bending body is not aimed from (trace.cpp:579
				// aimsFromCollision), so the vertex only scatters
				const DeviceMaterial& body = A.looks.materials[medium < cFrame.materialCount ? medium : 0u];
				const float3 point         = make_float3(A.paths.from[p].x, A.paths.from[p].y, A.paths.from[p].z) + heading * collidedAt;
				if (absorbing) T = mul4(T, keptOver(collidedAt));
				const uint32_t stood = collisions + 1u;
				// weight.cpp:23 atDepthCap: the surfaces stood on, or the collisions
				if (surfaceDepth < cFrame.surfaces && stood < cFrame.collisionCap) {
					const uint32_t px     = A.paths.pixel[p];
					const uint64_t stream = streamOf(cFrame, px % uint32_t(cFrame.width), px / uint32_t(cFrame.width));
					const uint32_t index  = A.paths.sample[p];
					const float3 incoming = phaseDirection(body.lean, heading, number(cFrame.sobol, stream, index, depth, DirectionU),
					                                       number(cFrame.sobol, stream, index, depth, DirectionV));
					float4 carried        = T; // the phase's weight is 1
					bool alive            = true;
					if (depth >= 4) {
						const float survival = fminf(0.95f, max4(carried));
						if (!(number(cFrame.sobol, stream, index, depth, Survival) < survival)) alive = false;
						else carried = scale4(carried, 1.0f / survival);
					}
					if (alive) {
						onward              = true;
						T                   = carried;
						next                = makeRay(point, incoming, __int_as_float(0x7f800000), medium);
						A.paths.drawn[p]    = 0.0f; // the next leg's meets take their light whole
						A.paths.from[p]     = make_float4(point.x, point.y, point.z, 0.0f);
						A.paths.collided[p] = stood;
						A.paths.state[p]    = uint32_t(surfaceDepth) | (st & (1u << 9)) | ((medium + 1u) << 16);
					}
				}
			} else {
				const uint32_t material = hit.leaf < A.looks.leafCount ? A.looks.leafMaterial[hit.leaf] : 0u;
				const DeviceMaterial& m = A.looks.materials[material < cFrame.materialCount ? material : 0u];
				const float3 point      = make_float3(hit.point[0], hit.point[1], hit.point[2]);
				float3 normal           = make_float3(hit.normal[0], hit.normal[1], hit.normal[2]);
				// trace.cpp:529 stoodOn: the leg's body keeps its share
				if (absorbing) {
					const float3 leg = point - origin;
					T                = mul4(T, keptOver(sqrtf(dot3(leg, leg))));
				}
				// meet a glow (trace.cpp:415 metGlow): the glow bsdfAt gives
				// where the ray arrives from outside, mixed across a blend
				// seam; no sampler aims at it, so the meet takes it whole
				if (dot3(normal, heading) < 0.0f) {
					float3 glow = make_float3(m.glow[0], m.glow[1], m.glow[2]);
					if (hit.other != kNoLeaf && hit.share > 0.0f) {
						const DeviceMaterial& o = materialOfLeaf(hit.other, A.looks);
						const float s           = hit.share;
						glow = make_float3(glow.x * (1.0f - s) + o.glow[0] * s, glow.y * (1.0f - s) + o.glow[1] * s, glow.z * (1.0f - s) + o.glow[2] * s);
					}
					if (glow.x > 0.0f || glow.y > 0.0f || glow.z > 0.0f) R = add4(R, mul4(T, spectrumOf(glow.x, glow.y, glow.z, nm)));
				}
				if (dot3(normal, heading) >= 0.0f) normal = normal * -1.0f;
				const float4 T0         = T; // what reached this vertex
				const float lift        = kBias + 2.0f * hit.loosened;
				const uint32_t x        = A.paths.pixel[p] % uint32_t(cFrame.width);
				const uint32_t y        = A.paths.pixel[p] / uint32_t(cFrame.width);
				const uint64_t stream   = streamOf(cFrame, x, y);
				const uint32_t index    = A.paths.sample[p];
				const bool capped       = surfaceDepth + 1 >= cFrame.surfaces || collisions >= cFrame.collisionCap;
				const float3 outgoing   = heading * -1.0f;
				const float3 rgb        = albedoAt(hit, normal, A.looks);
				const Shading surf      = surfaceOf<Films>(m, rgb, normal, outgoing, nm, medium, A.looks.materials, A.looks.boundaries);
				// trace.cpp:583 aimable: from outside every body, or from inside
				// the glass being crossed where it bends; trace.cpp:590
				// openSide: the side a line leaves by
				const bool aimable = medium == kNoMaterial || (medium == material && m.kind == 3 && surf.within.x != surf.beyond.x);
				// the learned guide's lobes at this vertex (one-sample MIS with the BSDF)
				const float* lobes = (A.lobes != nullptr && depth < kGuideDepth && guidable(m.kind)) ? A.lobes + size_t(q) * kGuideLobeFloats : nullptr;
				const float share  = A.guideShare;
				const float3 open  = surf.inside ? normal * -1.0f : normal;
				// aim: offer every lamp and a charted sky (the light after the
				// lamps, sampler.cpp:312 skyAim), trace one offer drawn by its
				// lane mean; with --use sampler=each_lamp_first each of the
				// first kOwnLines lamps whose offer is bright traces a line of
				// its own at the first vertex, outside the reservoir
				// (trace.cpp:935, each_lamp_first.cpp:7 eachLampFirst)
				if (!m.exact && aimable && (cFrame.lampCount > 0 || (Extras && cFrame.skyChart != nullptr))) {
					uint32_t owned   = 0;
					// the first vertex's aim is shared by a group (path.cpp:37 sharedDraw)
					// and counts once a group in its weight (weight.cpp:15 sharedAim)
					const uint32_t aimIndex = Extras && depth == 0 ? index / cFrame.split : index;
					const float aimCount    = Extras && depth == 0 ? 1.0f / float(cFrame.split) : 1.0f;
					const float u0   = number(cFrame.sobol, stream, aimIndex, depth, LightU);
					const float v0   = number(cFrame.sobol, stream, aimIndex, depth, LightV);
					float choice     = number(cFrame.sobol, stream, aimIndex, depth, Pick);
					float total      = 0.0f, picked = 0.0f;
					float4 chosen    = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
					float3 chosenDir = make_float3(0.0f, 0.0f, 1.0f);
					float chosenDist = 0.0f;
					for (uint32_t k = 0; k < cFrame.lampCount + (Extras && cFrame.skyChart != nullptr ? 1u : 0u); ++k) {
						Aim a = k < cFrame.lampCount ? (Extras ? aimLamp(cFrame.lamps[k], point, u0, v0) : aimArea(cFrame.lamps[k], point, u0, v0))
						                                   : aimSky(cFrame, u0, v0, plainNumber(stream, aimIndex, depth, AimPart), plainNumber(stream, aimIndex, depth, AimJitterU),
						                                            plainNumber(stream, aimIndex, depth, AimJitterV));
						if (!a.found) continue;
						if (Extras && k < cFrame.lampCount) a.arriving = a.arriving * moonLit(cFrame, cFrame.lamps[k], a.toward);
						const float facing = dot3(open, a.toward);
						if (facing <= 0.0f || a.distance <= 0.0f) continue;
						const Response f = respond(surf, m, outgoing, a.toward, nm);
						float w          = 1.0f;
						if (a.density > 0.0f) {
							const float pm = capped ? 0.0f : (lobes ? share * mixtureDensity(lobes, a.toward) + (1.0f - share) * f.density : f.density);
							const float pa = a.density * aimCount;
							w              = pa * pa / (pa * pa + pm * pm);
						}
						float4 arriving    = spectrumOf(a.arriving.x, a.arriving.y, a.arriving.z, nm);
						if (Extras && k < cFrame.lampCount) arriving = mul4(arriving, lampTint(cFrame, k, nm));
						const float4 offer = scale4(mul4(mul4(T, f.value), arriving), facing * w);
						const float weight = mean4(offer);
						if (!(weight > 0.0f)) continue;
						if (Extras && cFrame.eachLamp && depth == 0 && k < cFrame.lampCount && owned < kOwnLines) {
							ownLine(A.shadow, A.lineCapacity, p, owned++, point + open * lift, a.toward, a.distance - lift, offer);
							continue;
						}
						total           = total + weight;
						const float keep = weight / total;
						if (choice < keep) {
							chosen     = offer;
							picked     = weight;
							chosenDir  = a.toward;
							chosenDist = a.distance;
							choice     = choice / keep;
						} else {
							choice = (choice - keep) / (1.0f - keep);
						}
					}
					if (picked > 0.0f) {
						lined        = true;
						lineRadiance = scale4(chosen, total / picked);
						line         = makeRay(point + open * lift, chosenDir, chosenDist - lift, kNoMaterial);
					}
				}
				// scatter (trace.cpp:1020 scatteredFrom)
				if (!capped) {
					float lobe       = number(cFrame.sobol, stream, index, depth, Lobe);
					const float side = number(cFrame.sobol, stream, index, depth, Side);
					const float du   = number(cFrame.sobol, stream, index, depth, DirectionU);
					const float dv   = number(cFrame.sobol, stream, index, depth, DirectionV);
					Scatter s;
					if (lobes != nullptr && lobe < share) {
						// drawn from the guide: weighed by the mixture's density
						s               = noScatter();
						s.incoming      = mixtureSample(lobes, lobe / share, du, dv);
						const Response f = respond(surf, m, outgoing, s.incoming, nm);
						s.density       = share * mixtureDensity(lobes, s.incoming) + (1.0f - share) * f.density;
						const float cosine = fabsf(dot3(s.incoming, normal));
						s.found         = s.density > 0.0f && max4(f.value) > 0.0f;
						s.weight        = scale4(f.value, cosine / fmaxf(s.density, 1e-30f));
					} else {
						if (lobes != nullptr) lobe = (lobe - share) / (1.0f - share);
						s = sampleSurface(surf, m, outgoing, nm, lobe, side, du, dv, material, medium);
						if (lobes != nullptr && s.found && !s.delta) {
							// the BSDF's draw weighed by the mixture's density
							const Response f   = respond(surf, m, outgoing, s.incoming, nm);
							s.density          = share * mixtureDensity(lobes, s.incoming) + (1.0f - share) * f.density;
							const float cosine = fabsf(dot3(s.incoming, normal));
							s.weight           = scale4(f.value, cosine / fmaxf(s.density, 1e-30f));
						}
					}
					const float sideOf = dot3(s.incoming, normal);
					const bool below   = s.through ? sideOf >= 0.0f : sideOf <= 0.0f;
					if (s.found && !below) {
						float4 carried  = mul4(T, s.weight);
						// trace.cpp:961 carriedThroughput: past a dispersing bend only the hero lane goes on
						const bool wasDispersed = (st >> 9) & 1u;
						if (s.dispersed && !wasDispersed) carried = make_float4(carried.x * 4.0f, 0.0f, 0.0f, 0.0f);
						bool alive      = true;
						if (depth >= 4) {
							const float survival = fminf(0.95f, max4(carried));
							if (!(number(cFrame.sobol, stream, index, depth, Survival) < survival)) alive = false;
							else carried = scale4(carried, 1.0f / survival);
						}
						if (alive) {
							// trace.cpp:956 aimedAlong: the next leg's meets are weighed
							// against aiming where the scatter left by the open side of
							// an aimable vertex
							const bool aimed = !s.delta && s.density > 0.0f && s.through == (medium != kNoMaterial) && aimable;
							if (s.through) medium = s.mediumAfter;
							onward                = true;
							T                     = carried;
							const float off       = sideOf > 0.0f ? lift : -lift;
							next                  = makeRay(point + normal * off, s.incoming, __int_as_float(0x7f800000), medium);
							A.paths.drawn[p]      = aimed ? s.density : 0.0f;
							if (A.records != nullptr && depth < kGuideDepth && guidable(m.kind)) {
								GuideRecord& r = A.records[size_t(p) * kGuideDepth + depth];
								r.point[0] = point.x, r.point[1] = point.y, r.point[2] = point.z;
								r.normal[0] = normal.x, r.normal[1] = normal.y, r.normal[2] = normal.z;
								r.direction[0] = s.incoming.x, r.direction[1] = s.incoming.y, r.direction[2] = s.incoming.z;
								r.reached = T0.x + T0.y + T0.z + T0.w;
							}
							A.paths.from[p]       = make_float4(point.x, point.y, point.z, 0.0f);
							uint32_t stNext       = uint32_t(surfaceDepth + 1) | (medium == kNoMaterial ? 0u : ((medium + 1u) << 16));
							if (s.dispersed || ((st >> 9) & 1u)) stNext |= 1u << 9;
							A.paths.state[p]      = stNext;
						}
					}
				}
			}
			A.paths.throughput[p] = T;
			A.paths.radiance[p]   = R;
		}
		const uint32_t slot = warpSlot(A.out.count, onward);
		if (onward && slot < A.capacity) {
			A.out.paths[slot] = p;
			A.out.rays[slot]  = next;
			if (resumes) A.out.carry[slot] = carryOut;
		}
		const uint32_t lineSlot = warpSlot(A.shadow.count, lined);
		if (lined && lineSlot < A.lineCapacity) {
			A.shadow.rays[lineSlot]         = line;
			A.shadow.paths[lineSlot]        = p;
			A.shadow.contribution[lineSlot] = lineRadiance;
		}
	}
}

// ---- K-line: add each shadow line that reached its lamp (trace.cpp:1294 lineAnswered) ----
// A line whose march was carried goes on in the next launch (out) and its
// path waits for it (kLinesPending counts it in); an answered line that had
// been carried counts out.  A path has at most one reservoir line in flight
// and, at its first vertex with own lines, kOwnLines more: each own line
// answers into its own held slot, so no two threads add to one path.
__global__ void __launch_bounds__(kBlock) linesKernel(PathBuffers P, ShadowBuffers S, ShadowBuffers out, uint32_t capacity) {
	const uint32_t n = *S.count;
	for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
		const uint32_t s = base + threadIdx.x;
		bool carried     = false;
		HitState h {};
		uint32_t p = 0;
		if (s < n) {
			h       = S.states[s];
			p       = S.paths[s];
			carried = h.kind == kCarried;
			const kdn_ray& r = S.rays[s];
			const bool resumed = r.pad_[0] & kRayResumes;
			if (!carried) {
				if (r.pad_[1] != 0) {
					P.held[size_t(p) * kOwnLines + (r.pad_[1] - 1u)] = h.kind == 0 ? S.contribution[s] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
				} else if (h.kind == 0) {
					P.radiance[p] = add4(P.radiance[p], S.contribution[s]);
				}
				if (resumed) atomicSub(&P.state[p], kLineWaiting);
			} else if (!resumed) {
				atomicAdd(&P.state[p], kLineWaiting);
			}
		}
		const uint32_t slot = warpSlot(out.count, carried);
		if (carried && slot < capacity) {
			kdn_ray r = S.rays[s];
			r.pad_[0] |= kRayResumes;
			out.rays[slot]         = r;
			out.carry[slot]        = make_uint2(__float_as_uint(h.distance), h.steps);
			out.paths[slot]        = p;
			out.contribution[slot] = S.contribution[s];
		}
	}
}

// ---- K-fold: per pixel, the samples' colours (frame.cpp:273 foldPixels) ----
// With light, also this call's mean a pixel (the frame record's light).
__global__ void __launch_bounds__(kBlock) foldKernel(const __grid_constant__ FrameConstants cFrame, PathBuffers P, uint32_t firstPixel, uint32_t pixels, uint32_t spp, double* sums, float* light) {
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < pixels; i += gridDim.x * blockDim.x) {
		double r = 0.0, g = 0.0, b = 0.0;
		for (uint32_t k = 0; k < spp; ++k) {
			const uint32_t p = i * spp + k;
			float4 radiance  = P.radiance[p];
			// own lines of a path that ended at its first vertex
			if (P.held != nullptr) {
				for (uint32_t o = 0; o < kOwnLines; ++o) radiance = add4(radiance, P.held[size_t(p) * kOwnLines + o]);
			}
			const float3 c   = colourOf(cFrame, P.nanometres[p], P.density[p], radiance);
			r += double(c.x);
			g += double(c.y);
			b += double(c.z);
		}
		double* s = sums + 3ull * (firstPixel + i);
		s[0] += r;
		s[1] += g;
		s[2] += b;
		if (light) {
			float* l = light + 3ull * (firstPixel + i);
			l[0]     = float(r / double(spp));
			l[1]     = float(g / double(spp));
			l[2]     = float(b / double(spp));
		}
	}
}

__global__ void __launch_bounds__(kBlock) meansKernel(const double* sums, uint32_t pixels, double taken, float* out) {
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < pixels * 3u; i += gridDim.x * blockDim.x) {
		out[i] = float(sums[i] / taken);
	}
}

uint32_t gridFor(uint64_t n, int smCount) {
	const uint64_t blocks = (n + kBlock - 1) / kBlock;
	return uint32_t(std::max<uint64_t>(1, std::min<uint64_t>(blocks, uint64_t(smCount) * 16)));
}

} // namespace

cudaError_t launchCamera(const FrameConstants& frame, const PathBuffers& paths, const QueueBuffers& queue, uint32_t firstPixel, uint32_t n, cudaStream_t stream, int smCount) {
	cameraKernel<<<gridFor(n, smCount), kBlock, 0, stream>>>(frame, paths, queue, firstPixel, n);
	return cudaGetLastError();
}

cudaError_t launchShade(const FrameConstants& frame, const ShadeArgs& args, cudaStream_t stream, int smCount) {
	const uint32_t grid = gridFor(args.capacity, smCount);
	if (frame.films && frame.extras) shadeKernel<true, true><<<grid, kBlock, 0, stream>>>(frame, args);
	else if (frame.films) shadeKernel<true, false><<<grid, kBlock, 0, stream>>>(frame, args);
	else if (frame.extras) shadeKernel<false, true><<<grid, kBlock, 0, stream>>>(frame, args);
	else shadeKernel<false, false><<<grid, kBlock, 0, stream>>>(frame, args);
	return cudaGetLastError();
}

cudaError_t launchLines(const PathBuffers& paths, const ShadowBuffers& in, const ShadowBuffers& out, uint32_t capacity, cudaStream_t stream, int smCount) {
	linesKernel<<<gridFor(capacity, smCount), kBlock, 0, stream>>>(paths, in, out, capacity);
	return cudaGetLastError();
}

cudaError_t launchFold(const FrameConstants& frame, const PathBuffers& paths, uint32_t firstPixel, uint32_t pixels, uint32_t spp, double* sums, float* light, cudaStream_t stream, int smCount) {
	foldKernel<<<gridFor(pixels, smCount), kBlock, 0, stream>>>(frame, paths, firstPixel, pixels, spp, sums, light);
	return cudaGetLastError();
}

cudaError_t launchSurfaceRays(const FrameConstants& frame, const QueueBuffers& queue, uint32_t firstPixel, uint32_t n, cudaStream_t stream, int smCount) {
	surfaceRaysKernel<<<gridFor(n, smCount), kBlock, 0, stream>>>(frame, queue, firstPixel, n);
	return cudaGetLastError();
}

cudaError_t launchSurfaces(const SurfaceArgs& args, uint32_t n, cudaStream_t stream, int smCount) {
	surfacesKernel<<<gridFor(n, smCount), kBlock, 0, stream>>>(args);
	return cudaGetLastError();
}

cudaError_t launchMeans(const double* sums, uint32_t pixels, double taken, float* out, cudaStream_t stream, int smCount) {
	meansKernel<<<gridFor(uint64_t(pixels) * 3, smCount), kBlock, 0, stream>>>(sums, pixels, taken, out);
	return cudaGetLastError();
}

} // namespace kdn
