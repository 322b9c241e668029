// Device-side description of one frame: lens, lamps, sky, materials and the
// wavefront buffers of the path tracer.
#pragma once

#include "kdn.h"
#include "kernels.h"
#include "spectral.h"
#include "world.h"

#include <cuda_runtime.h>

#include <cstdint>

namespace kdn {

constexpr uint32_t kMaxLamps = 16;
constexpr uint32_t kNoMaterial = 0xFFFFFFFFu;

// A lamp with what aiming at it and meeting it read, worked out once
// (plugins/transport/paths/light/light.cpp:78 lampOf).
struct DeviceLamp {
	uint32_t kind;   // sdf/scene.h LightKind: 0 point, 1 directional, 2 sphere, 3 quad, 4 sun, 5 moon
	uint32_t square; // a quad whose edges are at right angles (light.cpp:145 squareQuad)
	float at[3], along[3], across[3], facing[3], cross[3];
	float ex[3], ey[3], raw[3];
	float alongLength, acrossLength;
	float radius, area;
	float radiance[3], power[3];
	// a directional light, a sun or a moon: the unit direction toward it;
	// a sun or a moon: 1 - the cosine of its disc's half angle (the cone
	// it is aimed in, kept apart from 1 so that a small disc keeps its size)
	float direction[3];
	float oneLess;
	// a moon: its direction and the sine of its half angle in double, for
	// the lit share of its disc (sky_layers.cpp:273 moonLit)
	double disc[3];
	double discRadius;
};

// What the transport reads of a material (sdf/scene.h Material and the
// finish the reference derives from it, material.cpp:204 finishWith).
struct DeviceMaterial {
	uint32_t kind;
	float albedo[3];
	float roughness;
	float index;      // refraction (glass), 1 otherwise
	float dispersion; // Cauchy B, square micrometres
	float absorb[3];
	float width;      // GGX width of the facets
	float facetShare; // share of facet sampling for metal
	float body;       // mean luminance of the albedo
	float escapeAverage;
	float coatFront, coatTwice, coatRoom;
	uint32_t exact;   // a smooth glass answered exactly
	uint32_t sharp;
	float glow[3];    // material.cpp:325 glowOf: the glow colour times its strength
	uint32_t world;   // the pattern is read in world space (sdf/scene.h Albedo::world)
	float escape[32]; // material/energy.h:12 Escape: the share a view keeps after one scatter
	// sdf/scene.h Albedo as a ramp over a pattern program: its steps in the
	// frame's pattern steps (count 0: the flat albedo) and its stops (3
	// floats each) in the frame's stops
	uint32_t patternFirst, patternCount, patternResult;
	uint32_t stopFirst, stopCount;
	// a rough glass: gives back what single scattering loses, read off its
	// boundary tables (kBoundaryFloats floats at boundaryFirst of Looks::boundaries)
	uint32_t losesMuch, boundaryFirst;
	// material.cpp:106 filmOf: the thin film a metal, plastic or glass wears
	// (thickness in nanometres, 0 for none; its index)
	float filmThickness, filmIndex;
	// scattering.cpp:7 scatters: a glass whose body turns aside `scatter` a
	// unit of travel (0: none), by Henyey-Greenstein's phase of g = lean
	float scatter, lean;
};

// material/energy.h Boundary as floats: rarer and denser (17 ratios x 32
// views each), then 17 rarer averages, 17 denser averages, 17 rarer-through
// shares.
constexpr int kBoundaryRatios = 17, kBoundaryViews = 32;
constexpr int kBoundaryFloats = 2 * kBoundaryRatios * kBoundaryViews + 3 * kBoundaryRatios;

// A step of a pattern program (sdf/program.h Step) on the device: operands
// are steps of the same program (a pattern has at most kPatternSteps), an
// argument is folded to the constant it reads.
constexpr uint32_t kPatternSteps = 64;
struct PatternStep {
	uint8_t op;
	uint8_t a, b, c;
	float value;
};

// What the albedo at a hit reads (material.cpp:345 bsdfAt): the materials,
// each leaf's material and placement (12 floats: linear row by row, then
// origin), the pattern steps and the ramps' stops.
struct Looks {
	const DeviceMaterial* materials;
	const uint32_t* leafMaterial;
	uint32_t leafCount;
	uint32_t placementCount;
	const float* placements;
	const PatternStep* patternSteps;
	const float* stops;
	const float* boundaries;
	uint32_t materialCount;
};

struct FrameConstants {
	float eye[3], forward[3], right[3], up[3];
	float reach, aspect;
	// core/camera.cpp:9 lensOf: a thin lens's radius (0: a pinhole) and the
	// distance it is sharp at along the forward axis
	float aperture, focus;
	int32_t width, height;
	uint64_t seedMix;
	int32_t surfaces;
	uint32_t spp;
	uint32_t firstSample;
	uint32_t lampCount;
	uint32_t materialCount;
	uint32_t absorbs; // absorption.cpp:18 sceneAbsorbs: some glass absorbs
	uint32_t films;   // some metal, plastic or glass wears a thin film
	// core/camera.h:65 FilmPlan: a drawn pixel's samples aim at the shown
	// pixel (x * factor + phase % factor, y * factor + phase / factor); its
	// G-buffer ray passes through that pixel's centre (core/camera.cpp:51
	// filmCentre, in drawn pixels)
	uint32_t factor, phase;
	float centre[2];
	// --use sampler=sobol: the Sobol byte tables (sobol.h), or null for
	// independent numbers
	const uint32_t* sobol;
	// --use sampler=sky_map: the sky's chart (skymap.h), or null where the
	// sky is only met
	const double* skyChart;
	// --use sampler=each_lamp_first: at the first vertex each of the first
	// kOwnLines lamps whose offer is bright traces a line of its own
	uint32_t eachLamp;
	// scattering.cpp:29 sceneScatters: some glass body scatters; render.h
	// collisions: the most collisions a path stands on (weight.cpp:23 atDepthCap)
	uint32_t scatters;
	uint32_t collisionCap;
	// render.split: how many samples share a first vertex (1: none)
	uint32_t split;
	// any of the rarer parts the plain shade kernel leaves out: scattering
	// bodies, lamps other than quads and spheres, a physical sky or a glow,
	// the sky map, own lines, a split
	uint32_t extras;
	float zenith[3], horizon[3], ground[3];
	// sdf/scene.cpp:306 firstSun: the first sun's unit direction, where the
	// scene has one (a moon's phase follows it)
	double sunDirection[3];
	uint32_t hasSun;
	// a physical sky lit by the first sun (atmosphere.h): the air's and the
	// haze's tables (kAirTable floats each, null for none), the sky's frame,
	// the sun's light thinned to the ground (`sunLamp` the lamp it thins) and
	// what lands on the ground, the sunlight above the air and the ground's albedo
	const float* airTables;
	float airUp[3], airSun[3], airLevel[3], airAside[3];
	float airPassed[33], airLanding[33];
	float sunlight[3], airGround[3];
	uint32_t sunLamp;
	// sky_layers.cpp:181 glowSeen: the glow about the first sun (its colour
	// times its strength, the angle it falls by e over, the sun's elevation)
	uint32_t glows;
	float glow[3], glowSpread, sunElevation;
	// sky_layers.cpp:240 starlight: the stars (count over the sphere, the
	// brightest's strength, a disc's angle), seen above the horizon at night
	uint32_t stars;
	float starCount, starStrength, starAngle, starNight;
	DeviceLamp lamps[kMaxLamps];
	SpectralTables spectral;
};

// The wavefront state of one chunk of paths, structure of arrays.
struct PathBuffers {
	uint32_t* pixel;      // pixel index within the frame
	uint32_t* sample;     // sample index of the pixel
	float4* throughput;   // four lanes
	float4* radiance;
	float4* nanometres;
	float4* density;
	float* drawn;         // density of the last scattered direction, 0 when exact
	uint32_t* state;      // depth (bits 0-7), camera leg (bit 8), dispersed (bit 9), lines pending (bits 10-12), medium + 1 (bits 16-31)
	float4* from;         // xyz: where the leg was drawn from
	// with --use sampler=each_lamp_first: what each own line of the first
	// vertex brought (kOwnLines a path, in the lamps' order; zero where none
	// or blocked), added to the radiance at the next vertex or at the fold
	float4* held;
	// where a body scatters: the collisions each path has stood on (the
	// path's depth is state's surface count plus these)
	uint32_t* collided;
};

// PathBuffers::state bits 10-12: how many of the path's shadow lines were
// carried to a later trace launch and are not answered yet; while any is,
// the path's next vertex waits (its radiance takes the lines' shares before
// the next vertex's meets, in the order of a frame without a march budget).
constexpr uint32_t kLineWaiting  = 1u << 10;
constexpr uint32_t kLinesPending = 7u << 10;

// plugins/sampler/each_lamp_first/each_lamp_first.cpp:5 lampsWithOwnRay:
// the lamps that trace a line of their own at the first vertex; a path
// holds at most this many lines beside the reservoir's one.
constexpr uint32_t kOwnLines = 4;

struct QueueBuffers {
	uint32_t* paths;      // path index of each queued ray
	kdn_ray* rays;
	uint32_t* count;      // device count
	uint2* carry;         // resume data of each ray slot (TraceArgs::carry)
};

struct ShadowBuffers {
	kdn_ray* rays;
	uint32_t* paths;
	float4* contribution;
	uint32_t* count;
	HitState* states;
	uint2* carry;         // resume data of each line slot
};

struct ShadeArgs {
	PathBuffers paths;
	QueueBuffers in;
	QueueBuffers out;
	ShadowBuffers shadow;
	const kdn_hit* hits;
	const HitState* states; // where each ray's march ended (a held path resumes there)
	Looks looks;
	uint32_t capacity;
	uint32_t lineCapacity; // the shadow queue's room: capacity, or (1 + kOwnLines) capacity with own lines
	uint32_t* error;
	// where set (a denoised frame), the first surface of each pixel's last
	// sample (core/frame.cpp record surfaces): FP16 bits, the leaf
	uint16_t* firstDistance;
	uint16_t* firstNormal;
	uint16_t* firstAlbedo;
	uint32_t* firstLeaf;
	// the learned guide: where set, each queue entry's lobes (kGuideLobeFloats
	// floats, written for guidable hits), and the share of guided draws; the
	// records of a training frame (kGuideDepth a path)
	const float* lobes;
	float guideShare;
	struct GuideRecord* records;
};

// The surfaces pass: the first surface through each pixel's centre, as the
// denoiser's features (FP16 bits; leaf 0xFFFFFFFF where the ray missed).
struct SurfaceArgs {
	QueueBuffers rays;    // paths[i] is the pixel of ray i
	const kdn_hit* hits;
	Looks looks;
	uint16_t* distance;
	uint16_t* normal;
	uint16_t* albedo;
	uint32_t* leaf;
};

cudaError_t launchCamera(const FrameConstants& frame, const PathBuffers& paths, const QueueBuffers& queue, uint32_t firstPixel, uint32_t n, cudaStream_t stream, int smCount);
cudaError_t launchShade(const FrameConstants& frame, const ShadeArgs& args, cudaStream_t stream, int smCount);
// Answers the lines traced in a launch (in); carried lines go on in out.
cudaError_t launchLines(const PathBuffers& paths, const ShadowBuffers& in, const ShadowBuffers& out, uint32_t capacity, cudaStream_t stream, int smCount);
// light (may be null): each pixel's mean of this call's samples, RGB float
cudaError_t launchFold(const FrameConstants& frame, const PathBuffers& paths, uint32_t firstPixel, uint32_t pixels, uint32_t spp, double* sums, float* light, cudaStream_t stream, int smCount);
cudaError_t launchMeans(const double* sums, uint32_t pixels, double taken, float* out, cudaStream_t stream, int smCount);
cudaError_t launchSurfaceRays(const FrameConstants& frame, const QueueBuffers& queue, uint32_t firstPixel, uint32_t n, cudaStream_t stream, int smCount);
cudaError_t launchSurfaces(const SurfaceArgs& args, uint32_t n, cudaStream_t stream, int smCount);

} // namespace kdn
