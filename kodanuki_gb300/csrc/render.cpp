// Frame entry points: kdn_render and kdn_render_device.
//
// A frame's paths are drawn in chunks of whole pixels (all samples of a pixel
// in one chunk, pixel-major), each chunk driven through the wavefront:
//   K-cam -> [K-trace -> K-hit -> K-shade -> K-trace(lines) -> K-line] x surfaces -> K-fold
// with every queue count kept on the device, so a chunk runs with no host
// synchronisation.  Pixel sums are kept in double on the device and persist
// across calls (progressive accumulation) until a call starts afresh.
#include "context.h"
#include "atmosphere.h"
#include "skymap.h"
#include "sobol.h"
#include "temporal.h"
#include "upscale.h"
#include "frame.h"
#include "guide.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace kdn {

// Streams a frame's chunks go round (render lanes).
constexpr int kLanes = 4;
static_assert(kLanes >= 1 && kLanes <= 64, "a lane takes one of the context's 64 fetch counters");

struct FrameState {
	DeviceBuffer pixel, sample, throughput, radiance, nanometres, density, drawn, state, from;
	DeviceBuffer queuePaths[2], queueRays[2], queueCarry[2], hits, states, counts;
	DeviceBuffer shadowPaths[2], shadowContribution[2];
	DeviceBuffer held;     // the own lines' answers (--use sampler=each_lamp_first)
	DeviceBuffer collided; // each path's collisions inside scattering bodies
	// the surfaces pass's own queue, states and hits, so it runs beside the
	// lanes' chunks on its own stream
	DeviceBuffer surfacePaths, surfaceRays, surfaceStates, surfaceHits;
	uint32_t surfaceCapacity = 0;
	DeviceBuffer sums, out, materials;
	DeviceBuffer patternSteps, stops, placements; // what patterned albedos read (Looks)
	DeviceBuffer boundaries;                      // rough glasses' boundary tables (Looks)
	// the shown frame (KDN_FRAME_DENOISE): the record of this frame (each
	// pixel's light and the first surface of its last sample), and the
	// G-buffer and the temporal state twice, this frame's and the one before
	DeviceBuffer frameLight, firstDistance, firstNormal, firstAlbedo, firstLeaf;
	DeviceBuffer gDistance[2], gNormal[2], gAlbedo[2], gLeaf[2];
	DeviceBuffer tColour[2], tMoment[2], tLength[2];
	// at a film factor above 1: the drawn frame the a-trous filter leaves,
	// and the upscale member's state twice (colour and depth a shown pixel)
	DeviceBuffer internal, upState[2];
	UpscaleScratch upscale;
	DeviceBuffer skyChart; // --use sampler=sky_map's chart of the frame
	// a physical sky's tables (air then haze, floats) and what they were
	// marched for (the sun's direction and the haze), with the frame, passed
	// and landing tables the constants take
	DeviceBuffer airTables;
	double airKey[4]   = { 0, 0, 0, -1 };
	AirFrame airFrame  = {};
	float airPassed[kAirColours] = {}, airLanding[kAirColours] = {};
	DeviceBuffer guideLobes, guideRecords; // the learned guide's, a lane's capacity each
	uint32_t capacity = 0;
	uint32_t lineRoom = 1; // the shadow queues' room, in capacities (1 + kOwnLines with own lines)
	int32_t width = 0, height = 0;
	double taken = 0;
	int current    = 0;     // which of the pairs the next denoised frame writes
	int shown      = -1;    // which of them the last denoised frame wrote; -1: none
	double lens[14] = {};   // the last denoised frame's lens
	int32_t stateWidth = 0, stateHeight = 0;
	uint32_t stateFactor = 1, statePhase = 0; // the film the temporal state was drawn at
	// the upscale state: which of upState the last frame wrote (-1: none),
	// its shown size, and upscale.cpp's moved flag and settling count
	int upShown = -1;
	int32_t upWidth = 0, upHeight = 0;
	bool upMoved = false;
	int upSettling = 0;
	bool last_denoised = false; // the last frame drawn was a denoised one
	bool surfaced() const { return last_denoised && shown >= 0; }
	std::vector<cudaEvent_t> events;
	cudaStream_t side[kLanes - 1] = {};   // the streams of the lanes after the first
	cudaEvent_t started           = nullptr; // the first lane's work before the chunks
	cudaEvent_t ended[kLanes - 1] = {};   // each other lane's end of the chunks
	cudaStream_t surfaceStream    = nullptr; // the surfaces pass
	cudaEvent_t surfacesDone      = nullptr; // its end
	kdn_frame_stats stats {};
};

void Context::releaseFrame() {
	if (frame == nullptr) return;
	FrameState& f = *frame;
	for (DeviceBuffer* b : { &f.pixel, &f.sample, &f.throughput, &f.radiance, &f.nanometres, &f.density, &f.drawn, &f.state, &f.from, &f.queuePaths[0], &f.queuePaths[1], &f.queueRays[0], &f.queueRays[1], &f.queueCarry[0], &f.queueCarry[1], &f.hits, &f.states, &f.counts, &f.shadowPaths[0], &f.shadowPaths[1], &f.shadowContribution[0], &f.shadowContribution[1], &f.held, &f.collided, &f.surfacePaths, &f.surfaceRays, &f.surfaceStates, &f.surfaceHits, &f.sums, &f.out, &f.materials, &f.patternSteps, &f.stops, &f.placements, &f.boundaries, &f.frameLight, &f.firstDistance, &f.firstNormal, &f.firstAlbedo, &f.firstLeaf, &f.gDistance[0], &f.gDistance[1], &f.gNormal[0], &f.gNormal[1], &f.gAlbedo[0], &f.gAlbedo[1], &f.gLeaf[0], &f.gLeaf[1], &f.tColour[0], &f.tColour[1], &f.tMoment[0], &f.tMoment[1], &f.tLength[0], &f.tLength[1], &f.internal, &f.upState[0], &f.upState[1], &f.upscale.samples, &f.upscale.axes, &f.skyChart, &f.airTables, &f.guideLobes, &f.guideRecords }) {
		if (b->ptr) cudaFree(b->ptr);
		b->ptr   = nullptr;
		b->bytes = 0;
	}
	for (cudaEvent_t e : f.events) cudaEventDestroy(e);
	if (f.started) cudaEventDestroy(f.started);
	for (cudaEvent_t e : f.ended) {
		if (e) cudaEventDestroy(e);
	}
	for (cudaStream_t side : f.side) {
		if (side == nullptr) continue;
		cudaStreamSynchronize(side);
		cudaStreamDestroy(side);
	}
	if (f.surfaceStream) {
		cudaStreamSynchronize(f.surfaceStream);
		cudaStreamDestroy(f.surfaceStream);
	}
	if (f.surfacesDone) cudaEventDestroy(f.surfacesDone);
	delete frame;
	frame = nullptr;
}

namespace {

struct V3 {
	double x, y, z;
};
V3 v3(const double* a) { return { a[0], a[1], a[2] }; }
V3 sub(V3 a, V3 b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
V3 scale(V3 a, double s) { return { a.x * s, a.y * s, a.z * s }; }
double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 cross(V3 a, V3 b) { return { a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x }; }
double length(V3 a) { return std::sqrt(dot(a, a)); }
V3 normalized(V3 a) { return scale(a, 1.0 / length(a)); }
void put(float* out, V3 a) {
	out[0] = float(a.x);
	out[1] = float(a.y);
	out[2] = float(a.z);
}

// plugins/transport/paths/light/light.cpp:78 lampOf
DeviceLamp lampOf(const kdn_light& l) {
	DeviceLamp d {};
	d.kind             = l.kind;
	const V3 along     = v3(l.along), across = v3(l.across);
	const V3 crossed   = cross(along, across);
	const double area  = length(crossed);
	const double al    = length(along), ac = length(across);
	put(d.at, v3(l.at));
	put(d.along, along);
	put(d.across, across);
	put(d.cross, crossed);
	if (area > 0) put(d.facing, normalized(crossed));
	if (al > 0 && ac > 0) {
		const V3 ex = scale(along, 1.0 / al), ey = scale(across, 1.0 / ac);
		put(d.ex, ex);
		put(d.ey, ey);
		put(d.raw, cross(ex, ey));
	}
	d.alongLength  = float(al);
	d.acrossLength = float(ac);
	d.square       = std::fabs(dot(along, across)) < 1e-9 * al * ac ? 1u : 0u;
	d.radius       = l.radius;
	const double pi = 3.14159265358979323846;
	double k        = 1.0;
	if (l.kind == 3) {
		d.area = float(area);
		k      = area > 0 ? 1.0 / area : 0.0;
	} else if (l.kind == 2) {
		d.area = float(4 * pi * double(l.radius) * double(l.radius));
		k      = l.radius > 0 ? 1.0 / (pi * double(l.radius) * double(l.radius)) : 0.0;
	} else if (l.kind == 4 || l.kind == 5) {
		// light.cpp:37 a far disc's radiance over its half angle's sine squared
		const double half = 0.5 * double(l.angle);
		const double sine = std::sin(half);
		k                 = sine != 0 ? 1.0 / (pi * sine * sine) : 0.0;
		// 1 - cos(half) as 2 sin^2(half / 2): exact for a small disc
		const double quarter = std::sin(0.5 * half);
		d.oneLess            = float(std::cos(half) < 1 ? 2 * quarter * quarter : 0.0);
		d.discRadius         = sine;
	}
	// light.cpp:86 lampOf: the direction normalised
	const V3 toward = v3(l.direction);
	if (length(toward) > 0) {
		put(d.direction, normalized(toward));
		const V3 unit = normalized(toward);
		d.disc[0] = unit.x, d.disc[1] = unit.y, d.disc[2] = unit.z;
	}
	for (int c = 0; c < 3; ++c) {
		d.radiance[c] = float(l.power[c] * k);
		d.power[c]    = float(l.power[c]);
	}
	return d;
}

DeviceMaterial materialOf(const kdn_material& m, const kdn_finish& f) {
	DeviceMaterial d {};
	d.kind = m.kind;
	for (int c = 0; c < 3; ++c) {
		d.albedo[c] = m.albedo[c];
		d.absorb[c] = m.absorb[c];
		d.glow[c]   = float(double(m.glow[c]) * double(m.strength));
	}
	d.roughness     = m.roughness;
	d.index         = float(f.index);
	d.dispersion    = m.kind == 3 ? m.dispersion : 0.0f;
	d.exact         = f.exact;
	d.sharp         = f.sharp;
	d.width         = float(f.width);
	d.facetShare    = float(f.facet_share);
	d.body          = float(f.body);
	d.escapeAverage = float(f.escape_average);
	d.coatFront     = float(f.coat_front);
	d.coatTwice     = float(f.coat_twice);
	d.coatRoom      = float(f.coat_room);
	d.losesMuch     = m.kind == 3 && !f.exact && f.loses_much ? 1u : 0u;
	d.filmThickness = m.kind == 0 ? 0.0f : float(f.film[0]);
	d.filmIndex     = float(f.film[1]);
	d.scatter       = m.kind == 3 && m.scatter > 0.0f ? m.scatter : 0.0f;
	d.lean          = m.lean;
	for (int k = 0; k < 32; ++k) d.escape[k] = float(f.escape[k]);
	return d;
}

// sdf/scene.h Albedo as the device reads it: each patterned material's
// program with its arguments folded in, its stops, and the leaves'
// placements where a pattern is read in a painted leaf's space.
struct PatternTables {
	std::vector<PatternStep> steps;
	std::vector<float> stops;
	std::vector<float> placements;
};

kdn_status patternTables(Context* ctx, const std::vector<kdn_material>& mats, std::vector<DeviceMaterial>& dm, PatternTables& t) {
	bool any = false;
	for (const kdn_material& m : mats) any = any || (m.flags_ & 1u) != 0;
	if (!any) return KDN_OK;
	const std::vector<kdn_pattern> patterns = ctx->block<kdn_pattern>("looks.patterns");
	if (patterns.size() != mats.size()) return ctx->fail(KDN_NOT_READY, "kdn_render: a patterned albedo needs the looks.patterns block, one pattern per material");
	const std::vector<kdn_step> steps     = ctx->block<kdn_step>("looks.pattern_steps");
	const std::vector<double> arguments   = ctx->block<double>("looks.pattern_arguments");
	const std::vector<float> stops        = ctx->block<float>("looks.stops");
	const std::vector<kdn_placement> placements = ctx->block<kdn_placement>("looks.placements");
	bool local = false;
	for (size_t k = 0; k < mats.size(); ++k) {
		if ((mats[k].flags_ & 1u) == 0) continue;
		const kdn_pattern& p   = patterns[k];
		const std::string what = "kdn_render: the pattern of material " + std::to_string(k);
		if (p.count == 0 || p.count > kPatternSteps) return ctx->fail(KDN_BAD_ARG, what + " has " + std::to_string(p.count) + " steps (1 to 64 are drawn)");
		if (uint64_t(p.first) + p.count > steps.size() || p.result >= p.count) return ctx->fail(KDN_BAD_ARG, what + " lies outside looks.pattern_steps");
		if (p.stop_count == 0 || (uint64_t(p.stop_first) + p.stop_count) * 3 > stops.size()) return ctx->fail(KDN_BAD_ARG, what + ": its stops lie outside looks.stops");
		if (uint64_t(p.argument_first) + p.argument_count > arguments.size()) return ctx->fail(KDN_BAD_ARG, what + ": its arguments lie outside looks.pattern_arguments");
		DeviceMaterial& d = dm[k];
		d.patternFirst    = uint32_t(t.steps.size());
		d.patternCount    = p.count;
		d.patternResult   = p.result;
		d.stopFirst       = uint32_t(t.stops.size() / 3);
		d.stopCount       = p.stop_count;
		d.world           = p.world ? 1u : 0u;
		local             = local || !p.world;
		for (uint32_t i = 0; i < p.count; ++i) {
			const kdn_step& s = steps[size_t(p.first) + i];
			if (s.opcode >= OpCount) return ctx->fail(KDN_BAD_ARG, what + ": step " + std::to_string(i) + " has an unknown opcode");
			if (s.a >= p.count || s.b >= p.count || s.c >= p.count) return ctx->fail(KDN_BAD_ARG, what + ": step " + std::to_string(i) + " reads past the program");
			PatternStep q {};
			q.op    = s.opcode;
			q.a     = uint8_t(s.a);
			q.b     = uint8_t(s.b);
			q.c     = uint8_t(s.c);
			q.value = float(s.value);
			if (s.opcode == OpArgument) {
				// sdf/program.cpp runStep: Argument reads arguments[a]
				if (s.a >= p.argument_count) return ctx->fail(KDN_BAD_ARG, what + ": step " + std::to_string(i) + " reads an argument past its own");
				q.op    = OpConstant;
				q.value = float(arguments[size_t(p.argument_first) + s.a]);
			}
			t.steps.push_back(q);
		}
		for (uint32_t i = 0; i < 3 * p.stop_count; ++i) t.stops.push_back(stops[3 * size_t(p.stop_first) + i]);
	}
	if (local) {
		const size_t leaves = ctx->block<uint32_t>("scene.leaves").size();
		if (placements.size() != leaves) return ctx->fail(KDN_NOT_READY, "kdn_render: a pattern read in a painted leaf's space needs the looks.placements block, one placement per leaf");
		t.placements.reserve(placements.size() * 12);
		for (const kdn_placement& pl : placements) {
			for (int r = 0; r < 3; ++r) {
				for (int c = 0; c < 3; ++c) t.placements.push_back(float(pl.linear[r][c]));
			}
			for (int c = 0; c < 3; ++c) t.placements.push_back(float(pl.origin[c]));
		}
	}
	return KDN_OK;
}

// Why a material cannot be drawn by these kernels, or null.
const char* unsupported(const kdn_material& m, const kdn_finish& f) {
	if (m.kind > 3) return "a medium (scattering body)";
	if (m.kind == 3 && m.refraction == 1.0f && m.dispersion == 0.0f && !(f.film[0] > 0)) return "a passable glass";
	return nullptr;
}

} // namespace

} // namespace kdn

using kdn::Context;
using kdn::FrameState;
using kdn::kLanes;

namespace {

// Device bytes one path of a chunk holds (the buffers ensureFrame sizes).
// pixel, sample, drawn, state, collided; throughput, radiance, nanometres, density,
// from; the two queues' path indices, rays and resume data (a path ray and
// a shadow line each); hits; hit states of a path ray and a line; the two
// line queues' path indices and contributions.
constexpr size_t kPathBytes = 5 * 4 + 5 * 16 + 2 * 4 + 2 * 2 * (sizeof(kdn_ray) + sizeof(uint2)) + sizeof(kdn_hit) + 2 * sizeof(kdn::HitState) + 2 * (4 + 16);
static_assert(kPathBytes == 420, "path bytes");
// ... and with own lines (--use sampler=each_lamp_first) kOwnLines more
// lines a path in each queue, their hit states and their held answers
constexpr size_t kOwnPathBytes = kdn::kOwnLines * (2 * (sizeof(kdn_ray) + sizeof(uint2)) + sizeof(kdn::HitState) + 2 * (4 + 16) + 16);

// A lane's device counts: [0], [1] the two ray queues, [2], [3] the two
// line queues, [4] zero; the first lane's [6]: the surfaces pass's queue.
constexpr int kCountsPerLane = 8;

// The paths the lanes' chunks hold together: the whole frame where the
// device has room for it (at most 2^28 paths, half the free memory), so
// every launch has a large share of the frame's rays to spread over the GPU
// and the slow rays of a launch hold back one thread each, not a small
// chunk's whole tail.
// with the learned guide, a path also holds its queue entry's lobes and its
// training records
constexpr size_t kGuidePathBytes = kdn::kGuideLobeFloats * sizeof(float) + kdn::kGuideDepth * sizeof(kdn::GuideRecord);

uint64_t chunkPaths(Context* ctx, uint64_t framePaths, bool ownLines) {
	size_t freeBytes = 0, totalBytes = 0;
	if (cudaMemGetInfo(&freeBytes, &totalBytes) != cudaSuccess) freeBytes = 0;
	const size_t pathBytes = kPathBytes + (ctx->guideFlags != 0 ? kGuidePathBytes : 0) + (ownLines ? kOwnPathBytes : 0);
	const uint64_t held = ctx->frame ? uint64_t(ctx->frame->capacity) * kLanes * (kPathBytes + (ctx->frame->lineRoom > 1 ? kOwnPathBytes : 0)) + ctx->frame->guideLobes.bytes +
	                                       ctx->frame->guideRecords.bytes
	                                 : 0;
	uint64_t room = (uint64_t(freeBytes) + held) / 2 / pathBytes;
	if (ctx->frameBudget > 0) room = std::min<uint64_t>(room, ctx->frameBudget / pathBytes);
	const uint64_t least = ctx->frameBudget > 0 ? uint64_t(1) << 16 : uint64_t(1) << 20;
	return std::min<uint64_t>(framePaths, std::min<uint64_t>(uint64_t(1) << 28, std::max<uint64_t>(room, least)));
}

// The path buffers for a chunk of `capacity` paths on each lane, with
// shadow queues of `lineRoom` capacities.
kdn_status ensureFrame(Context* ctx, uint32_t capacity, uint32_t lineRoom) {
	if (ctx->frame == nullptr) ctx->frame = new FrameState();
	FrameState& f = *ctx->frame;
	if (f.capacity >= capacity && f.lineRoom >= lineRoom) return KDN_OK;
	capacity       = std::max(capacity, f.capacity);
	lineRoom       = std::max(lineRoom, f.lineRoom);
	const size_t n = size_t(capacity) * kLanes;
	const size_t m = n * lineRoom;
	kdn_status s;
	struct Want {
		kdn::DeviceBuffer* b;
		size_t bytes;
	};
	const Want wants[] = {
		{ &f.pixel, n * 4 }, { &f.sample, n * 4 }, { &f.collided, n * 4 }, { &f.throughput, n * 16 }, { &f.radiance, n * 16 }, { &f.nanometres, n * 16 },
		{ &f.density, n * 16 }, { &f.drawn, n * 4 }, { &f.state, n * 4 }, { &f.from, n * 16 },
		// a lane's queue holds a bounce's path rays in [0, capacity) and the
		// shadow lines of the bounce before in [capacity, (1 + lineRoom)
		// capacity): one trace launch takes both
		{ &f.queuePaths[0], n * 4 }, { &f.queuePaths[1], n * 4 }, { &f.queueRays[0], (n + m) * sizeof(kdn_ray) }, { &f.queueRays[1], (n + m) * sizeof(kdn_ray) },
		{ &f.queueCarry[0], (n + m) * sizeof(uint2) }, { &f.queueCarry[1], (n + m) * sizeof(uint2) },
		{ &f.hits, n * sizeof(kdn_hit) }, { &f.states, (n + m) * sizeof(kdn::HitState) }, { &f.counts, kLanes * kCountsPerLane * sizeof(uint32_t) },
		{ &f.shadowPaths[0], m * 4 }, { &f.shadowPaths[1], m * 4 }, { &f.shadowContribution[0], m * 16 }, { &f.shadowContribution[1], m * 16 },
		{ &f.held, lineRoom > 1 ? n * kdn::kOwnLines * 16 : 0 },
	};
	for (const Want& w : wants) {
		if ((s = ctx->ensure(*w.b, w.bytes)) != KDN_OK) return s;
	}
	f.capacity = capacity;
	f.lineRoom = lineRoom;
	return KDN_OK;
}

kdn_status renderFrame(Context* ctx, const kdn_frame* fr, float* out, cudaStream_t stream, bool hostOut) {
	using namespace kdn;
	if (!ctx->built) return ctx->fail(KDN_NOT_READY, "kdn_render: no world built (kdn_build)");
	if (fr->width <= 0 || fr->height <= 0 || fr->samples <= 0 || fr->surfaces <= 0 || fr->surfaces > 255) return ctx->fail(KDN_BAD_ARG, "kdn_render: width, height, samples and surfaces (1..255) must be positive");
	if (uint64_t(fr->width) * uint64_t(fr->height) > (uint64_t(1) << 26)) return ctx->fail(KDN_BAD_ARG, "kdn_render: frame larger than 2^26 pixels");
	if (fr->collisions < 0 || fr->collisions > 4096) return ctx->fail(KDN_BAD_ARG, "kdn_render: collisions must be 0 (the default, 256) or 1..4096");
	// core/frame.cpp:296 fittedSplit: a split divides the samples into whole groups
	const uint32_t split = fr->split > 1 ? fr->split : 1u;
	if ((split != 1 && split != 2 && split != 4 && split != 8) || uint32_t(fr->samples) % split != 0 || fr->first % split != 0)
		return ctx->fail(KDN_BAD_ARG, "kdn_render: a split of 2, 4 or 8 needs whole groups of samples (samples and first multiples of it)");
	if (fr->samples > (1 << 20)) return ctx->fail(KDN_BAD_ARG, "kdn_render: more than 2^20 samples a pixel in one call (accumulate over calls)");
	// core/camera.h:65 FilmPlan: the frame is drawn at 1/factor of its size
	const uint32_t factor = fr->factor > 1 ? fr->factor : 1u;
	if (factor > 4) return ctx->fail(KDN_BAD_ARG, "kdn_render: the film factor must be 1 to 4");
	const bool upsampled = factor > 1 && (fr->flags & KDN_FRAME_UPSAMPLE);
	if (factor > 1) {
		if (!(fr->flags & KDN_FRAME_DENOISE) && !upsampled)
			return ctx->fail(KDN_BAD_ARG, "kdn_render: a film factor above 1 needs a reconstruction chain to the shown size (KDN_FRAME_DENOISE or KDN_FRAME_UPSAMPLE)");
		if (fr->width % int32_t(factor) != 0 || fr->height % int32_t(factor) != 0) return ctx->fail(KDN_BAD_ARG, "kdn_render: the size must be a multiple of the film factor");
		if (fr->phase >= factor * factor) return ctx->fail(KDN_BAD_ARG, "kdn_render: the phase must be below the film factor's square");
	}
	const int32_t drawnWidth = fr->width / int32_t(factor), drawnHeight = fr->height / int32_t(factor);
	if (!ctx->has("shot.camera") || !ctx->has("looks.materials")) return ctx->fail(KDN_NOT_READY, "kdn_render: the shot.camera and looks.materials blocks are needed");
	if (!ctx->check(cudaSetDevice(ctx->device), "cudaSetDevice")) return KDN_CUDA_ERROR;
	const kdn_camera cam                     = ctx->block<kdn_camera>("shot.camera")[0];
	const std::vector<kdn_light> lights      = ctx->block<kdn_light>("lighting.lights");
	const std::vector<kdn_material> mats     = ctx->block<kdn_material>("looks.materials");
	const std::vector<kdn_sky> skies         = ctx->block<kdn_sky>("lighting.sky");
	if (lights.size() > kMaxLamps) return ctx->fail(KDN_BAD_ARG, "kdn_render: more than 16 lights");
	if (mats.empty()) return ctx->fail(KDN_BAD_ARG, "kdn_render: no materials");
	if (!skies.empty() && skies[0].kind > 1) return ctx->fail(KDN_BAD_ARG, "kdn_render: a painted sky, which this build does not draw");
	const std::vector<kdn_finish> finishes = ctx->block<kdn_finish>("transport.finishes");
	if (finishes.size() != mats.size()) return ctx->fail(KDN_NOT_READY, "kdn_render: the transport.finishes block needs one finish per material");
	for (size_t k = 0; k < mats.size(); ++k) {
		const char* why = unsupported(mats[k], finishes[k]);
		if (why) return ctx->fail(KDN_BAD_ARG, "kdn_render: material " + std::to_string(k) + " is " + why + ", which this build does not draw");
	}
	const uint32_t pixels      = uint32_t(drawnWidth) * uint32_t(drawnHeight); // drawn
	const uint32_t shownPixels = uint32_t(fr->width) * uint32_t(fr->height);
	const uint32_t spp         = uint32_t(fr->samples);
	// a chunk a lane: the frame's paths halved where they fit, else as many as
	// the lanes' share of the room holds
	// with own lines a path holds up to 1 + kOwnLines lines at its first vertex
	const bool ownLines        = (fr->flags & KDN_FRAME_EACH_LAMP) != 0 && !lights.empty();
	const uint32_t lineRoom    = ownLines ? 1u + kOwnLines : 1u;
	const uint64_t want        = chunkPaths(ctx, uint64_t(pixels) * spp, ownLines) / kLanes;
	const uint32_t chunkPixels = uint32_t(std::max<uint64_t>(1, (want + spp - 1) / spp));
	const uint32_t capacity    = chunkPixels * spp;
	const uint32_t lineCapacity = capacity * lineRoom;
	kdn_status s = ensureFrame(ctx, capacity, lineRoom);
	if (s != KDN_OK) return s;
	FrameState& f = *ctx->frame;
	// the learned guide: draws from it once it is trained, records for training
	const bool guiding = ctx->guide != nullptr && (ctx->guideFlags & KDN_GUIDE_SAMPLE) && kdn_guide_ready(ctx->guide);
	const bool training = ctx->guide != nullptr && (ctx->guideFlags & KDN_GUIDE_TRAIN);
	if (guiding && (s = ctx->ensure(f.guideLobes, size_t(f.capacity) * kLanes * kGuideLobeFloats * sizeof(float))) != KDN_OK) return s;
	if (training && (s = ctx->ensure(f.guideRecords, size_t(f.capacity) * kLanes * kGuideDepth * sizeof(GuideRecord))) != KDN_OK) return s;
	// pixel sums: fresh unless accumulating onto a frame of the same size
	const bool fresh = !fr->accumulate || f.width != drawnWidth || f.height != drawnHeight || f.sums.ptr == nullptr;
	if ((s = ctx->ensure(f.sums, size_t(pixels) * 3 * sizeof(double))) != KDN_OK) return s;
	const bool denoised = (fr->flags & KDN_FRAME_DENOISE) != 0;
	if (denoised) {
		const size_t px = pixels;
		const struct {
			DeviceBuffer* b;
			size_t bytes;
		} wants[] = { { &f.frameLight, px * 12 }, { &f.firstDistance, px * 2 }, { &f.firstNormal, px * 6 }, { &f.firstAlbedo, px * 6 }, { &f.firstLeaf, px * 4 },
			          { &f.gDistance[0], px * 2 }, { &f.gDistance[1], px * 2 }, { &f.gNormal[0], px * 6 }, { &f.gNormal[1], px * 6 },
			          { &f.gAlbedo[0], px * 6 }, { &f.gAlbedo[1], px * 6 }, { &f.gLeaf[0], px * 4 }, { &f.gLeaf[1], px * 4 },
			          { &f.tColour[0], px * 12 }, { &f.tColour[1], px * 12 }, { &f.tMoment[0], px * 4 }, { &f.tMoment[1], px * 4 },
			          { &f.tLength[0], px * 4 }, { &f.tLength[1], px * 4 } };
		for (const auto& w : wants) {
			if ((s = ctx->ensure(*w.b, w.bytes)) != KDN_OK) return s;
		}
		if (factor > 1 && !upsampled) {
			for (DeviceBuffer* b : { &f.upState[0], &f.upState[1] }) {
				if ((s = ctx->ensure(*b, size_t(shownPixels) * 16)) != KDN_OK) return s;
			}
		}
	}
	if (factor > 1 && (s = ctx->ensure(f.internal, size_t(pixels) * 12)) != KDN_OK) return s;
	if (fresh) {
		if (!ctx->check(cudaMemsetAsync(f.sums.ptr, 0, size_t(pixels) * 3 * sizeof(double), stream), "clear sums")) return KDN_CUDA_ERROR;
		f.taken = 0;
	}
	const int cur = f.current; // the G-buffer and state pair this frame writes
	f.width  = drawnWidth;
	f.height = drawnHeight;
	// constants
	FrameConstants c {};
	const V3 eye = v3(cam.eye), target = v3(cam.target), up = v3(cam.up);
	const V3 forward = normalized(sub(target, eye));
	const V3 right   = normalized(cross(forward, up));
	put(c.eye, eye);
	put(c.forward, forward);
	put(c.right, right);
	put(c.up, cross(right, forward));
	c.reach         = float(std::tan(cam.fov / 2));
	c.aperture      = float(std::max(cam.aperture, 0.0));
	c.focus         = float(cam.focus > 0 ? cam.focus : length(sub(target, eye)));
	c.aspect        = float(double(drawnWidth) / double(drawnHeight));
	c.width         = drawnWidth;
	c.height        = drawnHeight;
	c.factor        = factor;
	c.phase         = factor > 1 ? fr->phase : 0u;
	filmCentreOf(factor, c.phase, c.centre);
	c.sobol         = nullptr;
	if (fr->flags & KDN_FRAME_SOBOL) {
		if (ctx->sobolTables.ptr == nullptr) {
			std::vector<uint32_t> tables(kSobolTableWords);
			buildSobolTables(tables.data());
			if ((s = ctx->upload(ctx->sobolTables, tables.data(), tables.size() * sizeof(uint32_t))) != KDN_OK) return s;
			if (!ctx->check(cudaStreamSynchronize(ctx->stream), "sobol tables")) return KDN_CUDA_ERROR;
		}
		c.sobol = static_cast<const uint32_t*>(ctx->sobolTables.ptr);
	}
	// the first sun (sdf/scene.cpp:306 firstSun)
	uint32_t firstSun = uint32_t(lights.size());
	for (size_t k = 0; k < lights.size(); ++k) {
		if (lights[k].kind == 4) {
			firstSun = uint32_t(k);
			break;
		}
	}
	const bool hasSun = firstSun < lights.size();
	// a physical sky lit by a sun (atmosphere.cpp:308 atmosphereOf): its
	// tables marched once a sun direction and haze
	c.airTables = nullptr;
	c.sunLamp   = 0xFFFFFFFFu;
	if (!skies.empty() && skies[0].kind == 1 && hasSun) {
		const kdn_light& sun = lights[firstSun];
		const double key[4]  = { sun.direction[0], sun.direction[1], sun.direction[2], double(skies[0].haze) };
		if (f.airTables.ptr == nullptr || !std::equal(key, key + 4, f.airKey)) {
			std::vector<double> air(static_cast<size_t>(kAirTable)), haze(static_cast<size_t>(kAirTable)), passed(static_cast<size_t>(kAirColours)),
			    landing(static_cast<size_t>(kAirColours));
			buildAtmosphere(sun.direction, double(skies[0].haze), f.airFrame, air.data(), haze.data(), passed.data(), landing.data());
			std::vector<float> tables(size_t(2) * kAirTable);
			for (int k = 0; k < kAirTable; ++k) {
				tables[size_t(k)]             = float(air[size_t(k)]);
				tables[size_t(kAirTable + k)] = float(haze[size_t(k)]);
			}
			for (int k = 0; k < kAirColours; ++k) {
				f.airPassed[k]  = float(passed[size_t(k)]);
				f.airLanding[k] = float(landing[size_t(k)]);
			}
			if ((s = ctx->upload(f.airTables, tables.data(), tables.size() * sizeof(float))) != KDN_OK) return s;
			if (!ctx->check(cudaStreamSynchronize(ctx->stream), "air tables")) return KDN_CUDA_ERROR;
			std::copy(key, key + 4, f.airKey);
		}
		c.airTables = static_cast<const float*>(f.airTables.ptr);
		for (int a = 0; a < 3; ++a) {
			c.airUp[a]     = float(f.airFrame.up[a]);
			c.airSun[a]    = float(f.airFrame.sun[a]);
			c.airLevel[a]  = float(f.airFrame.level[a]);
			c.airAside[a]  = float(f.airFrame.aside[a]);
			c.sunlight[a]  = float(sun.power[a]);
			c.airGround[a] = float(skies[0].ground[a]);
		}
		std::copy(f.airPassed, f.airPassed + kAirColours, c.airPassed);
		std::copy(f.airLanding, f.airLanding + kAirColours, c.airLanding);
		c.sunLamp = firstSun;
	}
	// sky_layers.cpp:164 skyGlows: a glow given and a sun
	c.glows = 0;
	if (!skies.empty() && hasSun) {
		const double strength = skies[0].strength;
		for (int a = 0; a < 3; ++a) c.glow[a] = float(skies[0].glow[a] * strength);
		if (c.glow[0] > 0.0f || c.glow[1] > 0.0f || c.glow[2] > 0.0f) {
			const V3 sun   = normalized(v3(lights[firstSun].direction));
			c.glows        = 1;
			c.glowSpread   = float(skies[0].spread);
			c.sunElevation = float(std::asin(std::clamp(sun.z, -1.0, 1.0)));
		}
	}
	// sky_layers.cpp:240 starlight, :264 starNight: the stars fade in as the
	// first sun sinks from 2 to 12 degrees below the horizon
	c.stars = 0;
	if (!skies.empty() && skies[0].stars) {
		c.stars        = 1;
		c.starCount    = skies[0].star_count;
		c.starStrength = skies[0].star_strength;
		c.starAngle    = skies[0].star_angle;
		double night   = 1.0;
		if (hasSun) {
			const double pi = 3.14159265358979323846;
			const V3 sun    = normalized(v3(lights[firstSun].direction));
			const double e  = std::asin(std::clamp(sun.z, -1.0, 1.0));
			double t        = std::clamp((e - (-12.0 * pi / 180.0)) / ((-2.0 * pi / 180.0) - (-12.0 * pi / 180.0)), 0.0, 1.0);
			night           = 1.0 - t * t * (3.0 - 2.0 * t);
		}
		c.starNight = float(night);
	}
	if ((fr->flags & KDN_FRAME_SKY_MAP) && (c.airTables != nullptr || c.glows || c.stars)) return ctx->fail(KDN_BAD_ARG, "kdn_render: the sky map charts a gradient sky without a glow or stars only");
	c.skyChart = nullptr;
	if (fr->flags & KDN_FRAME_SKY_MAP) {
		// plugins/sampler/sky_map/plugin.cpp:15 chartedSkyPrepared: charted
		// each frame from the sky, the lamps and the region's middle
		SkyGradient g {};
		if (!skies.empty()) {
			for (int k = 0; k < 3; ++k) {
				g.zenith[k]  = skies[0].zenith[k];
				g.horizon[k] = skies[0].horizon[k];
				g.ground[k]  = skies[0].ground[k];
			}
		}
		std::vector<ChartLamp> chartLamps(lights.size());
		for (size_t k = 0; k < lights.size(); ++k) {
			chartLamps[k].kind = lights[k].kind;
			for (int a = 0; a < 3; ++a) {
				chartLamps[k].at[a]     = lights[k].at[a];
				chartLamps[k].along[a]  = lights[k].along[a];
				chartLamps[k].across[a] = lights[k].across[a];
				chartLamps[k].power[a]  = lights[k].power[a];
			}
		}
		const std::vector<kdn_region> region = ctx->block<kdn_region>("geometry.region");
		double middle[3] = { 0, 0, 0 };
		if (!region.empty()) {
			for (int a = 0; a < 3; ++a) middle[a] = region[0].lower[a] + 0.5 * region[0].size[a];
		}
		std::vector<double> chart(kChartDoubles);
		if (buildSkyChart(g, chartLamps.data(), uint32_t(chartLamps.size()), middle, chart.data())) {
			if ((s = ctx->upload(f.skyChart, chart.data(), chart.size() * sizeof(double))) != KDN_OK) return s;
			if (!ctx->check(cudaStreamSynchronize(ctx->stream), "sky chart")) return KDN_CUDA_ERROR;
			c.skyChart = static_cast<const double*>(f.skyChart.ptr);
		}
	}
	c.eachLamp      = ownLines ? 1u : 0u;
	c.collisionCap  = fr->collisions > 0 ? uint32_t(fr->collisions) : 256u;
	c.split         = split;
	c.seedMix       = mixedBits(uint64_t(int64_t(fr->seed)));
	c.surfaces      = fr->surfaces;
	c.spp           = spp;
	c.firstSample   = fr->first;
	c.lampCount     = uint32_t(lights.size());
	c.materialCount = uint32_t(mats.size());
	for (const kdn_material& m : mats) {
		if (m.kind == 3 && (m.absorb[0] > 0 || m.absorb[1] > 0 || m.absorb[2] > 0)) c.absorbs = 1;
	}
	for (size_t k = 0; k < lights.size(); ++k) c.lamps[k] = lampOf(lights[k]);
	for (size_t k = 0; k < lights.size(); ++k) {
		if (lights[k].kind == 4) {
			for (int a = 0; a < 3; ++a) c.sunDirection[a] = c.lamps[k].disc[a];
			c.hasSun = length(v3(lights[k].direction)) > 0 ? 1u : 0u;
			break;
		}
	}
	if (!skies.empty()) {
		put(c.zenith, v3(skies[0].zenith));
		put(c.horizon, v3(skies[0].horizon));
		put(c.ground, v3(skies[0].ground));
	}
	buildSpectralTables(c.spectral);
	std::vector<DeviceMaterial> dm;
	for (size_t k = 0; k < mats.size(); ++k) {
		dm.push_back(materialOf(mats[k], finishes[k]));
		if (dm.back().filmThickness > 0.0f) c.films = 1;
		if (dm.back().scatter > 0.0f) c.scatters = 1;
	}
	c.extras = c.scatters || c.airTables != nullptr || c.glows || c.stars || c.skyChart != nullptr || c.eachLamp || c.split > 1 ? 1u : 0u;
	for (const kdn_light& l : lights) c.extras |= l.kind != 2 && l.kind != 3 ? 1u : 0u;
	// material/energy.h Boundary of each rough glass that loses much
	std::vector<float> boundaryTables;
	{
		const std::vector<kdn_boundary> boundaries = ctx->block<kdn_boundary>("transport.boundaries");
		for (size_t k = 0; k < dm.size(); ++k) {
			if (!dm[k].losesMuch) continue;
			if (boundaries.size() != mats.size()) return ctx->fail(KDN_NOT_READY, "kdn_render: a rough glass that loses much needs the transport.boundaries block, one boundary per material");
			const kdn_boundary& b = boundaries[k];
			dm[k].boundaryFirst   = uint32_t(boundaryTables.size() / kBoundaryFloats);
			for (int r = 0; r < kBoundaryRatios; ++r) {
				for (int v = 0; v < kBoundaryViews; ++v) boundaryTables.push_back(float(b.rarer[r][v]));
			}
			for (int r = 0; r < kBoundaryRatios; ++r) {
				for (int v = 0; v < kBoundaryViews; ++v) boundaryTables.push_back(float(b.denser[r][v]));
			}
			for (int r = 0; r < kBoundaryRatios; ++r) boundaryTables.push_back(float(b.rarer_average[r]));
			for (int r = 0; r < kBoundaryRatios; ++r) boundaryTables.push_back(float(b.denser_average[r]));
			for (int r = 0; r < kBoundaryRatios; ++r) boundaryTables.push_back(float(b.rarer_through[r]));
		}
	}
	if ((s = ctx->upload(f.boundaries, boundaryTables.data(), boundaryTables.size() * sizeof(float))) != KDN_OK) return s;
	PatternTables tables;
	if ((s = patternTables(ctx, mats, dm, tables)) != KDN_OK) return s;
	if ((s = ctx->upload(f.materials, dm.data(), dm.size() * sizeof(DeviceMaterial))) != KDN_OK) return s;
	if ((s = ctx->upload(f.patternSteps, tables.steps.data(), tables.steps.size() * sizeof(PatternStep))) != KDN_OK) return s;
	if ((s = ctx->upload(f.stops, tables.stops.data(), tables.stops.size() * sizeof(float))) != KDN_OK) return s;
	if ((s = ctx->upload(f.placements, tables.placements.data(), tables.placements.size() * sizeof(float))) != KDN_OK) return s;
	Looks looks {};
	looks.materials      = static_cast<const DeviceMaterial*>(f.materials.ptr);
	looks.leafMaterial   = static_cast<const uint32_t*>(ctx->leafMaterial.ptr);
	looks.leafCount      = uint32_t(ctx->leafMaterial.bytes / 4);
	looks.placementCount = uint32_t(tables.placements.size() / 12);
	looks.placements     = static_cast<const float*>(f.placements.ptr);
	looks.patternSteps   = static_cast<const PatternStep*>(f.patternSteps.ptr);
	looks.stops          = static_cast<const float*>(f.stops.ptr);
	looks.boundaries     = static_cast<const float*>(f.boundaries.ptr);
	looks.materialCount  = uint32_t(dm.size());
	if ((s = ctx->ensure(ctx->counters, 8 * sizeof(unsigned long long))) != KDN_OK) return s;
	if (!ctx->check(cudaMemsetAsync(ctx->counters.ptr, 0, 8 * sizeof(unsigned long long), stream), "clear counters")) return KDN_CUDA_ERROR;

	PathBuffers P;
	P.pixel      = static_cast<uint32_t*>(f.pixel.ptr);
	P.sample     = static_cast<uint32_t*>(f.sample.ptr);
	P.throughput = static_cast<float4*>(f.throughput.ptr);
	P.radiance   = static_cast<float4*>(f.radiance.ptr);
	P.nanometres = static_cast<float4*>(f.nanometres.ptr);
	P.density    = static_cast<float4*>(f.density.ptr);
	P.drawn      = static_cast<float*>(f.drawn.ptr);
	P.state      = static_cast<uint32_t*>(f.state.ptr);
	P.from       = static_cast<float4*>(f.from.ptr);
	P.held       = ownLines ? static_cast<float4*>(f.held.ptr) : nullptr;
	P.collided   = c.scatters ? static_cast<uint32_t*>(f.collided.ptr) : nullptr;
	// Lanes: the frame's chunks go round kLanes streams, each lane with its own
	// share of the path buffers, queues and counters, so one chunk's work
	// fills the SMs another chunk's launch leaves idle in its tail (the
	// slowest rays of a trace launch).
	uint32_t* counts = static_cast<uint32_t*>(f.counts.ptr); // kCountsPerLane a lane
	if (!ctx->check(cudaMemsetAsync(counts, 0, kLanes * kCountsPerLane * sizeof(uint32_t), stream), "clear counts")) return KDN_CUDA_ERROR;
	cudaStream_t lanes[kLanes] = { stream };
	for (int l = 1; l < kLanes; ++l) {
		if (f.side[l - 1] == nullptr && !ctx->check(cudaStreamCreateWithPriority(&f.side[l - 1], cudaStreamNonBlocking, ctx->priority), "cudaStreamCreate")) return KDN_CUDA_ERROR;
		if (f.ended[l - 1] == nullptr && !ctx->check(cudaEventCreateWithFlags(&f.ended[l - 1], cudaEventDisableTiming), "cudaEventCreate")) return KDN_CUDA_ERROR;
		lanes[l] = f.side[l - 1];
	}
	if (f.started == nullptr && !ctx->check(cudaEventCreateWithFlags(&f.started, cudaEventDisableTiming), "cudaEventCreate")) return KDN_CUDA_ERROR;
	struct Lane {
		PathBuffers P;
		QueueBuffers Q[2];   // a bounce's path rays in [0, capacity) of rays and carry
		ShadowBuffers S[2];  // the shadow lines traced with Q[k], in [capacity, capacity + lineCapacity)
		HitState* states;
		kdn_hit* hits;
		uint32_t* none;
		uint32_t* fetch;
		float* lobes;
		GuideRecord* records;
	};
	Lane lane[kLanes];
	for (int l = 0; l < kLanes; ++l) {
		const size_t base = size_t(l) * capacity;
		Lane& L           = lane[l];
		uint32_t* lc      = counts + kCountsPerLane * l;
		L.P               = P;
		L.P.pixel         = P.pixel + base;
		L.P.sample        = P.sample + base;
		L.P.throughput    = P.throughput + base;
		L.P.radiance      = P.radiance + base;
		L.P.nanometres    = P.nanometres + base;
		L.P.density       = P.density + base;
		L.P.drawn         = P.drawn + base;
		L.P.state         = P.state + base;
		L.P.from          = P.from + base;
		L.P.held          = ownLines ? P.held + base * kOwnLines : nullptr;
		L.P.collided      = P.collided ? P.collided + base : nullptr;
		// a queue's path rays and hit states in [0, capacity), the shadow lines
		// traced with them in [capacity, capacity + lineCapacity): one trace
		// launch takes both
		L.states = static_cast<HitState*>(f.states.ptr) + (1 + lineRoom) * base;
		L.hits   = static_cast<kdn_hit*>(f.hits.ptr) + base;
		for (int k = 0; k < 2; ++k) {
			L.Q[k].paths        = static_cast<uint32_t*>(f.queuePaths[k].ptr) + base;
			L.Q[k].rays         = static_cast<kdn_ray*>(f.queueRays[k].ptr) + (1 + lineRoom) * base;
			L.Q[k].carry        = static_cast<uint2*>(f.queueCarry[k].ptr) + (1 + lineRoom) * base;
			L.Q[k].count        = lc + k;
			L.S[k].rays         = L.Q[k].rays + capacity;
			L.S[k].carry        = L.Q[k].carry + capacity;
			L.S[k].paths        = static_cast<uint32_t*>(f.shadowPaths[k].ptr) + lineRoom * base;
			L.S[k].contribution = static_cast<float4*>(f.shadowContribution[k].ptr) + lineRoom * base;
			L.S[k].count        = lc + 2 + k;
			L.S[k].states       = L.states + capacity;
		}
		L.none    = lc + 4;
		L.fetch   = static_cast<uint32_t*>(ctx->fetch.ptr) + l;
		L.lobes   = guiding ? static_cast<float*>(f.guideLobes.ptr) + base * kGuideLobeFloats : nullptr;
		L.records = training ? static_cast<GuideRecord*>(f.guideRecords.ptr) + base * kGuideDepth : nullptr;
	}

	// Rounds a chunk: surfaces + 1 (+ the collision cap where a body
	// scatters; each traces the bounce's path rays and
	// the lines of the bounce before; the last, the last lines).  With a
	// march budget a path waits a round each time its ray or its line is
	// carried, at most once a round, so surfaces + 1 more rounds without a
	// budget finish every path that waited.
	const bool budgeted     = ctx->marchBudget > 0 && ctx->marchBudget < kMarchSteps && !guiding;
	// with scattering bodies a path also stands on up to collisionCap
	// collisions, a round each
	const int mainRounds    = fr->surfaces + 1 + (c.scatters ? int(c.collisionCap) : 0);
	const int rounds        = budgeted ? 2 * mainRounds : mainRounds;

	// timing: one event pair around the frame, one around each trace launch
	const uint32_t chunks = (pixels + chunkPixels - 1) / chunkPixels;
	const size_t traceEvents = size_t(chunks) * size_t(rounds) * 2;
	const size_t needEvents  = 2 + traceEvents;
	while (f.events.size() < needEvents) {
		cudaEvent_t e;
		if (!ctx->check(cudaEventCreate(&e), "cudaEventCreate")) return KDN_CUDA_ERROR;
		f.events.push_back(e);
	}
	size_t ev = 2;
	if (!ctx->check(cudaEventRecord(f.events[0], stream), "event")) return KDN_CUDA_ERROR;
	uint32_t launches = 0;
	// the other lanes (and the surfaces pass) start after what the first holds so far
	if (!ctx->check(cudaEventRecord(f.started, stream), "event")) return KDN_CUDA_ERROR;
	for (int l = 1; l < kLanes; ++l) {
		if (!ctx->check(cudaStreamWaitEvent(lanes[l], f.started, 0), "stream wait")) return KDN_CUDA_ERROR;
	}
	if (denoised) {
		// core/surfaces.cpp:133 tracedSurfaces: the denoiser's features, on a
		// stream of its own beside the chunks, its own queue and hits
		if (f.surfaceStream == nullptr && !ctx->check(cudaStreamCreateWithPriority(&f.surfaceStream, cudaStreamNonBlocking, ctx->priority), "cudaStreamCreate")) return KDN_CUDA_ERROR;
		if (f.surfacesDone == nullptr && !ctx->check(cudaEventCreateWithFlags(&f.surfacesDone, cudaEventDisableTiming), "cudaEventCreate")) return KDN_CUDA_ERROR;
		const uint32_t sc = std::min<uint32_t>(pixels, 1u << 22);
		const struct {
			DeviceBuffer* b;
			size_t bytes;
		} wants[] = { { &f.surfacePaths, size_t(sc) * 4 }, { &f.surfaceRays, size_t(sc) * sizeof(kdn_ray) }, { &f.surfaceStates, size_t(sc) * sizeof(HitState) },
			          { &f.surfaceHits, size_t(sc) * sizeof(kdn_hit) } };
		for (const auto& w : wants) {
			if ((s = ctx->ensure(*w.b, w.bytes)) != KDN_OK) return s;
		}
		const cudaStream_t on = f.surfaceStream;
		if (!ctx->check(cudaStreamWaitEvent(on, f.started, 0), "stream wait")) return KDN_CUDA_ERROR;
		QueueBuffers sq;
		sq.paths = static_cast<uint32_t*>(f.surfacePaths.ptr);
		sq.rays  = static_cast<kdn_ray*>(f.surfaceRays.ptr);
		sq.count = counts + kCountsPerLane * 0 + 6; // lane 0's spare count
		sq.carry = nullptr;
		for (uint32_t first = 0; first < pixels; first += sc) {
			const uint32_t n = std::min(sc, pixels - first);
			if (!ctx->check(launchSurfaceRays(c, sq, first, n, on, ctx->smCount), "surface rays kernel")) return KDN_CUDA_ERROR;
			TraceArgs t;
			t.world          = ctx->world;
			t.rays           = sq.rays;
			t.n              = n;
			t.states         = static_cast<HitState*>(f.surfaceStates.ptr);
			t.objectMaterial = static_cast<const uint32_t*>(ctx->objectMaterial.ptr);
			t.maxSteps       = kMarchSteps;
			t.counters       = nullptr;
			t.count          = sq.count;
			t.fetch          = static_cast<uint32_t*>(ctx->fetch.ptr) + kLanes;
			if (!ctx->check(launchTrace(t, on, ctx->smCount), "surface trace kernel")) return KDN_CUDA_ERROR;
			HitArgs h;
			h.world  = ctx->world;
			h.rays   = sq.rays;
			h.states = t.states;
			h.n      = n;
			h.hits   = static_cast<kdn_hit*>(f.surfaceHits.ptr);
			h.count  = sq.count;
			if (!ctx->check(launchHits(h, on, ctx->smCount), "surface hit kernel")) return KDN_CUDA_ERROR;
			SurfaceArgs g;
			g.rays         = sq;
			g.hits         = h.hits;
			g.looks        = looks;
			g.distance     = static_cast<uint16_t*>(f.gDistance[cur].ptr);
			g.normal       = static_cast<uint16_t*>(f.gNormal[cur].ptr);
			g.albedo       = static_cast<uint16_t*>(f.gAlbedo[cur].ptr);
			g.leaf         = static_cast<uint32_t*>(f.gLeaf[cur].ptr);
			if (!ctx->check(launchSurfaces(g, n, on, ctx->smCount), "surfaces kernel")) return KDN_CUDA_ERROR;
			launches += 4;
		}
		if (!ctx->check(cudaEventRecord(f.surfacesDone, on), "event")) return KDN_CUDA_ERROR;
	}
	uint32_t chunkIndex = 0;
	for (uint32_t first = 0; first < pixels; first += chunkPixels, ++chunkIndex) {
		const int l              = int(chunkIndex % kLanes);
		const Lane& L            = lane[l];
		const cudaStream_t on    = lanes[l];
		const uint32_t chunk     = std::min(chunkPixels, pixels - first);
		const uint32_t n         = chunk * spp;
		const PathBuffers& LP    = L.P;
		if (training && !ctx->check(cudaMemsetAsync(L.records, 0xFF, size_t(n) * kGuideDepth * sizeof(GuideRecord), on), "clear guide records")) return KDN_CUDA_ERROR;
		if (!ctx->check(launchCamera(c, LP, L.Q[0], first, n, on, ctx->smCount), "camera kernel")) return KDN_CUDA_ERROR;
		++launches;
		if (!ctx->check(cudaMemsetAsync(L.S[0].count, 0, 4, on), "clear lines")) return KDN_CUDA_ERROR;
		int q = 0;
		// each round traces the bounce's path rays and the bounce before's
		// shadow lines in one launch; a last round traces the last lines alone
		for (int round = 0; round < rounds; ++round) {
			const bool last = round == rounds - 1;
			const int nxt   = 1 - q;
			TraceArgs t;
			t.world          = ctx->world;
			t.rays           = L.Q[q].rays;
			t.n              = n;
			t.states         = L.states;
			t.objectMaterial = static_cast<const uint32_t*>(ctx->objectMaterial.ptr);
			t.maxSteps       = kMarchSteps;
			t.counters       = static_cast<unsigned long long*>(ctx->counters.ptr);
			t.count          = last ? L.none : L.Q[q].count;
			t.fetch          = L.fetch;
			t.secondCount    = L.S[q].count;
			t.second         = capacity;
			t.carry          = L.Q[q].carry;
			t.budget         = budgeted && round < mainRounds ? ctx->marchBudget : 0u;
			t.left           = last ? L.Q[q].count : nullptr;
			cudaEventRecord(f.events[ev++], on);
			if (!ctx->check(launchTrace(t, on, ctx->smCount), "trace kernel")) return KDN_CUDA_ERROR;
			cudaEventRecord(f.events[ev++], on);
			++launches;
			if (!last) {
				HitArgs h;
				h.world  = ctx->world;
				h.rays   = L.Q[q].rays;
				h.states = L.states;
				h.n      = n;
				h.hits   = L.hits;
				h.count  = L.Q[q].count;
				if (!ctx->check(launchHits(h, on, ctx->smCount), "hit kernel")) return KDN_CUDA_ERROR;
				++launches;
				if (guiding && round < kGuideDepth) {
					GuideQueue gq;
					gq.hits          = L.hits;
					gq.rays          = L.Q[q].rays;
					gq.count         = L.Q[q].count;
					gq.looks         = looks;
					gq.materialCount = looks.materialCount;
					gq.lobes         = L.lobes;
					if (!ctx->check(guideQueryQueue(ctx->guide, gq, n, on, ctx->smCount), "guide query kernel")) return KDN_CUDA_ERROR;
					++launches;
				}
			}
			if (!ctx->check(cudaMemsetAsync(L.S[nxt].count, 0, 4, on), "clear lines")) return KDN_CUDA_ERROR;
			if (round > 0) {
				// the bounce before's lines that reached their lamps; lines still
				// marching go on with the next round's
				if (!ctx->check(launchLines(LP, L.S[q], L.S[nxt], lineCapacity, on, ctx->smCount), "lines kernel")) return KDN_CUDA_ERROR;
				++launches;
			}
			if (last) break;
			if (!ctx->check(cudaMemsetAsync(L.Q[nxt].count, 0, 4, on), "clear queue")) return KDN_CUDA_ERROR;
			ShadeArgs a;
			a.paths         = LP;
			a.in            = L.Q[q];
			a.out           = L.Q[nxt];
			a.shadow        = L.S[nxt];
			a.hits          = L.hits;
			a.states        = L.states;
			a.looks         = looks;
			a.capacity      = capacity;
			a.lineCapacity  = lineCapacity;
			a.error         = nullptr;
			a.firstDistance = denoised ? static_cast<uint16_t*>(f.firstDistance.ptr) : nullptr;
			a.firstNormal   = denoised ? static_cast<uint16_t*>(f.firstNormal.ptr) : nullptr;
			a.firstAlbedo   = denoised ? static_cast<uint16_t*>(f.firstAlbedo.ptr) : nullptr;
			a.firstLeaf     = denoised ? static_cast<uint32_t*>(f.firstLeaf.ptr) : nullptr;
			a.lobes         = (guiding && round < kGuideDepth) ? L.lobes : nullptr;
			a.guideShare    = ctx->guideShare;
			a.records       = L.records;
			if (!ctx->check(launchShade(c, a, on, ctx->smCount), "shade kernel")) return KDN_CUDA_ERROR;
			++launches;
			q = nxt;
		}
		if (!ctx->check(launchFold(c, LP, first, chunk, spp, static_cast<double*>(f.sums.ptr), denoised ? static_cast<float*>(f.frameLight.ptr) : nullptr, on, ctx->smCount), "fold kernel")) return KDN_CUDA_ERROR;
		++launches;
		if (training) {
			if (!ctx->check(guideGather(ctx->guide, L.records, LP.radiance, n, uint64_t(pixels) * spp, uint32_t(fr->seed) * 0x85EBCA6Bu + first, on, ctx->smCount), "guide gather kernel")) return KDN_CUDA_ERROR;
			++launches;
		}
	}
	// the first lane goes on once the others and the surfaces pass are done
	for (int l = 1; l < kLanes; ++l) {
		if (!ctx->check(cudaEventRecord(f.ended[l - 1], lanes[l]), "event") || !ctx->check(cudaStreamWaitEvent(stream, f.ended[l - 1], 0), "stream wait")) return KDN_CUDA_ERROR;
	}
	if (denoised && !ctx->check(cudaStreamWaitEvent(stream, f.surfacesDone, 0), "stream wait")) return KDN_CUDA_ERROR;
	if (training && (s = guideTrainGathered(ctx->guide, stream)) != KDN_OK) return ctx->fail(s, std::string("kdn_render: guide training: ") + kdn_guide_last_error());
	f.taken += double(spp);
	f.last_denoised = denoised;
	if (!denoised) { // a frame without the shown chain drops the temporal and upscale histories
		f.shown   = -1;
		f.upShown = -1;
	}

	float* image = out;
	if (hostOut) {
		if ((s = ctx->ensure(f.out, size_t(shownPixels) * 3 * sizeof(float))) != KDN_OK) return s;
		image = static_cast<float*>(f.out.ptr);
	}
	// the drawn frame the chain's members before a change of size leave:
	// the shown frame itself at a film factor of 1
	float* drawnImage = factor > 1 ? static_cast<float*>(f.internal.ptr) : image;
	if (!denoised) {
		// reconstruction/mean (then upsample at a film factor above 1)
		if (!ctx->check(launchMeans(static_cast<const double*>(f.sums.ptr), pixels, f.taken, drawnImage, stream, ctx->smCount), "means kernel")) return KDN_CUDA_ERROR;
		++launches;
		if (factor > 1) {
			if (!ctx->check(launchUpsample(fr->width, fr->height, int(factor), drawnImage, image, stream, ctx->smCount), "upsample kernel")) return KDN_CUDA_ERROR;
			++launches;
		}
	} else {
		// the shown frame (core/frame.cpp shownSurfaces, then the reconstruction
		// chain temporal + a-trous): this frame's record and G-buffer through
		// the temporal member (its history kept where the frame before was of
		// this size and not restarted; moved where the lens changed), then its
		// state through the a-trous filter, demodulated
		// (plugins/reconstruction/atrous/atrous.cpp:513 denoisedFrame)
		const V3 lensUp = cross(right, forward);
		double lens[14];
		const V3* parts[4] = { &eye, &forward, &right, &lensUp };
		for (int k = 0; k < 4; ++k) {
			lens[3 * k]     = parts[k]->x;
			lens[3 * k + 1] = parts[k]->y;
			lens[3 * k + 2] = parts[k]->z;
		}
		lens[12]        = std::tan(cam.fov / 2);
		lens[13]        = double(drawnWidth) / double(drawnHeight);
		const int prev  = 1 - cur;
		const bool restarted = (fr->flags & KDN_FRAME_RESTART) != 0;
		const bool kept = f.shown == prev && f.stateWidth == drawnWidth && f.stateHeight == drawnHeight && !restarted;
		const bool moved = kept && std::memcmp(lens, f.lens, sizeof lens) != 0;
		TemporalArgs ta {};
		ta.width                  = drawnWidth;
		ta.height                 = drawnHeight;
		ta.moved                  = moved ? 1u : 0u;
		ta.recounted              = 0;
		ta.kept                   = kept ? 1u : 0u;
		ta.now                    = temporalCameraOf(lens, drawnWidth, drawnHeight);
		ta.before                 = temporalCameraOf(kept ? f.lens : lens, drawnWidth, drawnHeight);
		// temporal.cpp:187 temporalCentre: the grid read through the film each was drawn at
		filmCentreOf(factor, c.phase, ta.centre);
		if (kept) filmCentreOf(f.stateFactor, f.statePhase, ta.centreBefore);
		else filmCentreOf(factor, c.phase, ta.centreBefore);
		ta.io.light               = static_cast<const float*>(f.frameLight.ptr);
		ta.io.first_distance      = static_cast<const uint16_t*>(f.firstDistance.ptr);
		ta.io.first_normal        = static_cast<const uint16_t*>(f.firstNormal.ptr);
		ta.io.first_albedo        = static_cast<const uint16_t*>(f.firstAlbedo.ptr);
		ta.io.first_leaf          = static_cast<const uint32_t*>(f.firstLeaf.ptr);
		ta.io.centre_distance     = static_cast<const uint16_t*>(f.gDistance[cur].ptr);
		ta.io.centre_normal       = static_cast<const uint16_t*>(f.gNormal[cur].ptr);
		ta.io.centre_albedo       = static_cast<const uint16_t*>(f.gAlbedo[cur].ptr);
		ta.io.centre_leaf         = static_cast<const uint32_t*>(f.gLeaf[cur].ptr);
		ta.io.before_colour       = static_cast<const float*>(f.tColour[prev].ptr);
		ta.io.before_moment       = static_cast<const float*>(f.tMoment[prev].ptr);
		ta.io.before_length       = static_cast<const float*>(f.tLength[prev].ptr);
		ta.io.before_distance     = static_cast<const uint16_t*>(f.gDistance[prev].ptr);
		ta.io.before_normal       = static_cast<const uint16_t*>(f.gNormal[prev].ptr);
		ta.io.before_leaf         = static_cast<const uint32_t*>(f.gLeaf[prev].ptr);
		ta.io.colour              = static_cast<float*>(f.tColour[cur].ptr);
		ta.io.moment              = static_cast<float*>(f.tMoment[cur].ptr);
		ta.io.length              = static_cast<float*>(f.tLength[cur].ptr);
		// the chain `temporal` alone shows the temporal member's light
		const bool temporalOnly   = (fr->flags & KDN_FRAME_TEMPORAL) != 0;
		ta.io.image               = temporalOnly ? drawnImage : nullptr;
		if (!ctx->check(launchTemporal(ta, stream), "temporal kernel")) return KDN_CUDA_ERROR;
		++launches;
		kdn_denoise_frame df {};
		df.width  = drawnWidth;
		df.height = drawnHeight;
		for (int k = 0; k < 3; ++k) {
			df.eye[k]     = lens[k];
			df.forward[k] = lens[3 + k];
			df.right[k]   = lens[6 + k];
			df.up[k]      = lens[9 + k];
		}
		df.reach       = lens[12];
		df.aspect      = lens[13];
		df.demodulated = 1;
		if (!temporalOnly) {
			if ((s = denoiseOnDevice(ctx, &df, ta.io.colour, ta.io.moment, ta.io.length, ta.io.centre_distance, ta.io.centre_normal, ta.io.centre_albedo,
			                         ta.io.centre_leaf, drawnImage, stream)) != KDN_OK)
				return s;
			launches += 7;
		}
		if (upsampled) {
			// reconstruction/upsample as the chain's last member
			if (!ctx->check(launchUpsample(fr->width, fr->height, int(factor), drawnImage, image, stream, ctx->smCount), "upsample kernel")) return KDN_CUDA_ERROR;
			++launches;
			f.upShown = -1;
		} else if (factor > 1) {
			// plugins/reconstruction/upscale/upscale.cpp upscaledFrame: the
			// denoised drawn frame to the shown size, its history kept where
			// the last frame was upscaled to this size and the sequence goes on;
			// :557 settlingFrames counts the still frames after a movement
			const int upPrev     = f.upShown;
			const bool upKept    = upPrev >= 0 && f.upWidth == fr->width && f.upHeight == fr->height && !restarted;
			const bool lensMoved = f.upShown >= 0 && std::memcmp(lens, f.lens, sizeof lens) != 0;
			const int settling   = upKept ? (lensMoved ? 0 : (f.upMoved ? 4 : f.upSettling)) : 0;
			kdn_upscale_frame uf {};
			uf.width    = fr->width;
			uf.height   = fr->height;
			uf.factor   = factor;
			uf.phase    = c.phase;
			uf.kept     = upKept ? 1u : 0u;
			uf.settling = settling > 0 ? 1u : 0u;
			std::memcpy(uf.now, lens, sizeof lens);
			std::memcpy(uf.before, f.upShown >= 0 ? f.lens : lens, sizeof lens);
			const int upCur = upPrev >= 0 ? 1 - upPrev : 0;
			kdn_upscale_buffers ub {};
			ub.internal = drawnImage;
			ub.distance = ta.io.centre_distance;
			ub.before   = upKept ? static_cast<const float*>(f.upState[upPrev].ptr) : nullptr;
			ub.after    = static_cast<float*>(f.upState[upCur].ptr);
			ub.image    = image;
			if ((s = upscaleOnDevice(ctx, f.upscale, &uf, &ub, stream)) != KDN_OK) return s;
			launches += 2;
			f.upShown    = upCur;
			f.upWidth    = fr->width;
			f.upHeight   = fr->height;
			f.upMoved    = lensMoved;
			f.upSettling = std::max(settling - 1, 0);
		} else {
			f.upShown = -1;
		}
		std::memcpy(f.lens, lens, sizeof lens);
		f.stateWidth  = drawnWidth;
		f.stateHeight = drawnHeight;
		f.stateFactor = factor;
		f.statePhase  = c.phase;
		f.shown       = cur;
		f.current     = prev;
	}
	if (!ctx->check(cudaEventRecord(f.events[1], stream), "event")) return KDN_CUDA_ERROR;
	if (hostOut && !ctx->check(cudaMemcpyAsync(out, image, size_t(shownPixels) * 3 * sizeof(float), cudaMemcpyDeviceToHost, stream), "copy frame")) return KDN_CUDA_ERROR;
	if (!ctx->check(cudaStreamSynchronize(stream), "kdn_render")) return KDN_CUDA_ERROR;
	kdn_frame_stats st {};
	float ms = 0;
	cudaEventElapsedTime(&ms, f.events[0], f.events[1]);
	st.total_ms = ms;
	for (size_t k = 2; k + 1 < ev; k += 2) {
		float t = 0;
		cudaEventElapsedTime(&t, f.events[k], f.events[k + 1]);
		st.trace_ms += t;
	}
	unsigned long long host[8] = {};
	cudaMemcpy(host, ctx->counters.ptr, sizeof(host), cudaMemcpyDeviceToHost);
	st.march_steps   = host[0];
	st.program_steps = host[1];
	st.longest_march = uint32_t(host[2]);
	st.capped_rays   = host[3];
	st.segments      = host[4];
	st.carried_rays  = uint32_t(std::min<unsigned long long>(host[5], 0xFFFFFFFFull));
	// the rounds cover the longest wait a march budget can give a path: a
	// path ray left after the last round would be a fault of this backend
	if (host[6] != 0) return ctx->fail(KDN_CUDA_ERROR, "kdn_render: " + std::to_string(host[6]) + " path rays were left after the frame's last round");
	st.trace_launches = uint32_t((ev - 2) / 2);
	st.launches      = launches;
	st.other_ms      = st.total_ms - st.trace_ms;
	f.stats          = st;
	return KDN_OK;
}

} // namespace

extern "C" {

kdn_status kdn_render(kdn_ctx* handle, const kdn_frame* frame, float* out_rgb) {
	if (handle == nullptr || frame == nullptr || out_rgb == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->device < 0) return ctx->fail(KDN_NO_DEVICE, "kdn_render: a host-only context has no device");
	return renderFrame(ctx, frame, out_rgb, ctx->stream, true);
}

// Keep the learned guide where it pays.  Each method (plain, guided) draws
// pairs of independent pilot frames; a pair (A, B) gives the method's
// relative variance of one frame, mean((A - B)^2 / (((A + B) / 2)^2 + 0.01))
// / 2, and the mean of those times the mean device time of its frames (the
// frame's own CUDA events, kdn_frame_stats.total_ms, launch to last kernel)
// is its cost at equal time.  One untimed frame of each method comes first,
// so the guided path's buffers are allocated and both paths' kernels warm
// before any pilot is timed, and the methods' frames alternate so a drift in
// the GPU's clocks falls on both.  A frame's time varies far more than its
// variance (on small frames it is set by the few slowest rays), so pairs are
// drawn until the log of the cost ratio lies more than two standard errors
// (from the spread of the pairs' variances and of the frames' times) from
// the margin, kSelectLeastPairs at least and kSelectMostPairs at most.  The
// guide's sampling stays on only where its cost is below the plain cost by
// more than kSelectMargin.  Training (KDN_GUIDE_TRAIN) is left as it was,
// and off during the pilots.
constexpr int kSelectLeastPairs = 3;
constexpr int kSelectMostPairs  = 16;
constexpr double kSelectMargin  = 0.05;

namespace {

// Mean and squared relative standard error of the mean of n values from
// their sum and sum of squares.
struct Moments {
	double sum = 0.0, squares = 0.0;
	int n      = 0;
	void add(double v) {
		sum += v;
		squares += v * v;
		++n;
	}
	double mean() const { return n > 0 ? sum / n : 0.0; }
	double relativeError2() const {
		if (n < 2 || sum <= 0.0) return 0.0;
		const double m = sum / n, var = std::max(0.0, (squares - n * m * m) / (n - 1));
		return var / (n * m * m);
	}
};

} // namespace

kdn_status kdn_guide_select(kdn_ctx* handle, const kdn_frame* pilot, int* guided, double* plain_cost, double* guided_cost) {
	if (handle == nullptr || pilot == nullptr || guided == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (pilot->width <= 0 || pilot->height <= 0 || pilot->samples <= 0 || pilot->samples > (1 << 20) || pilot->surfaces <= 0 || pilot->surfaces > 255 ||
	    uint64_t(pilot->width) * uint64_t(pilot->height) > (uint64_t(1) << 26))
		return ctx->fail(KDN_BAD_ARG, "kdn_guide_select: the pilot's width and height (at most 2^26 pixels), samples (1..2^20) and surfaces (1..255) must be positive");
	if (ctx->device < 0) return ctx->fail(KDN_NO_DEVICE, "kdn_guide_select: a host-only context has no device");
	if (ctx->guide == nullptr || !kdn_guide_ready(ctx->guide)) return ctx->fail(KDN_NOT_READY, "kdn_guide_select: no trained guide on this context");
	const uint32_t flags = ctx->guideFlags;
	const size_t n       = size_t(pilot->width) * size_t(pilot->height) * 3;
	std::vector<float> img[2][2];
	for (auto& m : img) {
		for (auto& v : m) v.assign(n, 0.0f);
	}
	Moments ms[2], variance[2];
	kdn_frame fr       = *pilot;
	fr.accumulate      = 0;
	fr.flags           = 0;
	kdn_status s       = KDN_OK;
	// warm-up: one untimed frame a method
	for (int m = 0; m < 2 && s == KDN_OK; ++m) {
		ctx->guideFlags = m == 1 ? KDN_GUIDE_SAMPLE : 0u;
		fr.seed         = pilot->seed;
		s               = renderFrame(ctx, &fr, img[m][0].data(), ctx->stream, true);
	}
	const double threshold = -std::log(1.0 - kSelectMargin); // log(plain cost / guided cost) past which the guide pays
	double logRatio        = 0.0;
	for (int p = 0; p < kSelectMostPairs && s == KDN_OK; ++p) {
		for (int k = 0; k < 2 && s == KDN_OK; ++k) {
			for (int m = 0; m < 2 && s == KDN_OK; ++m) {
				ctx->guideFlags = m == 1 ? KDN_GUIDE_SAMPLE : 0u;
				fr.seed         = pilot->seed + uint32_t(2 * p + k + 1);
				s               = renderFrame(ctx, &fr, img[m][k].data(), ctx->stream, true);
				if (s == KDN_OK) ms[m].add(double(ctx->frame->stats.total_ms) * 1e-3);
			}
		}
		if (s != KDN_OK) break;
		for (int m = 0; m < 2; ++m) {
			const std::vector<float>& A = img[m][0];
			const std::vector<float>& B = img[m][1];
			double sum = 0.0;
			for (size_t i = 0; i < n; ++i) {
				const double d = double(A[i]) - double(B[i]), mean = 0.5 * (double(A[i]) + double(B[i]));
				sum += d * d / (mean * mean + 0.01);
			}
			variance[m].add(sum / double(n) / 2.0);
		}
		const double cp = variance[0].mean() * ms[0].mean(), cg = variance[1].mean() * ms[1].mean();
		logRatio        = cp > 0.0 && cg > 0.0 ? std::log(cp / cg) : 0.0;
		const double se = std::sqrt(variance[0].relativeError2() + variance[1].relativeError2() + ms[0].relativeError2() + ms[1].relativeError2());
		if (p + 1 >= kSelectLeastPairs && std::fabs(logRatio - threshold) > 2.0 * se) break;
	}
	if (s != KDN_OK) {
		ctx->guideFlags = flags;
		return s;
	}
	const double cost[2] = { variance[0].mean() * ms[0].mean(), variance[1].mean() * ms[1].mean() };
	*guided              = logRatio > threshold ? 1 : 0;
	ctx->guideFlags = (flags & ~KDN_GUIDE_SAMPLE) | (*guided ? KDN_GUIDE_SAMPLE : 0u);
	if (plain_cost) *plain_cost = cost[0];
	if (guided_cost) *guided_cost = cost[1];
	return KDN_OK;
}

kdn_status kdn_render_device(kdn_ctx* handle, const kdn_frame* frame, float* out_rgb, void* stream) {
	if (handle == nullptr || frame == nullptr || out_rgb == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->device < 0) return ctx->fail(KDN_NO_DEVICE, "kdn_render_device: a host-only context has no device");
	return renderFrame(ctx, frame, out_rgb, stream ? static_cast<cudaStream_t>(stream) : ctx->stream, false);
}

kdn_status kdn_frame_stats_get(kdn_ctx* handle, kdn_frame_stats* stats) {
	if (handle == nullptr || stats == nullptr) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->frame == nullptr) return ctx->fail(KDN_NOT_READY, "kdn_frame_stats_get: no frame drawn");
	*stats = ctx->frame->stats;
	return KDN_OK;
}

kdn_status kdn_frame_record(kdn_ctx* handle, float* light, uint16_t* distance, uint16_t* normal, uint16_t* albedo, uint32_t* leaf) {
	if (handle == nullptr || !light || !distance || !normal || !albedo || !leaf) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->frame == nullptr || !ctx->frame->surfaced()) return ctx->fail(KDN_NOT_READY, "kdn_frame_record: the last frame was not drawn with KDN_FRAME_DENOISE");
	const kdn::FrameState& f = *ctx->frame;
	const size_t n           = size_t(f.width) * size_t(f.height);
	if (!ctx->check(cudaSetDevice(ctx->device), "cudaSetDevice")) return KDN_CUDA_ERROR;
	const struct {
		void* to;
		const void* from;
		size_t bytes;
	} copies[] = { { light, f.frameLight.ptr, n * 12 }, { distance, f.firstDistance.ptr, n * 2 }, { normal, f.firstNormal.ptr, n * 6 },
		           { albedo, f.firstAlbedo.ptr, n * 6 }, { leaf, f.firstLeaf.ptr, n * 4 } };
	for (const auto& c : copies) {
		if (!ctx->check(cudaMemcpyAsync(c.to, c.from, c.bytes, cudaMemcpyDeviceToHost, ctx->stream), "kdn_frame_record copy")) return KDN_CUDA_ERROR;
	}
	if (!ctx->check(cudaStreamSynchronize(ctx->stream), "kdn_frame_record")) return KDN_CUDA_ERROR;
	return KDN_OK;
}

kdn_status kdn_frame_surfaces(kdn_ctx* handle, uint16_t* distance, uint16_t* normal, uint16_t* albedo, uint32_t* leaf) {
	if (handle == nullptr || !distance || !normal || !albedo || !leaf) return KDN_BAD_ARG;
	Context* ctx = reinterpret_cast<Context*>(handle);
	std::lock_guard<std::mutex> guard(ctx->lock);
	if (ctx->frame == nullptr || !ctx->frame->surfaced()) return ctx->fail(KDN_NOT_READY, "kdn_frame_surfaces: the last frame was not drawn with KDN_FRAME_DENOISE");
	const kdn::FrameState& f = *ctx->frame;
	const size_t n           = size_t(f.width) * size_t(f.height);
	if (!ctx->check(cudaSetDevice(ctx->device), "cudaSetDevice")) return KDN_CUDA_ERROR;
	const struct {
		void* to;
		const void* from;
		size_t bytes;
	} copies[] = { { distance, f.gDistance[f.shown].ptr, n * 2 }, { normal, f.gNormal[f.shown].ptr, n * 6 }, { albedo, f.gAlbedo[f.shown].ptr, n * 6 },
		           { leaf, f.gLeaf[f.shown].ptr, n * 4 } };
	for (const auto& c : copies) {
		if (!ctx->check(cudaMemcpyAsync(c.to, c.from, c.bytes, cudaMemcpyDeviceToHost, ctx->stream), "kdn_frame_surfaces copy")) return KDN_CUDA_ERROR;
	}
	if (!ctx->check(cudaStreamSynchronize(ctx->stream), "kdn_frame_surfaces")) return KDN_CUDA_ERROR;
	return KDN_OK;
}

} // extern "C"
