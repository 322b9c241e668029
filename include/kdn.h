/*
 * kdn.h -- C ABI of libkdn_gb300, the GB300 backend of the Kodanuki renderer.
 *
 * Plain C: every call takes plain pointers and sizes and returns a
 * kdn_status.  No call throws, prints or exits; the host plugin maps a status
 * to the reference's print-and-exit convention (reference rule 19,
 * core/render.cpp:140).  Calls on one context are serialised on the
 * context's CUDA stream; several worker threads may share a context (each
 * call takes the context's lock).
 *
 * Record layouts are the reference's plain-data types byte for byte where
 * one exists (Step, Ray, Hit) and the fields of the reference's scene types
 * otherwise; each is cited below (paths within the reference's source/).
 */
#ifndef KDN_H
#define KDN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum kdn_status {
	KDN_OK = 0,
	KDN_BAD_ARG = 1,    /* a null pointer, a bad block name or size, a size past a limit */
	KDN_OOM = 2,        /* device memory or the admission budget ran out */
	KDN_TIMEOUT = 3,    /* a device loop reached its iteration limit and stopped */
	KDN_CUDA_ERROR = 4, /* a CUDA call failed; kdn_last_error says which */
	KDN_NOT_READY = 5,  /* a call needs blocks or a build that are missing */
	KDN_NO_DEVICE = 6   /* no CUDA device, or the kernels were not built for it */
} kdn_status;

typedef struct kdn_ctx kdn_ctx;

/* sdf/program.h:56 Step: opcode (sdf/program.h:20 Opcode), operands, value, leaf. 32 bytes. */
typedef struct kdn_step {
	uint8_t opcode;
	uint32_t a, b, c;
	double value;
	uint32_t leaf;
} kdn_step;

/* One object program (sdf/scene.cpp:280 objectProgram) as a run of kdn_step. */
typedef struct kdn_program_ref {
	uint32_t first;  /* first step in the "scene.steps" block */
	uint32_t count;  /* number of steps */
	uint32_t result; /* the step whose value is the program's */
} kdn_program_ref;

/* core/batch.h:125 Ray, 36 bytes. */
typedef struct kdn_ray {
	float origin[3];
	float direction[3];
	float far;
	uint8_t inside;
	uint8_t pad_[3];
	uint32_t within; /* material index, 0xFFFFFFFF for none */
} kdn_ray;

/* core/batch.h:157 Hit, 56 bytes. kind: 0 missed, 1 surface, 2 solid. */
typedef struct kdn_hit {
	uint8_t kind;
	uint8_t pad0_[3];
	float distance;
	float point[3];
	float normal[3];
	uint32_t leaf;
	uint32_t other;
	float share;
	float loosened;
	uint8_t leaf_kind;
	uint8_t pad1_[3];
	uint32_t cell;
} kdn_hit;

/* sdf/scene.h Material (its fields the backend reads), 64 bytes. */
typedef struct kdn_material {
	uint32_t kind;      /* sdf/scene.h MaterialKind: 0 matte, 1 plastic, 2 metal, 3 glass */
	float albedo[3];    /* the first colour stop (a constant albedo) */
	float roughness;
	float refraction;
	float dispersion;   /* Cauchy B in square micrometres */
	float absorb[3];
	float glow[3];
	float strength;
	uint32_t flags_;    /* 1: the albedo is a ramp read off a pattern program ("looks.patterns") */
	float scatter;      /* a glass: how much of a unit of travel its body turns aside (0: none) */
	float lean;         /* Henyey-Greenstein's g of that scattering, in (-1, 1) */
	uint32_t pad_;
} kdn_material;

/* plugins/transport/paths/material/energy.h Boundary of a glass, 9112
 * bytes: what one bounce off a rough dielectric boundary returns, seen from
 * the rarer and the denser side (17 index ratios from 1 to 3 by 32 views),
 * their cosine-weighted averages and the share of the rarer side's loss
 * that comes back on the far side.  Part of the reference's Finish
 * (material.cpp:187 finishWith, boundaryOf); one per material in
 * "transport.boundaries" (zeros for a material that is no glass). */
typedef struct kdn_boundary {
	double rarer[17][32];
	double denser[17][32];
	double rarer_average[17];
	double denser_average[17];
	double rarer_through[17];
} kdn_boundary;

/* sdf/scene.h Albedo of one material, 32 bytes: a ramp over a pattern
 * program.  The program's steps are [first, first + count) of the
 * "looks.pattern_steps" block (at most 64 steps; operands index steps of
 * the same program, as sdf/program.h Step), its value is step `result`; an
 * Argument step reads "looks.pattern_arguments"[argument_first + a] (the
 * Scene::arguments the Albedo names); the ramp's stops are
 * [stop_first, stop_first + stop_count) of "looks.stops" (3 floats a stop,
 * spread evenly over 0..1); world: read in world space rather than the
 * painted leaf's (its "looks.placements" entry).  count 0 for a flat colour. */
typedef struct kdn_pattern {
	uint32_t first, count, result;
	uint32_t argument_first, argument_count;
	uint32_t stop_first, stop_count;
	uint32_t world;
} kdn_pattern;

/* sdf/scene.h Placement of one leaf, 96 bytes: the painted shape's space is
 * linear x (p - origin) (material.cpp:292 placedVector). */
typedef struct kdn_placement {
	double linear[3][3];
	double origin[3];
} kdn_placement;

/* plugins/transport/paths/material/material.h:70 Finish: how a material is
 * drawn, as the reference's transport derives it from the Material
 * (material.cpp:204 finishWith), its GGX width, facet share, coat and escape
 * table (material/energy.h:12 Escape: 32 views) included.  352 bytes. */
typedef struct kdn_finish {
	uint32_t kind;
	uint32_t sharp;
	uint32_t exact;      /* a smooth glass answered exactly */
	uint32_t loses_much; /* a rough glass that gives back what single scattering loses (its boundary tables in transport.boundaries) */
	double width;
	double facet_share;
	double body;
	double index;
	double coat_front, coat_twice, coat_room;
	double escape_average;
	double escape[32];
	double film[2];      /* the thin film (material.cpp:106 filmOf): thickness in nm (0: none), index */
} kdn_finish;

/* sdf/scene.h Light, 136 bytes. kind: sdf/scene.h LightKind (0 point, 1 directional, 2 sphere, 3 quad, 4 sun, 5 moon); direction: toward a directional light, a sun or a moon; angle: a sun's or a moon's disc, radians across. */
typedef struct kdn_light {
	uint32_t kind;
	float radius;
	float angle;
	float pad_;
	double at[3];
	double direction[3];
	double along[3];
	double across[3];
	double power[3]; /* linear RGB */
} kdn_light;

/* sdf/scene.h Sky and Stars, 136 bytes: its kind (SkyKind: 0 gradient, 1 physical;
 * a painted sky is refused); a gradient's linear RGB zenith, horizon and
 * ground; a physical sky's haze and ground albedo (`ground`); the glow
 * about the first sun (glow x strength, falling by e over `spread` radians:
 * plugins/feature/sky_layers/sky_layers.cpp:181 glowSeen). */
typedef struct kdn_sky {
	double zenith[3];
	double horizon[3];
	double ground[3];
	double glow[3];
	double strength;
	double spread;
	uint32_t kind;
	float haze;
	/* sdf/scene.h Stars (sky_layers.cpp:240 starlight): present (1), about
	 * how many over the sphere, the brightest's strength, a disc's angle */
	uint32_t stars;
	float star_count, star_strength, star_angle;
} kdn_sky;

/* sdf/scene.h Camera and the Render fields a frame reads. */
typedef struct kdn_camera {
	double eye[3];
	double target[3];
	double up[3];
	double fov;
	double aperture;
	double focus;
} kdn_camera;

/* core/geometry.h:14 Region: the box the world is built over. */
typedef struct kdn_region {
	double lower[3];
	double size[3];
} kdn_region;

/* How the cut octree is grown (plugins/geometry/tree/cut.cpp:463 cutCell per
 * cell): every surface cell is split down to min_depth, and further, down to
 * max_depth, while its kept programs hold more than split_steps steps. */
typedef struct kdn_build_options {
	int32_t min_depth;
	int32_t max_depth;
	uint32_t split_steps;
	uint32_t pad_;
} kdn_build_options;

/* One frame of fixed-count samples (stopping/fixed_count). */
typedef struct kdn_frame {
	int32_t width, height;
	int32_t samples;  /* samples per pixel drawn by this call, 1 .. 2^20 */
	int32_t surfaces; /* render.surfaces: the most surfaces a path stands on */
	int32_t seed;     /* render.seed */
	uint32_t first;   /* sample index of this call's first sample of every pixel */
	uint32_t accumulate; /* 1: add to the pixel sums of the previous call */
	uint32_t flags;      /* KDN_FRAME_DENOISE: return the denoised frame */
	/* core/camera.h:65 FilmPlan: with a factor of 2 to 4 (0 or 1: none) the
	 * frame is drawn at width / factor x height / factor, each drawn pixel's
	 * samples aimed at the shown pixel (x * factor + phase % factor,
	 * y * factor + phase / factor) (plugins/transport/paths/trace.cpp:93
	 * phasedDraw), and shown at width x height through the reconstruction
	 * chain temporal + a-trous + upscale (KDN_FRAME_DENOISE), or a chain
	 * ending in upsample (KDN_FRAME_UPSAMPLE); the size must be a multiple
	 * of the factor.  The pixel sums, the record and the G-buffer are at the
	 * drawn size. */
	uint32_t factor;
	uint32_t phase; /* 0 .. factor^2 - 1: core/shown.cpp bayerFilm gives the order */
	/* render.collisions: the most collisions inside scattering bodies a path
	 * stands on, apart from its surfaces (0: the reference's default, 256) */
	int32_t collisions;
	/* render.split: 2, 4 or 8 samples share a first vertex (its camera ray,
	 * wavelengths and aim; each branch scatters on its own,
	 * plugins/transport/paths/trace.cpp:1568 branchedFrom), the aim there
	 * weighed as one of that many (weight.cpp:15 sharedAim); 0 or 1: none */
	uint32_t split;
} kdn_frame;

/* With KDN_FRAME_DENOISE a frame returns what the reference shows through
 * its reconstruction chain temporal + a-trous: it also records each pixel's
 * light of this call and the first surface of its last sample, traces the
 * G-buffer (one ray through each pixel's centre, core/surfaces.cpp:133
 * tracedSurfaces: distance, normal facing the ray and albedo as FP16, and
 * the leaf), runs the temporal member (kdn_temporal_device: its history is
 * the last denoised frame's where that was of this size, reprojected when
 * the camera moved) and puts the temporal state through the a-trous
 * denoiser (kdn_denoise, demodulated).  A frame without the flag drops the
 * history.  `accumulate` still adds this call's samples to the pixel sums,
 * which a frame without the flag shows. */
#define KDN_FRAME_DENOISE 1u
/* With KDN_FRAME_DENOISE: start the temporal history over (the sequence's
 * cut: every member drops its history). */
#define KDN_FRAME_RESTART 2u
/* With KDN_FRAME_DENOISE: the chain stops after the temporal member (the
 * reference's --reconstruction temporal): no a-trous filter. */
#define KDN_FRAME_TEMPORAL 4u
/* At a film factor above 1: the chain's last member is upsample (bilinear,
 * no history) instead of upscale; without KDN_FRAME_DENOISE the chain is
 * mean + upsample (the drawn frame's pixel means blown up). */
#define KDN_FRAME_UPSAMPLE 8u
/* --use sampler=sobol (plugins/sampler/sobol): the first 28 dimensions of
 * every path's draws from a Sobol sequence Owen-scrambled per pixel
 * (plugins/transport/paths/sampler.cpp:16 numberAt), the rest hashed as
 * without it. */
#define KDN_FRAME_SOBOL 16u
/* --use sampler=sky_map (plugins/sampler/sky_map): the sky aimed at as a
 * light after the lamps, by a chart of its brightness (64 x 128 cells of
 * equal solid angle, a tenth of the draws uniform), unless the lamps
 * outshine it five times over at the region's middle; a path that meets
 * the sky weighs it against that aim. */
#define KDN_FRAME_SKY_MAP 32u
/* --use sampler=each_lamp_first (plugins/sampler/each_lamp_first): at a
 * path's first vertex each of the first four lamps whose offer is bright
 * traces a shadow line of its own, outside the one-offer reservoir
 * (plugins/transport/paths/trace.cpp:935); the aim densities, so the MIS
 * weights, are those without it. */
#define KDN_FRAME_EACH_LAMP 64u

/* Device times of the last kdn_render, from CUDA events on the context's stream. */
typedef struct kdn_frame_stats {
	double total_ms;
	double trace_ms;   /* every launch of the sphere-trace kernel (paths and lines) */
	double shade_ms;   /* arrive + aim + scatter */
	double other_ms;   /* camera, fold, compaction */
	uint64_t segments; /* rays traced (camera + scatter + shadow) */
	uint64_t march_steps;
	uint64_t program_steps; /* program steps run by the trace kernel */
	uint32_t launches;
	uint32_t longest_march; /* the most march steps one ray took */
	uint64_t capped_rays;   /* rays that ran out of march steps (65536) */
	uint32_t trace_launches; /* launches of the sphere-trace kernel in trace_ms */
	uint32_t carried_rays;   /* marches carried to a later launch (kdn_set_march_budget) */
} kdn_frame_stats;

const char* kdn_status_string(kdn_status status);
/* The message of the last failed call on this context (or of kdn_open). */
const char* kdn_last_error(const kdn_ctx* ctx);

/* Open a context on one CUDA device.  Replaces the reference's per-worker
 * Backend state (core/plugin.h:333 openWorkers).  KDN_HOST_ONLY opens a
 * context without a device: blocks and kdn_build/kdn_world_* work, every
 * device entry point returns KDN_NO_DEVICE. */
#define KDN_HOST_ONLY (-1)
kdn_status kdn_open(int device, kdn_ctx** out);
kdn_status kdn_close(kdn_ctx* ctx);

/* A context that draws frames of `scene`'s built world without a copy of
 * it: the world's device buffers are borrowed, the blocks copied, the frame
 * buffers, streams (created at `priority`, as cudaStreamCreateWithPriority:
 * lower is more urgent, clamped to the device's range) and counters its
 * own, so frames of one scene run side by side on several such contexts.
 * The scene may be neither rebuilt nor closed while a sharing context is
 * open (KDN_BAD_ARG).  A host-only scene gives a host-only context. */
kdn_status kdn_open_sharing(kdn_ctx* scene, int priority, kdn_ctx** out);

/* The most device bytes a frame's path buffers may take on this context
 * (0, the default: half the free device memory); a frame larger than that
 * is drawn in more chunks. */
kdn_status kdn_set_frame_budget(kdn_ctx* ctx, uint64_t bytes);

/* Size this context's kernel grids for `sms` SMs (0: all of the device's),
 * so its frames leave the other SMs to work on other streams. */
kdn_status kdn_set_sm_limit(kdn_ctx* ctx, int sms);

/* March steps a ray may take in one trace launch of this context's frames
 * (0, the default, or 65536 and above: no limit).  A ray past it stops with
 * its march state (distance and step count) and goes on in the next launch,
 * so no launch waits for the few rays that skim a surface for thousands of
 * steps (the reference marches each ray to its end in one call,
 * plugins/geometry/sphere_trace/sphere_trace.cpp:203, at most 65536 steps,
 * sphere_trace.h:20); a path whose shadow line is still marching waits for
 * it before its next vertex is shaded.  Frames are the same to the bit with
 * any budget.  Frames sampling the learned guide march without a budget. */
kdn_status kdn_set_march_budget(kdn_ctx* ctx, uint32_t steps);

/*
 * Copy one block into the context (core/block.h:565 Block {name, data,
 * count, size}).  Names and element sizes:
 *   "scene.steps"      kdn_step, 32        every object program end to end
 *   "scene.programs"   kdn_program_ref, 12 one per object (Scene::objectPrograms)
 *   "scene.leaves"     uint32_t, 4         the material of each leaf (Leaf::material)
 *   "looks.materials"  kdn_material, 64
 *   "transport.finishes" kdn_finish, 352 one per material (plugins/transport/paths/plugin.cpp:201)
 *   "lighting.lights"  kdn_light, 136
 *   "lighting.sky"     kdn_sky, 72         one
 *   "shot.camera"      kdn_camera, 96      one
 *   "geometry.region"  kdn_region, 48      one
 *   "looks.patterns"   kdn_pattern, 32     one per material, where any albedo is patterned
 *   "looks.pattern_steps" kdn_step, 32     the pattern programs end to end (Scene::programs)
 *   "looks.pattern_arguments" double, 8    the arguments they read (Scene::arguments)
 *   "looks.stops"      float, 4            the ramps' stops, 3 floats a stop
 *   "looks.placements" kdn_placement, 96   one per leaf (Leaf::placement)
 *   "transport.boundaries" kdn_boundary, 9112 one per material, where a rough glass loses much
 * A block replaces the one of the same name; the world must be rebuilt
 * (kdn_build) after any scene.* or geometry.* block changes.
 */
kdn_status kdn_upload_block(kdn_ctx* ctx, const char* name, const void* data, size_t count, size_t size);

/* Build the cut octree over the scene's programs and make the world
 * resident on the device (plugins/geometry/tree/plugin.cpp:37 treeBuilt). */
kdn_status kdn_build(kdn_ctx* ctx, const kdn_build_options* options);
/* Counts of the built world: cells, leaves, kept programs, program steps. */
kdn_status kdn_world_stats(kdn_ctx* ctx, uint64_t out[4]);
/* Copy cell i (depth-first pre-order) of the built octree: head = level,
 * place x/y/z, occupancy, program count; objects/results/counts get one
 * entry per kept program, steps the programs' kdn_steps end to end.  Pass
 * null arrays to read the head alone. */
kdn_status kdn_world_cell(kdn_ctx* ctx, uint64_t i, uint32_t head[6], uint32_t* objects, uint32_t* results, uint32_t* counts, kdn_step* steps, size_t steps_capacity);
/* The march form the trace kernel runs for cell i (depth-first pre-order),
 * run on the host: every kept program of the cell at n points (x, y, z
 * floats), values[k * n + j] for program k at point j, up to capacity
 * values; *programs gets the count.  A check of the march form against the
 * cell's programs (the same interpreter as the device's, FP32).
 * KDN_NOT_READY where the device layout could not be made. */
kdn_status kdn_world_march(kdn_ctx* ctx, uint64_t i, const float* points, uint32_t n, float* values, size_t capacity, uint32_t* programs);
/* The leaf of each of n points (x, y, z floats) as the trace kernel locates
 * it (the level-6 grid, then the descent) and by the descent from the root,
 * both run on the host: the two must name the same leaf for every point. */
kdn_status kdn_world_locate(kdn_ctx* ctx, const float* points, uint32_t n, uint32_t* by_grid, uint32_t* by_descent);

/* ExtendRays (core/step.cpp:132): the first hit of each ray, host arrays in
 * and out (a host-to-device and device-to-host copy each call).  The
 * caller passes only the pool slots that wait on a ray (core/batch.h:360
 * waitsOnRay) and marks them answered, as execution/single does
 * (plugins/execution/single/plugin.cpp:28-36); the pool's ray kinds are not
 * passed because the geometry traces every kind alike (the reference's
 * intersect takes none) and the kinds only feed the caller's ray counters
 * (kodanuki_gb300/reference_plugin/backend_gb300.cpp keeps them).  A hit's
 * cell holds the device's object index; the binding clears it, as the
 * reference's sphere-traced hits carry no tree cell. */
kdn_status kdn_extend(kdn_ctx* ctx, const kdn_ray* rays, uint32_t n, kdn_hit* hits);
/* The same over device arrays, on the given CUDA stream (0: the context's). */
kdn_status kdn_extend_device(kdn_ctx* ctx, const kdn_ray* rays, uint32_t n, kdn_hit* hits, void* stream);

/* Render samples of one frame into the context's pixel sums and write the
 * pixel means, linear RGB float, row-major, 3 floats a pixel.  out is a host
 * pointer (kdn_render) or a device pointer (kdn_render_device).  Matte,
 * plastic, metal and glass (smooth or rough, dispersive, absorbing, under a
 * thin film or not) are drawn; a scene with a medium (a scattering body) or
 * a passable glass (refraction 1 without dispersion or film) is refused
 * with KDN_BAD_ARG. */
kdn_status kdn_render(kdn_ctx* ctx, const kdn_frame* frame, float* out_rgb);
kdn_status kdn_render_device(kdn_ctx* ctx, const kdn_frame* frame, float* out_rgb, void* stream);
kdn_status kdn_frame_stats_get(kdn_ctx* ctx, kdn_frame_stats* stats);

/* The first surfaces of the last frame drawn with KDN_FRAME_DENOISE, a pixel
 * each, row-major, into host arrays: distance (FP16, infinite where the ray
 * missed), normal and albedo (FP16 x3), leaf (0xFFFFFFFF where missed).
 * Replaces core/frame.cpp:508 shownSurfaces.  KDN_NOT_READY when the last
 * frame kept none. */
kdn_status kdn_frame_surfaces(kdn_ctx* ctx, uint16_t* distance, uint16_t* normal, uint16_t* albedo, uint32_t* leaf);
/* The record of the last frame drawn with KDN_FRAME_DENOISE (core/shown.h
 * FrameRecord): each pixel's light of that call (RGB float), and the first
 * surface of its last sample (FP16 distance, normal, albedo; leaf), into
 * host arrays.  KDN_NOT_READY when the last frame kept none. */
kdn_status kdn_frame_record(kdn_ctx* ctx, float* light, uint16_t* distance, uint16_t* normal, uint16_t* albedo, uint32_t* leaf);

/* One frame of the denoiser's feature buffers: the frame size, whether the
 * light is already divided by the albedo (TemporalState::demodulated), and
 * the camera the frame was drawn with (core/camera.h Lens: eye, forward,
 * right, up, reach = tan(fov / 2), aspect = width / height). */
typedef struct kdn_denoise_frame {
	int32_t width, height;
	uint32_t demodulated;
	uint32_t pad_;
	double eye[3], forward[3], right[3], up[3];
	double reach, aspect;
} kdn_denoise_frame;

/*
 * The SVGF-like a-trous denoiser (plugins/reconstruction/atrous/atrous.cpp:513
 * denoisedFrame) over one frame's feature buffers, a pixel each, row-major:
 *   colour   float x3   the temporal light (TemporalPixel::colour)
 *   moment   float      its second moment of luminance
 *   length   float      the history length in samples
 *   distance FP16       camera distance of the first surface (inf or 0: sky)
 *   normal   FP16 x3    its normal
 *   albedo   FP16 x3    its albedo
 *   leaf     uint32     its leaf, 0xFFFFFFFF for the sky
 * out gets RGB float x3.  kdn_denoise takes host arrays (copied in and out
 * on the context's stream); kdn_denoise_device takes device arrays.  The
 * context keeps 68 bytes a pixel of scratch between calls.
 */
kdn_status kdn_denoise(kdn_ctx* ctx, const kdn_denoise_frame* frame, const float* colour, const float* moment, const float* length,
                       const uint16_t* distance, const uint16_t* normal, const uint16_t* albedo, const uint32_t* leaf, float* out_rgb);
kdn_status kdn_denoise_device(kdn_ctx* ctx, const kdn_denoise_frame* frame, const float* colour, const float* moment, const float* length,
                              const uint16_t* distance, const uint16_t* normal, const uint16_t* albedo, const uint32_t* leaf, float* out_rgb,
                              void* stream);

/*
 * kdn_denoise_device without a context and without allocating: for callers
 * that may not allocate device memory once running (a frame loop that
 * reserved its device-memory budget at start-up, or one that must not stall
 * its other streams on the synchronisation cudaMalloc/cudaFree can cause).
 * No counterpart in the reference: its denoiser runs on the host.
 *
 * Its scratch is a static device array of 17 MiB that every GPU loading
 * the library holds until exit; frames of more than 262144 pixels (512x512)
 * are refused with KDN_BAD_ARG.  It runs on the current device, on the given
 * stream; the arrays are device pointers as for kdn_denoise_device.  The
 * first call on a device looks the array's device address up; make that
 * first call before any stream capture.  A call copies nothing from host
 * memory: the lens travels in the kernels' parameters.  All calls share the
 * array: calls whose work overlaps on the GPU race.  Nothing in it has to
 * start at zero.
 * The message of a failed call is kdn_last_error(NULL) on the calling thread.
 */
kdn_status kdn_denoise_static(const kdn_denoise_frame* frame, const float* colour, const float* moment, const float* length, const uint16_t* distance,
                              const uint16_t* normal, const uint16_t* albedo, const uint32_t* leaf, float* out_rgb, void* stream);

/*
 * The temporal member (plugins/reconstruction/temporal/temporal.cpp:1001
 * temporalFrame) for one frame with a G-buffer: the drawn grid the
 * reference runs before the a-trous denoiser, each pixel's light divided by
 * the albedo of its sample's first surface.  At a film factor above 1 a
 * grid pixel's rays pass through the centre of the shown pixel its phase
 * aims at (core/camera.cpp:51 filmCentre), this frame's and, for the
 * history, the state before's.  Each pixel blends
 * this frame's light into its history: its own on a still camera, else the
 * frame before's pixels around where its G-buffer point was seen whose
 * surface lies on its plane (bilinear), clamped to this frame's 3x3
 * neighbourhood while the history is young or the camera moves; the state
 * after is its colour, moment and length, and what it shows is its
 * G-buffer surface.  kdn_render with KDN_FRAME_DENOISE runs it between the
 * frame and the a-trous denoiser; kdn_temporal_device runs it alone.
 */
typedef struct kdn_temporal_frame {
	int32_t width, height; /* the drawn grid */
	uint32_t moved;     /* the camera moved since the frame before */
	uint32_t recounted; /* the scene's shapes changed: leaves compare as hit or sky alone */
	uint32_t kept;      /* the state before holds a frame of this size */
	uint32_t factor;    /* this frame's film factor (0 or 1: none) and phase */
	uint32_t phase;
	uint32_t before_factor; /* the state before's film factor and phase */
	uint32_t before_phase;
	uint32_t pad_;
	double now[14], before[14]; /* lenses: eye, forward, right, up, reach, aspect */
} kdn_temporal_frame;

/* Device arrays, a pixel each, row-major.  FP16 fields are bit patterns. */
typedef struct kdn_temporal_buffers {
	const float* light;              /* x3: the frame's pixel means */
	const uint16_t* first_distance;  /* the first surface of each pixel's last sample */
	const uint16_t* first_normal;    /* x3 */
	const uint16_t* first_albedo;    /* x3 */
	const uint32_t* first_leaf;
	const uint16_t* centre_distance; /* the G-buffer: the surface through the pixel's centre */
	const uint16_t* centre_normal;
	const uint16_t* centre_albedo;
	const uint32_t* centre_leaf;
	const float* before_colour;      /* x3: the state before (read when kept) */
	const float* before_moment;
	const float* before_length;
	const uint16_t* before_distance; /* the frame before's G-buffer */
	const uint16_t* before_normal;
	const uint32_t* before_leaf;
	float* colour;                   /* x3: the state after (demodulated light) */
	float* moment;
	float* length;
	float* image;                    /* x3: the shown light, or null */
} kdn_temporal_buffers;

kdn_status kdn_temporal_device(kdn_ctx* ctx, const kdn_temporal_frame* frame, const kdn_temporal_buffers* buffers, void* stream);

/*
 * The upscale member (plugins/reconstruction/upscale/upscale.cpp
 * upscaledFrame) for one frame at a film factor of 2 to 4: a frame drawn at
 * 1/factor of the shown size, each drawn pixel's samples aimed at one
 * phase of the factor^2 shown pixels it covers, gathered to the shown size.
 * Each shown pixel takes the 3x3 drawn pixels around it (Gaussian and
 * Catmull-Rom weights) and blends them into the shown pixels of the frame
 * before where its nearest surface was seen there and the depth matches,
 * the history clamped to the 3x3's mean and deviation.  kdn_render with
 * KDN_FRAME_DENOISE at a film factor above 1 runs it after the a-trous
 * denoiser; kdn_upscale_device runs it alone.  Its answers are the
 * reference's to the bit.
 */
typedef struct kdn_upscale_frame {
	int32_t width, height; /* the shown size: the drawn size times the factor */
	uint32_t factor;       /* 2, 3 or 4 */
	uint32_t phase;        /* the phase this frame's draws aimed at, 0 .. factor^2 - 1 */
	uint32_t kept;         /* the state before is of this size and the sequence goes on */
	uint32_t settling;     /* upscale.cpp:557 settlingFrames is above 0: blend at alpha 1 */
	double now[14], before[14]; /* lenses at the shown size: eye, forward, right, up, reach, aspect */
} kdn_upscale_frame;

/* Device arrays, row-major. */
typedef struct kdn_upscale_buffers {
	const float* internal;    /* x3 at the drawn size: the reconstructed frame (temporal + a-trous) */
	const uint16_t* distance; /* FP16 bits at the drawn size: the G-buffer's distances; null: every sample sky */
	const float* before;      /* x4 at the shown size: the state before, colour and depth (read when kept) */
	float* after;             /* x4: the state after */
	float* image;             /* x3: the shown frame */
} kdn_upscale_buffers;

kdn_status kdn_upscale_device(kdn_ctx* ctx, const kdn_upscale_frame* frame, const kdn_upscale_buffers* buffers, void* stream);

/* The upsample member (plugins/reconstruction/upsample/upsample.cpp
 * upsampledImage): the drawn frame (device RGB float, width / factor x
 * height / factor) bilinearly to width x height (device RGB float), the
 * taps clamped to the drawn frame; its answers are the reference's to the
 * bit.  factor 1 to 4; the size a multiple of it. */
kdn_status kdn_upsample_device(kdn_ctx* ctx, int32_t width, int32_t height, uint32_t factor, const float* drawn, float* shown, void* stream);

/* Write a buffer larger than the L2 cache on the context's stream, so that
 * the next launch starts with a cold cache. */
kdn_status kdn_flush_l2(kdn_ctx* ctx);

/*
 * The serving loop (the render host's request loop, core/plugin.h:241
 * hostRenderer, as continuous batching): resident scenes, requests of any
 * scene, size and spp submitted as they arrive and drawn side by side on
 * the device, progressive sessions whose accumulation and denoiser history
 * stay resident, admission against a device-memory budget, and the
 * latency of every request.
 *
 * Each request runs on a context sharing its scene's world
 * (kdn_open_sharing) from a pool per scene; a session keeps its own until
 * it ends.  Up to `slots` requests are on the device at once, each on its
 * own streams; a request is admitted, interactive requests first and each
 * kind oldest first, when a slot is free (at most batch_slots of them
 * holding requests that are not interactive) and its path buffers (its
 * paths x 364 bytes, capped at budget / slots, or at batch_frame_bytes for
 * a batch request) fit in what the running requests leave of the budget.
 * Interactive requests (KDN_REQUEST_INTERACTIVE) run on high-priority
 * streams over every SM; batch requests run in short chunks on grids sized
 * for batch_sm_percent of the SMs between them, so an interactive frame
 * finds SMs free and a batch launch gives its SMs back soon.  Latency percentiles count the requests that
 * completed.  A frame's result
 * equals the same request drawn alone (kdn_render on a context of the same
 * scene).
 */
typedef struct kdn_server kdn_server;

typedef struct kdn_serve_options {
	int32_t device;             /* CUDA device, or KDN_HOST_ONLY (requests then end in KDN_NO_DEVICE) */
	uint32_t slots;             /* requests on the device at once, 1..64 */
	uint64_t budget_bytes;      /* device bytes the running requests' path buffers may take; 0: 120 GB */
	uint32_t batch_slots;       /* of the slots, the most that hold requests not interactive; 0: a quarter (at least 1) */
	uint32_t batch_sm_percent;  /* the SMs the batch requests' grids are sized for together; 0: 50 */
	uint64_t batch_frame_bytes; /* a batch request's path buffers, larger frames drawn in more chunks (short launches); 0: 1 GiB */
} kdn_serve_options;

#define KDN_REQUEST_INTERACTIVE 4u /* drawn on high-priority streams */

typedef struct kdn_request {
	uint32_t scene;   /* from kdn_serve_add_scene */
	int32_t width, height;
	int32_t samples;  /* a pixel, this request */
	int32_t surfaces;
	int32_t seed;
	uint32_t flags;   /* KDN_FRAME_DENOISE, KDN_REQUEST_INTERACTIVE */
	uint32_t pad_;
	uint64_t session; /* 0: a single frame; else a progressive session: its
	                     frames accumulate in order onto one resident frame
	                     (and denoiser history) until kdn_serve_end_session */
} kdn_request;

typedef struct kdn_served {
	kdn_status status;
	uint32_t frame;     /* the session's frame index (0 for a single frame) */
	double queued_ms;   /* submit to start */
	double render_ms;   /* start to the result in host memory */
	double latency_ms;  /* submit to the result */
} kdn_served;

kdn_status kdn_serve_open(const kdn_serve_options* options, kdn_server** out);
/* Register a built scene context (it stays the caller's; close it after the server). */
kdn_status kdn_serve_add_scene(kdn_server* server, kdn_ctx* scene, uint32_t* id);
/* Queue a request; out_rgb (width x height x 3 floats, host) is written
 * before kdn_serve_wait returns for its ticket. */
kdn_status kdn_serve_submit(kdn_server* server, const kdn_request* request, float* out_rgb, uint64_t* ticket);
/* Wait for a request (each ticket once). */
kdn_status kdn_serve_wait(kdn_server* server, uint64_t ticket, kdn_served* out);
/* Drop every queued request not yet started: its wait returns
 * KDN_NOT_READY at once (requests on the device finish). */
kdn_status kdn_serve_cancel_queued(kdn_server* server, uint64_t* cancelled);
/* End a session: its context goes back when its frames are done. */
kdn_status kdn_serve_end_session(kdn_server* server, uint64_t session);
/* Latency percentiles over the requests waited for so far (all, or only
 * the interactive ones). */
kdn_status kdn_serve_latency(kdn_server* server, int interactive_only, double* p50_ms, double* p99_ms, uint64_t* count);
/* Forget the latencies counted so far (after a warm-up). */
kdn_status kdn_serve_reset_latency(kdn_server* server);
const char* kdn_serve_last_error(const kdn_server* server);
/* Stop the workers (after the requests on the device finish), drop what is
 * still queued and close the server's contexts; call it once every ticket
 * that will be waited for has been. */
kdn_status kdn_serve_close(kdn_server* server);

/*
 * The learned guide (an added form: the reference's guides are the highlight
 * guide, plugins/sampler/highlight_guide/mixture.cpp:113 mixtureDirection,
 * and the plain BSDF sampling of the default sampler, paths/sampler.cpp:93
 * drawDirection; this is the guiding plugin point's learned proposal).
 *
 * A multiresolution hash-grid encoding of the position (16 levels, 2
 * features a level, 2^table_log2 entries a level, FP16 table) and the
 * vertex's faced normal feed a 3 x 64 ReLU network whose 40 outputs are a
 * mixture of eight von Mises-Fisher lobes over directions.  It is trained
 * online, on the device, on the radiance the tracer carries back to each
 * recorded vertex (loss mean(-w log q(direction)), Adam), and a frame
 * samples with it by one-sample MIS with the BSDF (kdn_set_guide), so the
 * estimate stays unbiased.  Both the training and the inference run on
 * the tensor cores (BF16 operands, FP32 accumulation).
 */
typedef struct kdn_guide kdn_guide;

typedef struct kdn_guide_options {
	uint32_t table_log2;      /* entries a level, log2: 19 for the full grid; 8..22 */
	uint32_t seed;            /* of the initial weights and table */
	float learning_rate;      /* Adam, 1e-2 */
	float region_lo[3];       /* the box positions are encoded over (clamped to it) */
	float region_hi[3];
	uint32_t batch;           /* samples an Adam step (0: 16384) */
	uint32_t max_steps;       /* Adam steps a training frame at most (0: 256) */
	uint32_t sample_capacity; /* training samples a frame keeps (0: 2^24), an even share of its records */
} kdn_guide_options;

kdn_status kdn_guide_open(int device, const kdn_guide_options* options, kdn_guide** out);
kdn_status kdn_guide_close(kdn_guide* guide);
const char* kdn_guide_last_error(void);
/* floats of the weights (14336: W0 64x48, W1 64x64, W2 64x64, W3 48x64, row
 * major, out x in) and of the table (16 << table_log2 entries x 2) */
kdn_status kdn_guide_sizes(const kdn_guide* guide, uint64_t* weights, uint64_t* table);
kdn_status kdn_guide_get_params(kdn_guide* guide, float* weights, float* table);
kdn_status kdn_guide_set_params(kdn_guide* guide, const float* weights, const float* table);
/* samples: n x 10 floats (point, faced normal, direction, weight = the
 * integrand's estimate over the density the direction was drawn with).
 * The loss and its gradients over the n samples, no step taken. */
kdn_status kdn_guide_gradients(kdn_guide* guide, const float* samples, uint32_t n, float* loss, float* dweights, float* dtable);
/* steps Adam steps of batch samples each over the n samples (0 steps: one
 * pass); last_loss: the last step's loss */
kdn_status kdn_guide_train(kdn_guide* guide, const float* samples, uint32_t n, uint32_t batch, uint32_t steps, float* last_loss);
/* rows: n x 6 floats (point, faced normal) -> lobes: n x 40 floats, lobe j
 * at 5j: weight, concentration, mean direction */
kdn_status kdn_guide_query(kdn_guide* guide, const float* rows, uint32_t n, float* lobes);
kdn_status kdn_guide_clear_samples(kdn_guide* guide);
int kdn_guide_ready(const kdn_guide* guide);

/* Frames of ctx use the guide (null: none).  flags: KDN_GUIDE_SAMPLE draws
 * the first kGuideDepth (3) vertices' directions on matte and plastic
 * surfaces from share x guide + (1 - share) x BSDF once the guide is
 * trained; KDN_GUIDE_TRAIN records those vertices and trains the guide on
 * them after each frame.  The guide must live on the context's device and
 * must not be used by two contexts' frames at once. */
#define KDN_GUIDE_SAMPLE 1u
#define KDN_GUIDE_TRAIN 2u
kdn_status kdn_set_guide(kdn_ctx* ctx, kdn_guide* guide, float share, uint32_t flags);
/* Keeps the guide's sampling only where it pays: after one untimed frame
 * of each method, draws pairs of pilot frames plain and guided (the pilot's
 * size, samples and surfaces; seeds seed + 1 ...), measures each method's
 * relative variance of a frame times its device frame time (the frame's
 * CUDA events), and keeps KDN_GUIDE_SAMPLE on ctx only where the guided
 * cost is more than 5% below the plain one; *guided says which.  Pairs are
 * drawn (3 to 16) until the cost ratio lies two standard errors from that
 * margin.  The costs (relative variance x seconds) are written where the
 * pointers are not null.  KDN_BAD_ARG for a pilot of no or too many pixels
 * (2^26), samples (2^20) or surfaces (255). */
kdn_status kdn_guide_select(kdn_ctx* ctx, const kdn_frame* pilot, int* guided, double* plain_cost, double* guided_cost);

#ifdef __cplusplus
}
#endif
#endif
