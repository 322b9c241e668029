/*
 * kdn_port -- the CPU oracle: a plain-C restatement of the reference
 * renderer's algorithms on the hot path, in double precision as the
 * reference computes them.  It is test infrastructure: the parity tests, the
 * smoke check and the CPU baseline of bench.py call it as the checker; no
 * product code links it.
 *
 * Each function cites the reference file:line whose algorithm it restates
 * (paths relative to the reference's source/ folder).
 */
#ifndef KDN_PORT_H
#define KDN_PORT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* sdf/program.h:20 Opcode, in the reference's order. */
enum kp_op {
	KP_CONSTANT, KP_ARGUMENT, KP_POINTX, KP_POINTY, KP_POINTZ, KP_NORMALX, KP_NORMALY, KP_NORMALZ,
	KP_ADD, KP_SUBTRACT, KP_MULTIPLY, KP_DIVIDE, KP_NEGATE, KP_SQRT, KP_ABS, KP_FLOOR, KP_SIN, KP_COS,
	KP_SIGN, KP_ATAN2, KP_POW, KP_MIN, KP_MAX, KP_SMIN, KP_POSSQ, KP_LESS, KP_LESSEQ, KP_EQUAL,
	KP_NOTEQUAL, KP_AND, KP_OR, KP_NOT, KP_SELECT
};

/* sdf/program.h:56 Step, field for field (the reference's is 32 bytes). */
typedef struct kp_step {
	uint8_t opcode;
	uint32_t a, b, c;
	double value;
	uint32_t leaf;
} kp_step;

typedef struct kp_program {
	const kp_step* steps;
	uint32_t count;
	uint32_t result;
} kp_program;

typedef struct kp_interval {
	double lower, upper;
} kp_interval;

typedef struct kp_dual {
	double v, g[3];
} kp_dual;

typedef struct kp_source {
	uint32_t leaf, other;
	double share;
} kp_source;

/* Program evaluation (sdf/program.cpp:57-140). regs holds count values. */
double kp_eval(const kp_program* p, const double pt[3], double* regs);
/* sdf/program.cpp evaluate<double> with every input: the point, the normal
 * and the arguments the program reads (a pattern's) */
double kp_eval_inputs(const kp_program* p, const double pt[3], const double n[3], const double* arguments, double* regs);
kp_interval kp_eval_interval(const kp_program* p, const kp_interval box[3], kp_interval* regs);
kp_dual kp_eval_dual(const kp_program* p, const double pt[3], kp_dual* regs);
/* sdf/program.cpp:505 keptSourceOf over a whole program, given its values. */
kp_source kp_source_of(const kp_program* p, const double* values);

/* ---- interval-cut octree (plugins/geometry/tree/cut.cpp) ---- */
enum kp_occupancy { KP_EMPTY = 0, KP_FILLED = 1, KP_SURFACE = 2 };

typedef struct kp_octree kp_octree;

/*
 * Build the cut octree: from the region's box, cutCell (cut.cpp:463) each
 * cell with its parent's programs and split a surface cell into its eight
 * octants (cut.cpp:519 octantBox) while it is above min_depth, or while its
 * programs hold more than split_steps steps and it is above max_depth.
 */
kp_octree* kp_octree_build(const kp_program* programs, uint32_t count, const double lower[3], const double size[3], int min_depth, int max_depth, uint32_t split_steps);
void kp_octree_free(kp_octree* tree);
uint64_t kp_octree_cells(const kp_octree* tree);
/*
 * Write cell i of the build's pre-order: level, place[3], occupancy, object
 * count; returns the number of objects.  kp_octree_cell_program gives the
 * k-th kept program of that cell.
 */
uint32_t kp_octree_cell(const kp_octree* tree, uint64_t i, uint32_t head[5]);
void kp_octree_cell_program(const kp_octree* tree, uint64_t i, uint32_t k, uint32_t* object, kp_program* program);

/* ---- geometry: hits (plugins/geometry/sphere_trace/sphere_trace.cpp) ---- */
typedef struct kp_ray {
	float origin[3], direction[3], far;
	uint32_t inside;
	uint32_t within;
} kp_ray;

typedef struct kp_hit {
	uint32_t kind; /* 0 missed, 1 surface (core/batch.h:88 HitKind) */
	float distance;
	float point[3];
	float normal[3];
	uint32_t leaf, other;
	float share;
	uint32_t object;
	uint32_t steps;
} kp_hit;

/* sphereTraced (sphere_trace.cpp:216) over every object, in double. */
void kp_sphere_trace(const kp_program* programs, uint32_t count, const uint32_t* leaf_material, const double lower[3], const double size[3], const kp_ray* rays, uint32_t n, kp_hit* hits);
/* The same march with a stopping rule: 0 the reference's tolerance, 1 the
 * FP32 device march's 2e-6 max(1, |p|_inf / 4) (a sensitivity check of the
 * reference's answer: which rays move when the tolerance does). */
void kp_sphere_trace_rule(const kp_program* programs, uint32_t count, const uint32_t* leaf_material, const double lower[3], const double size[3], const kp_ray* rays, uint32_t n, kp_hit* hits, int rule);
/* The same march with each step's field read from the cut programs of the
 * octree cell the point lies in, and empty cells skipped to their exit. */
void kp_octree_trace(const kp_octree* tree, const uint32_t* leaf_material, const kp_ray* rays, uint32_t n, kp_hit* hits);
/* sphere_trace.cpp:140 sphereNormal of one program at p(t) along a ray, and
 * the length of the program's gradient there (a hit's normal anywhere along
 * the stretch its stopping tolerance admits). */
void kp_normal_at(const kp_program* program, const kp_ray* ray, double t, double normal[3], double* gradient_length);

/* One tracer per thread: the same march, one ray at a time. */
typedef struct kp_tracer kp_tracer;
kp_tracer* kp_tracer_new(const kp_octree* tree, const uint32_t* leaf_material);
void kp_tracer_trace(kp_tracer* t, const kp_ray* ray, kp_hit* hit);
void kp_tracer_free(kp_tracer* t);

/* ---- transport (plugins/transport/paths) ---- */
/* A material as the transport draws it: the Material's kind and albedo and
 * the Finish derived from it (material.cpp:204 finishWith). */
typedef struct kp_material {
	uint32_t kind, exact;
	double albedo[3];
	double index, dispersion, width, facet_share, body;
	double coat_front, coat_twice, coat_room, escape_average;
	double escape[32];
	double glow[3];   /* material.cpp:325 glowOf: the glow colour times its strength */
	double absorb[3]; /* absorption.cpp:28 keptThrough: the body's absorption a unit length */
	/* sdf/scene.h Albedo: a ramp over a pattern program (pattern.count 0:
	 * the flat albedo above), its arguments, stops (3 a stop) and space */
	kp_program pattern;
	const double* pattern_arguments;
	const double* stops;
	uint32_t stop_count;
	uint32_t world;
	/* a rough glass (material.cpp:1002 glassResponse): whether it gives back
	 * what single scattering loses, and its material/energy.h Boundary (17 x
	 * 32 rarer, 17 x 32 denser, 17 rarer averages, 17 denser averages, 17
	 * rarer-through shares) */
	uint32_t loses_much;
	const double* boundary;
	/* material.cpp:106 filmOf: the thin film a metal, plastic or glass
	 * wears, thickness in nanometres (0: none) and index */
	double film[2];
	/* scattering.cpp:7 scatters: a glass whose body turns aside `scatter`
	 * a unit of travel (0: none), by Henyey-Greenstein's phase of g = lean */
	double scatter, lean;
} kp_material;

/* A lamp (light.cpp:78 lampOf): kind 0 point, 1 directional, 2 sphere,
 * 3 quad, 4 sun, 5 moon; direction toward a directional light, a sun or a
 * moon; angle across a sun's or a moon's disc, radians. */
typedef struct kp_lamp {
	uint32_t kind, square;
	double at[3], along[3], across[3], power[3], radius;
	double direction[3], angle;
} kp_lamp;

typedef struct kp_view {
	double eye[3], target[3], up[3], fov;
	double zenith[3], horizon[3], ground[3];
	int32_t width, height, spp, surfaces, seed;
	uint32_t lamp_count, material_count;
	/* core/camera.h:65 FilmPlan: width x height is the drawn frame; with a
	 * factor above 1 each pixel's samples aim at the shown pixel of the
	 * phase (plugins/transport/paths/trace.cpp:93 phasedDraw) */
	uint32_t factor, phase;
	/* 1: --use sampler=sobol */
	uint32_t sobol;
	/* 1: --use sampler=sky_map, charted against the lamps at `middle`, the
	 * middle of the scene's region */
	uint32_t sky_map;
	/* 1: --use sampler=each_lamp_first: at the first vertex each of the
	 * first four lamps that offer light traces a line of its own */
	uint32_t each_lamp;
	double middle[3];
	/* render.collisions: the most collisions a path stands on */
	int32_t collisions;
	/* sdf/scene.h Sky: its kind (0 gradient, 1 physical), a physical sky's
	 * haze (its ground albedo in `ground`), the glow about the first sun
	 * (colour, strength, spread) */
	uint32_t sky_kind;
	double haze, glow[3], strength, spread;
	/* core/camera.cpp:9 lensOf: a thin lens's radius (0: a pinhole) and
	 * the distance it is sharp at (0: the target's) */
	double aperture, focus;
	/* render.split: samples sharing a first vertex (1: none) */
	uint32_t split;
	/* sdf/scene.h Stars: present, count, strength, angle */
	uint32_t stars;
	double star_count, star_strength, star_angle;
} kp_view;

/*
 * Draw rows [row0, row0 + rows) of a frame, spp samples a pixel, on
 * `threads` threads: the reference's plain path transport
 * (trace.cpp:116 startedPathIn, :1547 walkArrived, :896 aimedFrom, :1020
 * scatteredFrom, frame.cpp:273 foldPixels) in double.  sums gets the summed
 * RGB of each pixel of the band (3 doubles a pixel).
 */
void kp_render_band(const kp_octree* tree, const uint32_t* leaf_material, const kp_material* materials, const kp_lamp* lamps, const kp_view* view,
                    const double* placements, int row0, int rows, int threads, double* sums);

/* material.cpp:345 bsdfAt's albedo for n hits (leaf, other, share, point,
 * the normal facing the ray): the leaf's material's colour or ramp over its
 * pattern, mixed with the other leaf's across a blend seam.  placements: 12
 * doubles a leaf (sdf/scene.h Placement: linear row by row, origin). */
/* respondBsdf and sampleBsdf at chosen vertices (transport.c, the
 * known-answer test against the reference's own) */
void kp_bsdf_answers(const kp_material* materials, uint32_t count, uint32_t n, const uint32_t* ids, const double* d, double* value, double* density,
                     uint32_t* seen, double* incoming, double* weight, double* drawn_density);

void kp_albedos(const kp_material* materials, uint32_t material_count, const uint32_t* leaf_material, uint32_t leaf_count, const double* placements,
                uint32_t n, const uint32_t* leaf, const uint32_t* other, const float* share, const double* point, const double* normal, double* rgb);

/* ---- denoiser (plugins/reconstruction/atrous/atrous.cpp:513 denoisedFrame) ----
 * lens: eye[3], forward[3], right[3], up[3], reach, aspect.  Per pixel:
 * colour[3], moment, length, distance, normal[3], leaf, albedo[3] (the
 * reference's TemporalPixel); out: RGB. */
void kp_denoise(int width, int height, int demodulated, const double lens[14], const double* colour, const double* moment, const float* length,
                const float* distance, const double* normal, const uint32_t* leaf, const double* albedo, float* out);

/* ---- the temporal member (plugins/reconstruction/temporal/temporal.cpp) ---- */
/* One frame of temporalFrame (:1001) at a film factor of 1 with a G-buffer
 * (the demodulated grid: what the reference runs before the a-trous
 * denoiser).  lens now / before: eye[3], forward[3], right[3], up[3], reach,
 * aspect.  Per pixel: light[3] (the record's), first (the record's first
 * surface of the pixel's last sample) and centre (the G-buffer's) as
 * kp_surface, before (the state before, ignored when kept is 0); out: the
 * state after and the image, RGB. */
typedef struct kp_surface {
	float distance;
	float normal[3];
	uint32_t leaf;
	float albedo[3];
} kp_surface;

typedef struct kp_tpixel {
	double colour[3];
	double moment;
	float length;
	float distance;
	double normal[3];
	uint32_t leaf;
	double albedo[3];
} kp_tpixel;

void kp_temporal(int width, int height, int moved, int recounted, int kept, const int film[4], const double lens_now[14], const double lens_before[14], const double* light,
                 const kp_surface* first, const kp_surface* centre, const kp_tpixel* before, kp_tpixel* after, float* image);

/* ---- numbers, wavelengths and colour (math/random.cpp, math/colour.cpp) ---- */
/* The upscale member (upscale.c; plugins/reconstruction/upscale/upscale.cpp
 * upscaledFrame) for one frame at a film factor above 1: width, height the
 * shown size; internal the drawn frame (RGB float, drawn size); distance the
 * G-buffer's distances at the drawn size or NULL; kept: the state before is
 * read; settling: the frame settles after movement (alpha 1). */
void kp_upscale(int width, int height, int factor, int phase, int moved, int kept, int settling, const double lens_now[14], const double lens_before[14],
                const float* internal, const float* distance, const double* before_colour, const float* before_depth, double* colour, float* depth,
                float* image);

/* The upsample member (upscale.c; plugins/reconstruction/upsample/
 * upsample.cpp upsampledImage): the drawn frame bilinearly to the shown
 * size width x height at a film factor. */
void kp_upsample(int width, int height, int factor, const float* drawn, float* shown);

/* --use sampler=sobol (spectral.c; plugins/sampler/sobol/sobol.cpp): the
 * byte tables of the 28 Sobol dimensions (28 x 512 words) and the number of
 * a dimension below 28 of a pixel stream's sample. */
#define KP_SOBOL_DIMENSIONS 28
#define KP_SOBOL_SHARED 6
void kp_sobol_tables(uint32_t* out);
double kp_sobol_number(const uint32_t* tables, uint64_t stream, uint32_t index, uint32_t dimension);

uint64_t kp_mixed_bits(uint64_t v);
double kp_unit_of(uint64_t bits);
double kp_hashed(uint64_t stream, uint64_t index, uint64_t coordinate);
/* basis: the red, green and blue upsampling curves at the four lanes */
void kp_sampled_wavelengths(double u, double nanometres[4], double density[4], double basis[12]);
double kp_wavelength_share(double start, uint32_t index);
void kp_spectrum_of(const double rgb[3], const double basis[12], double out[4]);
void kp_colour_of(const double nanometres[4], const double density[4], const double spectrum[4], double rgb[3]);

#ifdef __cplusplus
}
#endif
#endif
