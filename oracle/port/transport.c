/*
 * Oracle transport: the reference renderer's plain path tracer (Meet + Aim
 * strategies, plugins/transport/paths) restated in C over double precision,
 * on the oracle's octree sphere tracer.  Test infrastructure and the timed
 * CPU baseline (see kdn_port.h).
 *
 * Per sample (plugins/transport/paths/trace.cpp):
 *   startedPathIn (:116)  counter-based numbers keyed by pixel and sample,
 *                         hero wavelengths, the pinhole camera ray;
 *   walkArrived (:1547)   meet the lamps along the leg and the sky past it,
 *                         weighted by the power heuristic (weight.cpp:27);
 *                         camera legs see only the sky (light.cpp:132);
 *   stoodOn (:529)        the leg's absorbing body (absorption.cpp:28);
 *   metGlow (:415)        a surface's glow where the ray arrives from
 *                         outside, whole (the plain sampler aims at no glow);
 *   aimedFrom (:896)      offer every lamp, trace one offer drawn by its lane
 *                         mean (:830 offered); the aim takes the whole weight
 *                         at the surface cap (weight.cpp:107);
 *   scatteredFrom (:1020) the BSDF's own direction, roulette from depth 4
 *                         with survival at most 0.95;
 *   foldPixels (frame.cpp:273) spectral radiance to RGB (colour.cpp:213).
 */
#include "kdn_port.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define PI 3.14159265358979323846
#define BIAS 4e-3
#define NO_MATERIAL 0xFFFFFFFFu

typedef struct v3 {
	double x, y, z;
} v3;

static v3 mk(double x, double y, double z) {
	v3 r = { x, y, z };
	return r;
}
static v3 vd(const double* a) { return mk(a[0], a[1], a[2]); }
static v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 scl(v3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
static double dotv(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 crossv(v3 a, v3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static double len(v3 a) { return sqrt(dotv(a, a)); }
static v3 unit(v3 a) { return scl(a, 1.0 / len(a)); }
static double clampd(double x, double lo, double hi) { return x < lo ? lo : (hi < x ? hi : x); }
static double maxd(double a, double b) { return a < b ? b : a; }
static double mind(double a, double b) { return b < a ? b : a; }

/* math/random.cpp basisAround: any orthonormal frame about n */
typedef struct basis {
	v3 t, b, n;
} basis;

static basis basis_around(v3 n) {
	const double sign = copysign(1.0, n.z);
	const double a = -1.0 / (sign + n.z);
	const double b = n.x * n.y * a;
	basis f;
	f.t = mk(1.0 + sign * n.x * n.x * a, sign * b, -sign * n.x);
	f.b = mk(b, sign + n.y * n.y * a, -n.y);
	f.n = n;
	return f;
}
static v3 to_world(basis f, v3 v) { return add(add(scl(f.t, v.x), scl(f.b, v.y)), scl(f.n, v.z)); }
static v3 to_local(basis f, v3 v) { return mk(dotv(f.t, v), dotv(f.b, v), dotv(f.n, v)); }
static v3 mirrored(v3 v, v3 n) { return sub(scl(n, 2 * dotv(v, n)), v); }

typedef struct lanes {
	double nm[4], density[4], basis[12];
} lanes;

typedef struct spec {
	double v[4];
} spec;

static spec flat(double x) {
	spec s = { { x, x, x, x } };
	return s;
}
static spec smul(spec a, spec b) {
	for (int k = 0; k < 4; ++k) a.v[k] *= b.v[k];
	return a;
}
static spec sscale(spec a, double s) {
	for (int k = 0; k < 4; ++k) a.v[k] *= s;
	return a;
}
static spec sadd(spec a, spec b) {
	for (int k = 0; k < 4; ++k) a.v[k] += b.v[k];
	return a;
}
static double smean(spec a) { return 0.25 * (a.v[0] + a.v[1] + a.v[2] + a.v[3]); }
static double smax(spec a) { return maxd(maxd(a.v[0], a.v[1]), maxd(a.v[2], a.v[3])); }

static spec spectrum(const double rgb[3], const lanes* w) {
	spec s;
	kp_spectrum_of(rgb, w->basis, s.v);
	return s;
}

/* ---- numbers (trace.cpp:47 drawnNumber, path.cpp:22 dimensionOf) ---- */
enum { PIXEL_X, PIXEL_Y, LENS_U, LENS_V, LIGHT_U, LIGHT_V, DIRECTION_U, DIRECTION_V, LOBE, SIDE, SURVIVAL, PICK };

/* sampler.cpp:16 numberAt: hashed, or with the Sobol tables the scrambled
 * Sobol sequence's for the first 28 dimensions (a sample's index and its
 * group are the same at one sample a split) */
static double number(const uint32_t* sobol, uint64_t stream, uint32_t index, int event, int draw) {
	const uint64_t dim = draw < LIGHT_U ? (uint64_t) draw : (uint64_t) (4 + event * 8 + (draw - LIGHT_U));
	if (sobol != NULL && dim < KP_SOBOL_DIMENSIONS) return kp_sobol_number(sobol, stream, index, (uint32_t) dim);
	return kp_hashed(stream, index, dim);
}

/* ---- lamps (light.cpp) ---- */
typedef struct lamp {
	uint32_t kind, square;
	v3 at, along, across, facing, cross, ex, ey, raw;
	double along_len, across_len, area, radius;
	double radiance[3], power[3];
	/* light.cpp:86: the direction normalised; the cosine of a far disc's
	 * half angle; sky_layers.cpp:129: the sine of it */
	v3 direction;
	double cosine, disc_radius;
} lamp;

static lamp lamp_of(const kp_lamp* l) {
	lamp d;
	memset(&d, 0, sizeof d);
	d.kind = l->kind;
	d.at = vd(l->at);
	d.along = vd(l->along);
	d.across = vd(l->across);
	d.cross = crossv(d.along, d.across);
	d.area = len(d.cross);
	d.along_len = len(d.along);
	d.across_len = len(d.across);
	if (d.area > 0) d.facing = unit(d.cross);
	if (d.along_len > 0 && d.across_len > 0) {
		d.ex = scl(d.along, 1 / d.along_len);
		d.ey = scl(d.across, 1 / d.across_len);
		d.raw = crossv(d.ex, d.ey);
	}
	d.square = fabs(dotv(d.along, d.across)) < 1e-9 * d.along_len * d.across_len;
	d.radius = l->radius;
	double k = 1;
	if (l->kind == 3) {
		k = d.area > 0 ? 1 / d.area : 0;
	} else if (l->kind == 2) {
		k = l->radius > 0 ? 1 / (PI * l->radius * l->radius) : 0;
		d.area = 4 * PI * l->radius * l->radius;
	} else if (l->kind == 4 || l->kind == 5) {
		/* light.cpp:37: over pi sin^2 of the half angle */
		const double s = sin(0.5 * l->angle);
		k = 1 / (PI * s * s);
	}
	d.direction = unit(vd(l->direction));
	d.cosine = cos(0.5 * l->angle);
	d.disc_radius = sin(0.5 * l->angle);
	for (int c = 0; c < 3; ++c) {
		d.power[c] = l->power[c];
		d.radiance[c] = l->power[c] * k;
	}
	return d;
}

typedef struct rect {
	v3 x, y, z;
	double z0, x0, x1, y0, y1, b0, b1, k, angle;
} rect;

/* light.cpp:169 rectangleView: a spherical rectangle (Urena et al. 2013) */
static rect rect_view(const lamp* l, v3 origin) {
	rect r;
	const v3 off = sub(l->at, origin);
	r.z = dotv(off, l->raw) > 0 ? scl(l->raw, -1) : l->raw;
	r.x = l->ex;
	r.y = l->ey;
	r.z0 = dotv(off, r.z);
	r.x0 = dotv(off, r.x);
	r.y0 = dotv(off, r.y);
	r.x1 = r.x0 + l->along_len;
	r.y1 = r.y0 + l->across_len;
	const double sides[4] = { r.z0 * r.x1 - r.x0 * r.z0, r.y0 * r.z0 - r.z0 * r.y1, r.z0 * r.x0 - r.x1 * r.z0, r.y1 * r.z0 - r.z0 * r.y0 };
	const double heights[4] = { r.x0 * r.y0 - r.y0 * r.x1, r.x1 * r.y1 - r.y0 * r.x1, r.x1 * r.y1 - r.y1 * r.x0, r.x0 * r.y0 - r.y1 * r.x0 };
	double up[4];
	for (int s = 0; s < 4; ++s) {
		const double size = sqrt(sides[s] * sides[s] + heights[s] * heights[s]);
		up[s] = size > 0 ? heights[s] / size : heights[s];
	}
	const double g0 = acos(clampd(-(up[0] * up[1]), -1, 1));
	const double g1 = acos(clampd(-(up[1] * up[2]), -1, 1));
	const double g2 = acos(clampd(-(up[2] * up[3]), -1, 1));
	const double g3 = acos(clampd(-(up[3] * up[0]), -1, 1));
	r.b0 = up[0];
	r.b1 = up[2];
	r.k = 2 * PI - g2 - g3;
	r.angle = g0 + g1 - r.k;
	return r;
}

static v3 rect_point(const rect* r, v3 origin, double u, double v) {
	const double au = u * r->angle + r->k;
	const double fu = (cos(au) * r->b0 - r->b1) / sin(au);
	const double cu = clampd(copysign(1 / sqrt(fu * fu + r->b0 * r->b0), fu), -1, 1);
	const double xu = clampd(-(cu * r->z0) / sqrt(maxd(1 - cu * cu, 1e-14)), r->x0, r->x1);
	const double d = sqrt(xu * xu + r->z0 * r->z0);
	const double h0 = r->y0 / sqrt(d * d + r->y0 * r->y0);
	const double h1 = r->y1 / sqrt(d * d + r->y1 * r->y1);
	const double hv = h0 + v * (h1 - h0);
	const double hv2 = hv * hv;
	const double yv = hv2 < 1 - 1e-6 ? (hv * d) / sqrt(1 - hv2) : r->y1;
	return add(add(add(origin, scl(r->x, xu)), scl(r->y, yv)), scl(r->z, r->z0));
}

static double cone_density(double c) {
	const double cone = 2 * PI * (1 - c);
	return cone > 1e-12 ? 1 / cone : 0;
}

typedef struct aim {
	int found;
	v3 toward;
	double distance, density;
	double arriving[3];
} aim;

/* light.cpp:372 aimLight for every kind of lamp */
static aim aim_lamp(const lamp* l, v3 from, double u, double v) {
	aim a;
	memset(&a, 0, sizeof a);
	if (l->kind == 0) { /* :349 aimPoint: singular, density 0 */
		const v3 off = sub(l->at, from);
		const double d = len(off);
		if (d < 1e-9) return a;
		a.found = 1;
		a.toward = scl(off, 1 / d);
		a.distance = d;
		for (int c = 0; c < 3; ++c) a.arriving[c] = l->power[c] / (d * d);
		return a;
	}
	if (l->kind == 1) { /* :362 a directional light: singular, from afar */
		a.found = 1;
		a.toward = l->direction;
		a.distance = INFINITY;
		for (int c = 0; c < 3; ++c) a.arriving[c] = l->power[c];
		return a;
	}
	if (l->kind == 4 || l->kind == 5) { /* :334 aimSun: evenly in the disc's cone */
		if (!(l->cosine < 1)) return a;
		const double height = 1 - u * (1 - l->cosine);
		const double ring = sqrt(maxd(1 - height * height, 0));
		const double angle = 2 * PI * v;
		a.found = 1;
		a.toward = to_world(basis_around(l->direction), mk(ring * cos(angle), ring * sin(angle), height));
		a.distance = INFINITY;
		a.density = cone_density(l->cosine);
		for (int c = 0; c < 3; ++c) a.arriving[c] = l->radiance[c] / a.density;
		return a;
	}
	if (l->kind == 3) {
		if (l->area < 1e-12 || dotv(l->facing, sub(from, l->at)) <= 0) return a;
		if (l->square) {
			const rect r = rect_view(l, from);
			if (!(r.angle > 1e-7)) return a;
			const v3 spot = rect_point(&r, from, u, v);
			const v3 off = sub(spot, from);
			const double d = len(off);
			if (d < 1e-9) return a;
			a.found = 1;
			a.toward = scl(off, 1 / d);
			a.distance = d;
			a.density = 1 / r.angle;
			for (int c = 0; c < 3; ++c) a.arriving[c] = l->radiance[c] * r.angle;
			return a;
		}
		const v3 spot = add(add(l->at, scl(l->along, u)), scl(l->across, v));
		const v3 off = sub(spot, from);
		const double d = len(off);
		if (d < 1e-9) return a;
		a.toward = scl(off, 1 / d);
		const double tilt = -dotv(l->facing, a.toward);
		a.found = 1;
		a.distance = d;
		if (tilt <= 0) return a;
		for (int c = 0; c < 3; ++c) a.arriving[c] = l->radiance[c] * (tilt * l->area / (d * d));
		a.density = d * d / (tilt * l->area);
		return a;
	}
	if (l->kind == 2) {
		const v3 off = sub(l->at, from);
		const double d = len(off);
		if (d < 1e-9 || d <= l->radius) return a;
		const v3 axis = scl(off, 1 / d);
		const double side = l->radius / d;
		const double cosine = sqrt(maxd(1 - side * side, 0));
		const double height = 1 - u * (1 - cosine);
		const double ring = sqrt(maxd(1 - height * height, 0));
		const double angle = 2 * PI * v;
		const v3 toward = to_world(basis_around(axis), mk(ring * cos(angle), ring * sin(angle), height));
		const double h = dotv(toward, axis);
		const double r2 = sqrt(maxd(1 - h * h, 0));
		const double reach = d * h - sqrt(maxd(l->radius * l->radius - d * d * r2 * r2, 0));
		a.found = 1;
		a.toward = toward;
		a.distance = maxd(reach, 0);
		for (int c = 0; c < 3; ++c) a.arriving[c] = l->power[c] * (2 * (1 - cosine) / (l->radius * l->radius));
		a.density = cone_density(cosine);
	}
	return a;
}

/* light.cpp:463 aimDensity */
static double aim_density(const lamp* l, v3 from, v3 toward, double distance) {
	if (l->kind == 4 || l->kind == 5) return l->cosine < 1 && dotv(toward, l->direction) >= l->cosine ? cone_density(l->cosine) : 0;
	if (l->kind == 3) {
		if (l->area < 1e-12 || dotv(l->facing, sub(from, l->at)) <= 0) return 0;
		if (l->square) {
			const rect r = rect_view(l, from);
			return r.angle > 1e-7 ? 1 / r.angle : 0;
		}
		const double tilt = -dotv(l->facing, toward);
		if (tilt <= 0 || distance <= 0) return 0;
		return distance * distance / (tilt * l->area);
	}
	if (l->kind == 2) {
		const double away = len(sub(l->at, from));
		if (away <= l->radius || l->radius <= 0) return 0;
		const double side = l->radius / away;
		return cone_density(sqrt(maxd(1 - side * side, 0)));
	}
	return 0;
}

/* sky_layers.cpp:273 moonLit: the share of a moon's disc the first sun
 * lights where a direction meets it, eased; 1 for every other lamp */
static double moon_lit(const lamp* l, const v3* sun, v3 toward) {
	if (l->kind != 5 || sun == NULL) return 1;
	const double along = dotv(toward, l->direction);
	const double aside = maxd(1 - along * along, 0);
	const double reach = along - sqrt(maxd(l->disc_radius * l->disc_radius - aside, 0));
	const v3 normal = scl(sub(scl(toward, reach), l->direction), 1 / l->disc_radius);
	double lit = dotv(normal, *sun) / 0.1 + 0.5;
	lit = lit < 0 ? 0 : (lit > 1 ? 1 : lit);
	return lit * lit * (3 - 2 * lit);
}

/* light.cpp:498 meetLight for a lamp: a point or a directional light is
 * never met, a sun or a moon only by a ray that escaped (:478 meetSun) */
static int meet_lamp(const lamp* l, v3 origin, v3 dir, double limit, double* reach) {
	if (l->kind == 4 || l->kind == 5) {
		*reach = INFINITY;
		return l->cosine < 1 && isinf(limit) && dotv(dir, l->direction) >= l->cosine;
	}
	if (l->kind == 3) {
		const double leaning = dotv(l->cross, dir);
		if (l->area < 1e-12 || leaning >= -1e-12) return 0;
		*reach = dotv(l->cross, sub(l->at, origin)) / leaning;
		if (*reach <= 1e-9 || *reach >= limit) return 0;
		const v3 spot = sub(add(origin, scl(dir, *reach)), l->at);
		const double sq = l->area * l->area;
		const double u = dotv(crossv(spot, l->across), l->cross) / sq;
		const double v = dotv(crossv(l->along, spot), l->cross) / sq;
		return !(u < 0 || u > 1 || v < 0 || v > 1);
	}
	if (l->kind == 2) {
		if (l->radius <= 0) return 0;
		const v3 off = sub(origin, l->at);
		const double along = dotv(off, dir);
		const double under = along * along - (dotv(off, off) - l->radius * l->radius);
		if (under <= 0) return 0;
		const double root = sqrt(under);
		const double first = -along - root;
		*reach = first <= 1e-9 ? -along + root : first;
		return !(*reach <= 1e-9 || *reach >= limit);
	}
	return 0;
}

/* ---- materials (material/material.cpp, microfacet.cpp, energy.cpp) ---- */
static double facet_distribution(double c, double w) {
	if (c <= 0) return 0;
	const double sq = w * w, lo = c * c * (sq - 1) + 1;
	return sq / (PI * lo * lo);
}
static double smith_visibility(double l, double a, double w) {
	const double sq = w * w;
	const double t = a * sqrt(sq + (1 - sq) * l * l) + l * sqrt(sq + (1 - sq) * a * a);
	return t > 0 ? 0.5 / t : 0;
}
static double smith_masking(double c, double w) {
	const double sq = w * w, u = c + sqrt(sq + (1 - sq) * c * c);
	return u > 0 ? 2 * c / u : 0;
}
static v3 halfway(v3 o, v3 i, v3 n) {
	const v3 t = add(o, i);
	const double s = len(t);
	return s > 1e-12 ? scl(t, 1 / s) : n;
}
static double dielectric(double c, double ratio) {
	const double left = 1 - ratio * ratio * (1 - c * c);
	if (left <= 0) return 1;
	const double on = sqrt(left);
	const double pe = (ratio * c - on) / (ratio * c + on);
	const double pa = (ratio * on - c) / (ratio * on + c);
	return 0.5 * (pe * pe + pa * pa);
}
/* ---- thin films (material.cpp:106-172): a layer `thickness` nm deep of
 * index `index` between an outside and a beneath index, the light off its
 * two faces interfering ---- */

/* material.cpp:143 bentCosine: the cosine past a crossing from `before`
 * into `after`, -1 where it reflects totally */
static double bent_cosine(double before, double facing, double after) {
	const double sine = before / after * sqrt(maxd(1 - facing * facing, 0));
	return sine >= 1 ? -1 : sqrt(1 - sine * sine);
}

/* material.cpp:136 airySum */
static double airy_sum(double front, double back, double shift) {
	const double both = front * back;
	const double top = front * front + back * back + 2 * both * shift;
	const double bottom = 1 + both * both + 2 * both * shift;
	return bottom > 0 ? clampd(top / bottom, 0, 1) : 1;
}

/* material.cpp:129 faceAmplitude: the perpendicular [0] and parallel [1]
 * amplitudes of a face from index `before` into `after` */
static void face_amplitude(double before, double after, double facing, double onward, double a[2]) {
	a[0] = (before * facing - after * onward) / (before * facing + after * onward);
	a[1] = (after * facing - before * onward) / (after * facing + before * onward);
}

/* material.cpp:148 filmReflectance at one wavelength */
static double film_reflectance(const double film[2], double facing, double nm, double outside, double beneath) {
	const double inside = bent_cosine(outside, facing, film[1]);
	const double beyond = inside < 0 ? -1 : bent_cosine(film[1], inside, beneath);
	if (inside < 0 || beyond < 0) return 1;
	double near[2], far[2];
	face_amplitude(outside, film[1], facing, inside, near);
	face_amplitude(film[1], beneath, inside, beyond, far);
	const double shift = cos(4 * PI * film[1] * film[0] * inside / nm);
	return 0.5 * (airy_sum(near[0], far[0], shift) + airy_sum(near[1], far[1], shift));
}

/* material.cpp:515 stackedFilm over material.cpp:506 filmOver (air on both sides) */
static double stacked_film(const double film[2], double facing, double nm, double under) {
	if (!(film[0] > 0)) return under;
	const double front = film_reflectance(film, facing, nm, 1, 1);
	const double held = clampd(under, 0, 1);
	const double room = 1 - front * held;
	if (!(room > 1e-9)) return 1;
	return front + (1 - front) * (1 - front) * held / room;
}

/* material.cpp:528 coatFacing */
static double coat_facing(const double film[2], double onto, double nm) {
	if (!(film[0] > 0)) return dielectric(onto, 1 / 1.5);
	return film_reflectance(film, onto, nm, 1, 1.5);
}

static double escape_at(const double* table, double c) {
	const double place = clampd(c, 0, 1) * 32 - 0.5;
	int lower = (int) floor(place);
	lower = lower < 0 ? 0 : (lower > 31 ? 31 : lower);
	const int upper = lower + 1 < 31 ? lower + 1 : 31;
	const double share = clampd(place - lower, 0, 1);
	return table[lower] * (1 - share) + table[upper] * share;
}
static v3 visible_facet(basis f, v3 out, double w, double u, double v) {
	const v3 local = to_local(f, out);
	const v3 st = unit(mk(w * local.x, w * local.y, local.z));
	const double flat = st.x * st.x + st.y * st.y;
	const v3 first = flat > 1e-12 ? scl(mk(-st.y, st.x, 0), 1 / sqrt(flat)) : mk(1, 0, 0);
	const v3 second = crossv(st, first);
	const double reach = sqrt(u), angle = 2 * PI * v;
	const double across = reach * cos(angle);
	const double lean = 0.5 * (1 + st.z);
	const double along = (1 - lean) * sqrt(maxd(1 - across * across, 0)) + lean * reach * sin(angle);
	const double height = sqrt(maxd(1 - across * across - along * along, 0));
	const v3 raised = add(add(scl(first, across), scl(second, along)), scl(st, height));
	return to_world(f, unit(mk(w * raised.x, w * raised.y, maxd(raised.z, 1e-12))));
}

typedef struct shading {
	const kp_material* m;
	v3 normal;
	basis frame;
	spec albedo, twice, within, beyond;
	double rgb[3]; /* the albedo at the hit, blended across a shared seam */
	double leaving, left, share, masking;
	double nm[4]; /* the lanes' wavelengths */
	int parted, inside;
} shading;

static spec lane_indices(const kp_material* m, const lanes* w) {
	spec s;
	for (int k = 0; k < 4; ++k) {
		const double um = w->nm[k] * 1e-3;
		s.v[k] = m->dispersion == 0 ? m->index : m->index + m->dispersion / (um * um);
	}
	return s;
}

static shading shading_of(const kp_material* m, const double* rgb, const kp_material* all, v3 n, v3 out, const lanes* w, uint32_t medium) {
	shading s;
	memset(&s, 0, sizeof s);
	s.m = m;
	s.normal = n;
	s.frame = basis_around(n);
	for (int c = 0; c < 3; ++c) s.rgb[c] = rgb[c];
	s.albedo = spectrum(s.rgb, w);
	s.leaving = dotv(n, out);
	s.within = flat(1);
	s.beyond = flat(1);
	for (int k = 0; k < 4; ++k) s.nm[k] = w->nm[k];
	if (m->kind == 1 || m->kind == 2) {
		s.left = escape_at(m->escape, s.leaving);
		if (m->kind == 2) {
			s.share = m->facet_share;
		} else if (s.leaving > 0) {
			/* material.cpp:440 plasticShare */
			const double face = dielectric(s.leaving, 1 / 1.5);
			s.share = clampd(face / maxd(face + (1 - face) * m->body, 1e-12), 0.25, 0.9);
		}
		s.masking = smith_masking(s.leaving, m->width);
		if (m->kind == 2) {
			/* material.cpp:592 metalTwice over microfacet.cpp:116
			 * averagedFresnel under the film facing straight on */
			double avg[3];
			for (int c = 0; c < 3; ++c) avg[c] = s.rgb[c] + (1 - s.rgb[c]) * (1.0 / 21);
			const spec a = spectrum(avg, w);
			for (int k = 0; k < 4; ++k) {
				const double f = stacked_film(m->film, 1, w->nm[k], a.v[k]);
				s.twice.v[k] = f * f * m->escape_average / (1 - f * (1 - m->escape_average));
			}
		}
	} else if (m->kind == 3) {
		s.inside = medium != NO_MATERIAL;
		if (medium != NO_MATERIAL) {
			s.within = lane_indices(&all[medium], w);
			s.parted = all[medium].dispersion != 0;
		} else {
			s.beyond = lane_indices(m, w);
			s.parted = m->dispersion != 0;
		}
		/* dispersion.cpp:38 filmedSides: a filmed glass answers each lane apart */
		s.parted = s.parted || m->film[0] > 0;
	}
	return s;
}

typedef struct response {
	spec value;
	double density;
} response;

/* ---- rough glass (material.cpp:766-1032, energy.cpp:255-320) ---- */
#define RATIOS 17
#define VIEWS 32
#define DENSEST_RATIO 3.0

typedef struct table_row {
	int lower, upper;
	double share;
} table_row;

/* energy.cpp:255 rowOf: the place of the indices' ratio among the rows */
static table_row row_of(double near, double far) {
	const double ratio = maxd(near, far) / mind(near, far);
	const double place = (mind(ratio, DENSEST_RATIO) - 1) / (DENSEST_RATIO - 1) * (RATIOS - 1);
	int lower = (int) floor(place);
	lower = lower < 0 ? 0 : (lower > RATIOS - 1 ? RATIOS - 1 : lower);
	table_row r;
	r.lower = lower;
	r.upper = lower + 1 < RATIOS - 1 ? lower + 1 : RATIOS - 1;
	r.share = clampd(place - lower, 0, 1);
	return r;
}

static double blended_row(const double* values, table_row r) { return values[r.lower] * (1 - r.share) + values[r.upper] * r.share; }

typedef struct loss {
	double near_average, far_average, back, through, share;
} loss;

/* energy.cpp:284 lossAt */
static loss loss_at(const double* b, double near, double far) {
	const table_row row = row_of(near, far);
	const double rarer = blended_row(b + 2 * RATIOS * VIEWS, row);
	const double denser = blended_row(b + 2 * RATIOS * VIEWS + RATIOS, row);
	const double share = blended_row(b + 2 * RATIOS * VIEWS + 2 * RATIOS, row);
	const int from_rarer = near <= far;
	loss l;
	l.near_average = from_rarer ? rarer : denser;
	l.far_average = from_rarer ? denser : rarer;
	l.back = l.through = l.share = 0;
	const double near_lost = 1 - l.near_average, denser_lost = 1 - denser;
	if (!(near_lost > 1e-9) || !(denser_lost > 1e-9)) return l;
	const double turned = (far / near) * (far / near);
	l.through = from_rarer ? share / denser_lost : share / denser_lost * turned;
	const double given = mind(l.through * (1 - l.far_average), 1.0);
	l.back = (1 - given) / near_lost;
	l.share = given;
	return l;
}

/* energy.cpp:309 rowAt, :317 boundaryAt */
static double row_at(const double* table, int row, double c) {
	const double place = clampd(c, 0, 1) * VIEWS - 0.5;
	int lower = (int) floor(place);
	lower = lower < 0 ? 0 : (lower > VIEWS - 1 ? VIEWS - 1 : lower);
	const int upper = lower + 1 < VIEWS - 1 ? lower + 1 : VIEWS - 1;
	const double share = clampd(place - lower, 0, 1);
	return table[row * VIEWS + lower] * (1 - share) + table[row * VIEWS + upper] * share;
}

static double boundary_at(const double* b, double near, double far, double c) {
	const table_row row = row_of(near, far);
	const double* table = near <= far ? b : b + RATIOS * VIEWS;
	return row_at(table, row.lower, c) * (1 - row.share) + row_at(table, row.upper, c) * row.share;
}

/* material.cpp:780 lossLeft */
static double loss_left(const double* b, double near, double far, double c) { return maxd(1 - boundary_at(b, near, far, c), 0.0); }

typedef struct broad {
	double share, through;
} broad;

/* material.cpp:789 broadOf, over the hero lane's indices */
static broad broad_of(const shading* s, double leaving) {
	broad w = { 0, 0 };
	if (s->m->loses_much) {
		w.share = clampd(loss_left(s->m->boundary, s->within.v[0], s->beyond.v[0], leaving), 0.0, 1.0);
		w.through = loss_at(s->m->boundary, s->within.v[0], s->beyond.v[0]).share;
	}
	return w;
}

/* material.cpp:797 laneReflectance (Fresnel, or the film between the
 * sides at lane k's wavelength), :814 laneReflectances, :821 reflectChance */
static double lane_reflectance(const shading* s, double c, int k) {
	if (!(s->m->film[0] > 0)) return dielectric(c, s->within.v[k] / s->beyond.v[k]);
	return film_reflectance(s->m->film, c, s->nm[k], s->within.v[k], s->beyond.v[k]);
}

static spec lane_reflectances(const shading* s, double c) {
	if (!s->parted) return flat(lane_reflectance(s, c, 0));
	spec r;
	for (int k = 0; k < 4; ++k) r.v[k] = lane_reflectance(s, c, k);
	return r;
}

static double reflect_chance(const shading* s, double c) {
	if (!s->parted) return lane_reflectance(s, c, 0);
	const spec r = lane_reflectances(s, c);
	return 0.25 * (r.v[0] + r.v[1] + r.v[2] + r.v[3]);
}

/* material.cpp:836 reflectanceAcross: seen from the denser side, Fresnel of the arriving cosine */
static double reflectance_across(const shading* s, double leaving, double arriving, int k) {
	const double within = s->within.v[k], beyond = s->beyond.v[k];
	if (within <= beyond) return lane_reflectance(s, leaving, k);
	/* material.cpp:825 filmedFromDenser */
	if (s->m->film[0] > 0) return film_reflectance(s->m->film, arriving, s->nm[k], beyond, within);
	return dielectric(arriving, beyond / within);
}

/* material.cpp:846 backLoss, :850 throughLoss, :859 givenBack */
static spec given_back(const shading* s, double leaving, double arriving, int through) {
	if (!s->m->loses_much) return flat(0);
	const int lanes_n = s->parted ? 4 : 1;
	spec g = flat(0);
	for (int k = 0; k < lanes_n; ++k) {
		const double near = s->within.v[k], far = s->beyond.v[k];
		const loss l = loss_at(s->m->boundary, near, far);
		g.v[k] = through ? l.through * loss_left(s->m->boundary, near, far, leaving) * loss_left(s->m->boundary, far, near, -arriving) / PI
		                 : l.back * loss_left(s->m->boundary, near, far, leaving) * loss_left(s->m->boundary, near, far, arriving) / PI;
	}
	return s->parted ? g : flat(g.v[0]);
}

/* material.cpp:884 glassReflection */
static response glass_reflection(const shading* s, v3 out, v3 in, double leaving, double arriving) {
	const double width = s->m->width;
	const v3 facet = halfway(out, in, s->normal);
	const double onto = dotv(out, facet);
	const spec each = lane_reflectances(s, maxd(onto, 0.0));
	const double lobe = onto > 0 ? facet_distribution(dotv(s->normal, facet), width) : 0;
	const double back = s->parted ? 0.25 * (each.v[0] + each.v[1] + each.v[2] + each.v[3]) : each.v[0];
	const double facets = lobe * smith_masking(leaving, width) / (4 * leaving);
	const broad wide = broad_of(s, leaving);
	response r;
	r.value = sadd(sscale(each, lobe * smith_visibility(leaving, arriving, width)), given_back(s, leaving, arriving, 0));
	r.density = (1 - wide.share) * back * facets + wide.share * (1 - wide.through) * arriving / PI;
	return r;
}

/* material.cpp:947 lanePassage over :925 bentFacet */
static void lane_passage(const shading* s, v3 out, v3 in, double leaving, double arriving, int k, double* sent, double* facets) {
	const double width = s->m->width;
	const double near = s->within.v[k], far = s->beyond.v[k];
	*sent = *facets = 0;
	const v3 sum = add(scl(out, near), scl(in, far));
	const double size = len(sum);
	if (!(size > 1e-12)) return;
	const v3 facet = scl(sum, (dotv(sum, s->normal) < 0 ? -1 : 1) / size);
	const double into = dotv(in, facet);
	if (dotv(out, facet) <= 0 || into >= 0) return;
	const double stretch = far * far * -into / (size * size);
	if (stretch <= 0) return;
	const double onto = dotv(out, facet);
	const double lobe = facet_distribution(dotv(s->normal, facet), width) * onto * stretch;
	const double kept = 1 - reflectance_across(s, onto, -dotv(in, facet), k);
	*sent = kept * lobe * 4 * smith_visibility(leaving, -arriving, width);
	*facets = (1 - reflect_chance(s, onto)) * lobe * smith_masking(leaving, width) / leaving;
}

/* material.cpp:986 glassPassage */
static response glass_passage(const shading* s, v3 out, v3 in, double leaving, double arriving) {
	const int lanes_n = s->parted ? 4 : 1;
	spec sent = flat(0);
	double facets = 0;
	for (int k = 0; k < lanes_n; ++k) {
		double f;
		lane_passage(s, out, in, leaving, arriving, k, &sent.v[k], &f);
		if (k == 0) facets = f;
	}
	const broad wide = broad_of(s, leaving);
	response r;
	r.value = sadd(s->parted ? sent : flat(sent.v[0]), given_back(s, leaving, arriving, 1));
	r.density = (1 - wide.share) * facets + wide.share * wide.through * -arriving / PI;
	return r;
}

static response respond(const shading* s, v3 out, v3 in, const lanes* w) {
	response r;
	r.value = flat(0);
	const kp_material* m = s->m;
	const double arriving = dotv(s->normal, in);
	if (m->kind == 0) {
		r.density = maxd(arriving, 0) / PI;
		if (s->leaving > 0 && arriving > 0) r.value = sscale(s->albedo, 1 / PI);
		return r;
	}
	if (m->kind == 3) {
		/* material.cpp:1002 glassResponse */
		r.density = 0;
		if (s->leaving <= 0 || m->exact) return r;
		return arriving < 0 ? glass_passage(s, out, in, s->leaving, arriving) : glass_reflection(s, out, in, s->leaving, arriving);
	}
	const double cosd = maxd(arriving, 0) / PI;
	if (s->leaving <= 0 || arriving <= 0) {
		r.density = (m->kind == 1 && s->leaving <= 0) ? 0 : (1 - s->share) * cosd;
		return r;
	}
	const v3 h = halfway(out, in, s->normal);
	const double D = facet_distribution(dotv(s->normal, h), m->width);
	const double came = escape_at(m->escape, arriving);
	const double onto_raw = dotv(out, h);
	const double onto = maxd(onto_raw, 0);
	const double facets = D * smith_visibility(s->leaving, arriving, m->width);
	const double room = 1 - m->escape_average;
	const double lost = room <= 1e-6 ? 0 : (1 - s->left) * (1 - came) / (PI * room);
	if (m->kind == 2) {
		/* material.cpp:649 viewedMetal, microfacet.cpp:111 schlickOf */
		const double rest = pow(clampd(1 - onto, 0, 1), 5.0);
		double face[3];
		for (int c = 0; c < 3; ++c) face[c] = s->rgb[c] + (1 - s->rgb[c]) * rest;
		spec lanes_face = spectrum(face, w);
		for (int k = 0; k < 4; ++k) lanes_face.v[k] = stacked_film(m->film, onto, w->nm[k], lanes_face.v[k]);
		r.value = sadd(sscale(lanes_face, facets), sscale(s->twice, lost));
	} else if (!(m->film[0] > 0)) {
		/* material.cpp:661 viewedPlastic */
		const double through = m->coat_room > 1e-6 ? (1 - m->coat_front * s->left) * (1 - m->coat_front * came) / m->coat_room : 0;
		const double coated = dielectric(onto, 1 / 1.5) * facets + m->coat_twice * lost;
		r.value = sadd(sscale(s->albedo, through / PI), flat(coated));
	} else {
		/* material.cpp:661 viewedPlastic under a filmed coat: each lane's
		 * coat (:543 filmCoating, :604 laneCoats) at its wavelength */
		for (int k = 0; k < 4; ++k) {
			const double faced = coat_facing(m->film, 1, w->nm[k]);
			const double front = faced + (1 - faced) / 21;
			const double e = m->escape_average;
			const double twice = front * front * e / (1 - front * (1 - e));
			const double room_k = 1 - front * e;
			const double through = room_k > 1e-6 ? (1 - front * s->left) * (1 - front * came) / room_k : 0;
			r.value.v[k] = s->albedo.v[k] / PI * through + coat_facing(m->film, onto, w->nm[k]) * facets + twice * lost;
		}
	}
	const double fd = onto_raw <= 0 ? 0 : D * s->masking / (4 * s->leaving);
	r.density = s->share * fd + (1 - s->share) * cosd;
	return r;
}

typedef struct scatter {
	int found, through, delta, dispersed;
	v3 incoming;
	spec weight;
	double density;
	uint32_t medium_after;
} scatter;

static scatter sample(const shading* s, v3 out, const lanes* w, double lobe, double side, double u, double v, uint32_t material, uint32_t medium) {
	scatter o;
	memset(&o, 0, sizeof o);
	o.medium_after = NO_MATERIAL;
	const kp_material* m = s->m;
	if (m->kind == 0) {
		const double reach = sqrt(u), angle = 2 * PI * v, height = sqrt(maxd(1 - u, 0));
		o.incoming = to_world(s->frame, mk(reach * cos(angle), reach * sin(angle), height));
		o.density = maxd(dotv(s->normal, o.incoming), 0) / PI;
		o.found = o.density > 0;
		o.weight = s->albedo;
		return o;
	}
	if (m->kind == 1 || m->kind == 2) {
		if (s->leaving <= 0) return o;
		const int facet_lobe = lobe < s->share;
		const v3 facet = visible_facet(s->frame, out, m->width, u, v);
		v3 in;
		if (facet_lobe) {
			in = mirrored(out, facet);
		} else {
			const double reach = sqrt(u), angle = 2 * PI * v, height = sqrt(maxd(1 - u, 0));
			in = to_world(s->frame, mk(reach * cos(angle), reach * sin(angle), height));
		}
		const double arriving = dotv(s->normal, in);
		if ((facet_lobe && dotv(out, facet) <= 0) || arriving <= 0) return o;
		const response r = respond(s, out, in, w);
		if (r.density <= 0) return o;
		o.found = 1;
		o.incoming = in;
		o.density = r.density;
		o.weight = sscale(r.value, fabs(arriving) / r.density);
		return o;
	}
	if (!m->exact) {
		/* material.cpp:1328 glassScatter: the broad lobe (cosine about
		 * either side, :1236 broadChoice) or a visible facet, mirrored or
		 * bent by the hero lane (:1246 facetChoice) */
		const double leaving = s->leaving;
		if (leaving <= 0) return o;
		const broad wide = broad_of(s, leaving);
		int found = 1, reflected;
		v3 in;
		if (lobe < wide.share) {
			reflected = side >= wide.through;
			const basis around = basis_around(reflected ? s->normal : scl(s->normal, -1));
			const double reach = sqrt(u), angle = 2 * PI * v, height = sqrt(maxd(1 - u, 0));
			in = to_world(around, mk(reach * cos(angle), reach * sin(angle), height));
		} else {
			const v3 facet = visible_facet(s->frame, out, m->width, u, v);
			const double onto = dotv(out, facet);
			if (onto <= 0) return o;
			reflected = side < reflect_chance(s, onto);
			if (reflected) {
				in = mirrored(out, facet);
			} else {
				const double ratio = s->within.v[0] / s->beyond.v[0];
				const double leftover = 1 - ratio * ratio * (1 - onto * onto);
				found = leftover > 0;
				in = found ? sub(scl(sub(scl(facet, onto), out), ratio), scl(facet, sqrt(leftover))) : mk(0, 0, 0);
			}
		}
		const double arriving = dotv(s->normal, in);
		if (!found || (reflected ? arriving <= 0 : arriving >= 0)) return o;
		const response r = reflected ? glass_reflection(s, out, in, leaving, arriving) : glass_passage(s, out, in, leaving, arriving);
		if (r.density <= 0) return o;
		o.found = 1;
		o.incoming = in;
		o.density = r.density;
		o.weight = sscale(r.value, fabs(arriving) / r.density);
		o.through = !reflected;
		o.dispersed = o.through && s->parted && s->within.v[0] != s->beyond.v[0];
		o.medium_after = o.through ? (medium != NO_MATERIAL ? NO_MATERIAL : material) : NO_MATERIAL;
		return o;
	}
	/* material.cpp:1300 exactGlassScatter */
	if (s->leaving <= 0) return o;
	double refl[4];
	for (int k = 0; k < 4; ++k) refl[k] = lane_reflectance(s, s->leaving, k);
	if (!s->parted) refl[1] = refl[2] = refl[3] = refl[0];
	const double chance = s->parted ? 0.25 * (refl[0] + refl[1] + refl[2] + refl[3]) : refl[0];
	const double ratio = s->within.v[0] / s->beyond.v[0];
	const double leftover = 1 - ratio * ratio * (1 - s->leaving * s->leaving);
	const int passed = leftover > 0;
	o.found = 1;
	o.delta = 1;
	if (side < chance || !passed) {
		const double c = passed ? chance : 1;
		o.incoming = mirrored(out, s->normal);
		for (int k = 0; k < 4; ++k) o.weight.v[k] = refl[k] / c;
		return o;
	}
	const double c = 1 - chance;
	o.incoming = sub(scl(sub(scl(s->normal, s->leaving), out), ratio), scl(s->normal, sqrt(leftover)));
	for (int k = 0; k < 4; ++k) o.weight.v[k] = (1 - refl[k]) / c;
	o.through = 1;
	o.dispersed = s->parted && s->within.v[0] != s->beyond.v[0];
	o.medium_after = medium != NO_MATERIAL ? NO_MATERIAL : material;
	return o;
}

/* ---- --use sampler=sky_map (plugins/sampler/sky_map/sky_map.cpp): the
 * sky aimed at by a chart of its brightness, 64 rows of equal height by
 * 128 columns of equal turn (the sky's up is +z, so level and aside are +x
 * and +y), a tenth of the draws uniform; uncharted where the lamps outshine
 * it five times over at the region's middle ---- */
#define CHART_ROWS 64
#define CHART_COLUMNS 128
#define CHART_EVEN 0.1
#define CHART_DOUBLES (CHART_ROWS + 1 + CHART_ROWS * (CHART_COLUMNS + 1))

/* light.cpp:582 gradientColour's channel mean at a height */
static double sky_brightness(const kp_view* V, double height) {
	const double* far = height >= 0 ? V->zenith : V->ground;
	const double share = sqrt(fabs(height));
	double mean = 0;
	for (int c = 0; c < 3; ++c) mean += V->horizon[c] * (1 - share) + far[c] * share;
	return maxd(mean / 3, 0.0);
}

/* sky_map.cpp:99 chartedSky; 0 where the sky stays uncharted */
static int sky_chart(const kp_view* V, const kp_lamp* lamps, double* chart) {
	const double row_height = 2.0 / CHART_ROWS;
	double* weights = (double*) malloc(sizeof(double) * CHART_ROWS * CHART_COLUMNS);
	double total = 0;
	for (int row = 0; row < CHART_ROWS; ++row) {
		const double height = -1 + (row + 0.5) * row_height;
		for (int column = 0; column < CHART_COLUMNS; ++column) weights[row * CHART_COLUMNS + column] = sky_brightness(V, height);
	}
	for (int k = 0; k < CHART_ROWS * CHART_COLUMNS; ++k) total += weights[k];
	if (!(total > 0)) {
		free(weights);
		return 0;
	}
	double* rows = chart;
	double* cells = chart + CHART_ROWS + 1;
	rows[0] = 0;
	for (int row = 0; row < CHART_ROWS; ++row) {
		double* run = cells + row * (CHART_COLUMNS + 1);
		run[0] = 0;
		for (int column = 0; column < CHART_COLUMNS; ++column) run[column + 1] = run[column] + weights[row * CHART_COLUMNS + column];
		const double held = run[CHART_COLUMNS];
		for (int column = 1; column <= CHART_COLUMNS; ++column) run[column] = held > 0 ? run[column] / held : (double) column / CHART_COLUMNS;
		rows[row + 1] = rows[row] + held / total;
	}
	rows[CHART_ROWS] = 1;
	free(weights);
	const double brightness = total / (double) (CHART_ROWS * CHART_COLUMNS);
	/* sky_map.cpp:83 lampSent, :94 outshone */
	double lit = 0;
	for (uint32_t k = 0; k < V->lamp_count; ++k) {
		const kp_lamp* l = &lamps[k];
		/* a directional light, a sun or a moon sends its power's mean from afar */
		if (l->kind == 1 || l->kind == 4 || l->kind == 5) {
			lit += maxd((l->power[0] + l->power[1] + l->power[2]) / 3, 0.0);
			continue;
		}
		double apart = 0;
		for (int a = 0; a < 3; ++a) {
			const double place = l->kind == 3 ? l->at[a] + (l->along[a] + l->across[a]) * 0.5 : l->at[a];
			const double d = place - V->middle[a];
			apart += d * d;
		}
		const double mean = maxd((l->power[0] + l->power[1] + l->power[2]) / 3, 0.0);
		const double emitted = (l->kind == 3 ? PI : 4 * PI) * mean;
		lit += emitted / (4 * PI * maxd(apart, 1e-12));
	}
	return !(lit > 5 * 4 * PI * brightness);
}

/* sky_map.cpp:153 chartDensity */
static double chart_density(const double* chart, v3 t) {
	const double row_height = 2.0 / CHART_ROWS, column_width = 2 * PI / CHART_COLUMNS;
	const double height = clampd(t.z, -1.0, 1.0);
	const double angle = atan2(t.y, t.x);
	const double turn = angle < 0 ? angle + 2 * PI : angle;
	size_t row = (size_t) ((height + 1) / row_height), column = (size_t) (turn / column_width);
	if (row > CHART_ROWS - 1) row = CHART_ROWS - 1;
	if (column > CHART_COLUMNS - 1) column = CHART_COLUMNS - 1;
	const double* run = chart + CHART_ROWS + 1 + row * (CHART_COLUMNS + 1);
	const double held = (chart[row + 1] - chart[row]) * (run[column + 1] - run[column]);
	return CHART_EVEN / (4 * PI) + (1 - CHART_EVEN) * held / (row_height * column_width);
}

/* sky_map.cpp:131 foundIn (std::upper_bound over run[1..count]) */
static int chart_found(const double* run, int count, double target) {
	int lo = 0, hi = count;
	while (lo < hi) {
		const int mid = (lo + hi) / 2;
		if (target < run[1 + mid]) hi = mid;
		else lo = mid + 1;
	}
	return lo < count - 1 ? lo : count - 1;
}

/* respondBsdf and sampleBsdf (material.cpp:1076, :1366) at chosen
 * vertices, for the known-answer test against the reference's own: per
 * record ids (material, medium) and 17 doubles (albedo[3], normal[3],
 * outgoing[3], incoming[3], the wavelength share, draw numbers u, v, lobe,
 * side); out per record value[4], density, seen (found, through),
 * incoming[3], weight[4], drawn density. */
void kp_bsdf_answers(const kp_material* materials, uint32_t count, uint32_t n, const uint32_t* ids, const double* d, double* value, double* density,
                     uint32_t* seen, double* incoming, double* weight, double* drawn_density) {
	for (uint32_t i = 0; i < n; ++i) {
		const double* r = d + 17 * (size_t) i;
		const uint32_t material = ids[2 * i] < count ? ids[2 * i] : 0;
		const uint32_t medium = ids[2 * i + 1];
		lanes w;
		kp_sampled_wavelengths(r[12], w.nm, w.density, w.basis);
		const v3 normal = mk(r[3], r[4], r[5]), out = mk(r[6], r[7], r[8]), in = mk(r[9], r[10], r[11]);
		const shading s = shading_of(&materials[material], r, materials, normal, out, &w, medium);
		const response a = respond(&s, out, in, &w);
		for (int k = 0; k < 4; ++k) value[4 * i + k] = a.value.v[k];
		density[i] = a.density;
		const scatter o = sample(&s, out, &w, r[15], r[16], r[13], r[14], material, medium);
		seen[2 * i] = (uint32_t) o.found;
		seen[2 * i + 1] = (uint32_t) o.through;
		incoming[3 * i] = o.incoming.x;
		incoming[3 * i + 1] = o.incoming.y;
		incoming[3 * i + 2] = o.incoming.z;
		for (int k = 0; k < 4; ++k) weight[4 * i + k] = o.weight.v[k];
		drawn_density[i] = o.density;
	}
}

/* ---- the band renderer ---- */
typedef struct job {
	const kp_octree* tree;
	const uint32_t* leaf_material;
	const kp_material* materials;
	lamp lamps[16];
	const kp_view* view;
	int row0, rows, next;
	pthread_mutex_t lock;
	double* sums;
	v3 eye, forward, right, up;
	double reach, aspect;
	uint64_t seed_mix;
	int absorbs; /* absorption.cpp:18 sceneAbsorbs: some glass absorbs */
	const double* placements; /* 12 a leaf, or none */
	const uint32_t* sobol;    /* --use sampler=sobol's tables, or none */
	const double* chart;      /* --use sampler=sky_map's chart, or none (the sky only met) */
	v3 sun;                   /* sdf/scene.cpp:306 firstSun's direction ... */
	const v3* has_sun;        /* ... or none */
	struct air* sky_air;      /* a physical sky lit by the first sun, or none */
	uint32_t sun_lamp;        /* the first sun, whose light the air thins */
	int glows;                /* sky_layers.cpp:164 skyGlows */
	double glow[3], sun_elevation;
	double sun_elevation_any; /* the first sun's elevation, glow or not */
} job;

/* trace.cpp:179 keptOnLeg with absorption.cpp:28 keptThrough: what a leg of
 * `distance` inside `medium` keeps, exp(-absorption x distance) a lane;
 * whole outside any body or where no glass absorbs */
static spec kept_along(const job* J, uint32_t medium, double distance, const lanes* w) {
	if (medium == NO_MATERIAL || !J->absorbs) return flat(1);
	const kp_material* m = &J->materials[medium < J->view->material_count ? medium : 0];
	const spec depth = spectrum(m->absorb, w);
	spec kept;
	for (int k = 0; k < 4; ++k) kept.v[k] = exp(-depth.v[k] * distance);
	return kept;
}

static kp_ray ray_of(v3 o, v3 d, double far, uint32_t medium) {
	kp_ray r;
	r.origin[0] = (float) o.x;
	r.origin[1] = (float) o.y;
	r.origin[2] = (float) o.z;
	r.direction[0] = (float) d.x;
	r.direction[1] = (float) d.y;
	r.direction[2] = (float) d.z;
	r.far = (float) far;
	r.inside = medium != NO_MATERIAL;
	r.within = medium;
	return r;
}

static void sky_colour(const kp_view* view, v3 d, double out[3]) {
	const double h = d.z;
	const double* far = h >= 0 ? view->zenith : view->ground;
	const double share = sqrt(fabs(h));
	for (int c = 0; c < 3; ++c) out[c] = view->horizon[c] * (1 - share) + far[c] * share;
}

/* ---- a physical sky (plugins/feature/atmosphere/atmosphere.cpp) and the
 * glow about the first sun (plugins/feature/sky_layers/sky_layers.cpp:181
 * glowSeen): the air's and the haze's single scattering marched into tables
 * of height, bearing and wavelength (48 x 32 x 33), their phases applied
 * where the sky is met, the ground below the horizon lit by what lands on
 * it, the sun's light thinned by what passes the air ---- */
#define AIR_HEIGHTS 48
#define AIR_BEARINGS 32
#define AIR_COLOURS 33
#define AIR_TABLE (AIR_HEIGHTS * AIR_BEARINGS * AIR_COLOURS)
#define PLANET 6360.0
#define AIR_TOP 6420.0

typedef struct air {
	v3 up, sun, level, aside;
	double* air; /* AIR_TABLE, then the haze's AIR_TABLE */
	double passed[AIR_COLOURS], landing[AIR_COLOURS];
} air;

static double air_wavelength(int colour) { return 380.0 + 320.0 * colour / (double) (AIR_COLOURS - 1); }
static double air_scatter(double nm) { const double r = 440.0 / nm; return 33.1e-3 * r * r * r * r; }
static double haze_scatter(double nm, double haze) { return 0.004 * haze * haze * pow(550.0 / nm, 1.3); }
static double shell_leaving(v3 from, v3 d, double radius) {
	const double along = dotv(from, d);
	return -along + sqrt(maxd(along * along - (dotv(from, from) - radius * radius), 0.0));
}
static int ground_ahead(v3 from, v3 d) {
	const double along = dotv(from, d), under = along * along - (dotv(from, from) - PLANET * PLANET);
	return under >= 0.0 && -along - sqrt(under) > 0.0;
}
static void air_density(v3 at, double* a, double* h) {
	const double height = maxd(len(at) - PLANET, 0.0);
	*a = exp(-height / 8.0);
	*h = exp(-height / 1.2);
}
static void sunward(v3 from, v3 sun, double* a, double* h) {
	const double reach = shell_leaving(from, sun, AIR_TOP);
	*a = *h = 0;
	for (int k = 0; k < 12; ++k) {
		const double n0 = k / 12.0, n1 = (k + 1) / 12.0, mid = (k + 0.5) / 12.0;
		double da, dh;
		air_density(add(from, scl(sun, reach * mid * mid)), &da, &dh);
		*a += da * reach * (n1 * n1 - n0 * n0);
		*h += dh * reach * (n1 * n1 - n0 * n0);
	}
}
static double air_phase(double c) { return 3.0 / (16.0 * PI) * (1.0 + c * c); }
static double haze_phase(double c) {
	const double g = 0.76, g2 = g * g;
	return 3.0 / (8.0 * PI) * (1.0 - g2) * (1.0 + c * c) / ((2.0 + g2) * pow(1.0 + g2 - 2.0 * g * c, 1.5));
}
static double air_lookup(const double* t, double row, double column, double colour) {
	int r = (int) row, b = (int) column, l = (int) colour;
	r = r < AIR_HEIGHTS - 2 ? r : AIR_HEIGHTS - 2;
	b = b < AIR_BEARINGS - 2 ? b : AIR_BEARINGS - 2;
	l = l < AIR_COLOURS - 2 ? l : AIR_COLOURS - 2;
	double sum = 0;
	for (int dr = 0; dr < 2; ++dr)
		for (int db = 0; db < 2; ++db)
			for (int dl = 0; dl < 2; ++dl) {
				double fr = row - r, fb = column - b, fl = colour - l;
				fr = fr < 0 ? 0 : (fr > 1 ? 1 : fr);
				fb = fb < 0 ? 0 : (fb > 1 ? 1 : fb);
				fl = fl < 0 ? 0 : (fl > 1 ? 1 : fl);
				sum += (dr ? fr : 1 - fr) * (db ? fb : 1 - fb) * (dl ? fl : 1 - fl) * t[((r + dr) * AIR_BEARINGS + b + db) * AIR_COLOURS + l + dl];
			}
	return sum;
}
/* atmosphere.cpp:165 airPlaceOf and :222 skyTableAt at a table place */
static double air_sky_at(const air* A, v3 d, double colour) {
	const double rise = dotv(d, A->up) < -1 ? -1 : (dotv(d, A->up) > 1 ? 1 : dotv(d, A->up));
	const double height = asin(rise);
	const double bearing = fabs(atan2(dotv(d, A->aside), dotv(d, A->level)));
	const double row = sqrt(maxd(height, 0.0) / (0.5 * PI)) * (AIR_HEIGHTS - 1), column = bearing / PI * (AIR_BEARINGS - 1);
	const double c = dotv(d, A->sun);
	return air_phase(c) * air_lookup(A->air, row, column, colour) + haze_phase(c) * air_lookup(A->air + AIR_TABLE, row, column, colour);
}
/* atmosphere.cpp:308 atmosphereOf */
static void air_build(air* A, const double sun_direction[3], double haze) {
	A->up = mk(0, 0, 1);
	A->sun = unit(vd(sun_direction));
	const v3 flat_sun = sub(A->sun, scl(A->up, dotv(A->sun, A->up)));
	A->level = len(flat_sun) < 1e-9 ? mk(1, 0, 0) : unit(flat_sun);
	A->aside = crossv(A->up, A->level);
	A->air = (double*) calloc(2 * (size_t) AIR_TABLE, sizeof(double));
	const v3 sun = mk(dotv(A->sun, A->level), dotv(A->sun, A->aside), dotv(A->sun, A->up));
	const v3 eye = mk(0, 0, PLANET + 0.001);
	for (int row = 0; row < AIR_HEIGHTS; ++row) {
		const double along = row / (double) (AIR_HEIGHTS - 1), height = 0.5 * PI * along * along;
		for (int column = 0; column < AIR_BEARINGS; ++column) {
			const double bearing = PI * column / (double) (AIR_BEARINGS - 1);
			const v3 view = mk(cos(height) * cos(bearing), cos(height) * sin(bearing), sin(height));
			double* ta = A->air + (row * AIR_BEARINGS + column) * AIR_COLOURS;
			double* th = ta + AIR_TABLE;
			const double reach = shell_leaving(eye, view, AIR_TOP);
			double seen_a = 0, seen_h = 0;
			for (int k = 0; k < 40; ++k) {
				const double n0 = k / 40.0, n1 = (k + 1) / 40.0, mid = (k + 0.5) / 40.0, span = reach * (n1 * n1 - n0 * n0);
				const v3 at = add(eye, scl(view, reach * mid * mid));
				double da, dh;
				air_density(at, &da, &dh);
				seen_a += da * span * 0.5;
				seen_h += dh * span * 0.5;
				if (!ground_ahead(at, sun)) {
					double la, lh;
					sunward(at, sun, &la, &lh);
					for (int c = 0; c < AIR_COLOURS; ++c) {
						const double nm = air_wavelength(c), scattered = haze_scatter(nm, haze);
						const double thinned = exp(-(air_scatter(nm) * (seen_a + la) + scattered / 0.9 * (seen_h + lh)));
						ta[c] += thinned * da * span * air_scatter(nm);
						th[c] += thinned * dh * span * scattered;
					}
				}
				seen_a += da * span * 0.5;
				seen_h += dh * span * 0.5;
			}
		}
	}
	double sa, sh;
	sunward(eye, sun, &sa, &sh);
	const int set = ground_ahead(eye, sun);
	for (int c = 0; c < AIR_COLOURS; ++c) {
		const double nm = air_wavelength(c);
		A->passed[c] = set ? 0 : exp(-(air_scatter(nm) * sa + haze_scatter(nm, haze) / 0.9 * sh));
		A->landing[c] = 0;
	}
	for (int ring = 0; ring < 32; ++ring) {
		const double rise = (ring + 0.5) / 32, level = sqrt(1 - rise * rise);
		for (int spoke = 0; spoke < 64; ++spoke) {
			const double turn = 2 * PI * (spoke + 0.5) / 64;
			const v3 d = add(add(scl(A->level, level * cos(turn)), scl(A->aside, level * sin(turn))), scl(A->up, rise));
			for (int c = 0; c < AIR_COLOURS; ++c) A->landing[c] += air_sky_at(A, d, c) * rise * (2 * PI / (32 * 64));
		}
	}
	const double overhead = maxd(dotv(A->sun, A->up), 0);
	for (int c = 0; c < AIR_COLOURS; ++c) A->landing[c] += A->passed[c] * overhead;
}
/* math/spectrum.cpp:83 tablePlace, :88 spectrumTableAt */
static double table_place(double nm) {
	double along = (nm - 380.0) / 320.0;
	along = along < 0 ? 0 : (along > 1 ? 1 : along);
	return along * (AIR_COLOURS - 1);
}
static spec table_spectrum(const double* table, const lanes* w) {
	spec s;
	for (int k = 0; k < 4; ++k) {
		const double place = table_place(w->nm[k]);
		const int low = (int) place < AIR_COLOURS - 2 ? (int) place : AIR_COLOURS - 2;
		s.v[k] = table[low] + (table[low + 1] - table[low]) * (place - low);
	}
	return s;
}
/* atmosphere.cpp:312 airSeen */
static spec air_seen(const air* A, const kp_view* V, const double sunlight[3], v3 d, const lanes* w) {
	const spec light = spectrum(sunlight, w);
	const double rise = dotv(d, A->up) < -1 ? -1 : (dotv(d, A->up) > 1 ? 1 : dotv(d, A->up));
	if (asin(rise) < 0) return sscale(smul(smul(spectrum(V->ground, w), table_spectrum(A->landing, w)), light), 1 / PI);
	spec s;
	for (int k = 0; k < 4; ++k) s.v[k] = air_sky_at(A, d, table_place(w->nm[k]));
	return smul(s, light);
}
static double smooth_share(double from, double to, double value) {
	double s = (value - from) / (to - from);
	s = s < 0 ? 0 : (s > 1 ? 1 : s);
	return s * s * (3 - 2 * s);
}

/* sky_layers.cpp:240 starlight: one star a cell of a grid on each cube
 * face, placed, sized and coloured by hashes of its cell's key (:207
 * starDrawsOf), times the night's share (:264 starNight) */
static void starlight(const job* J, v3 d, double out_rgb[3]) {
	const kp_view* V = J->view;
	out_rgb[0] = out_rgb[1] = out_rgb[2] = 0;
	const double ax = fabs(d.x), ay = fabs(d.y), az = fabs(d.z);
	uint64_t face;
	v3 out, right, up;
	if (ax >= ay && ax >= az) {
		const double s = d.x >= 0 ? 1 : -1;
		face = d.x >= 0 ? 0 : 1, out = mk(s, 0, 0), right = mk(0, s, 0), up = mk(0, 0, 1);
	} else if (ay >= az) {
		const double s = d.y >= 0 ? 1 : -1;
		face = d.y >= 0 ? 2 : 3, out = mk(0, s, 0), right = mk(0, 0, s), up = mk(1, 0, 0);
	} else {
		const double s = d.z >= 0 ? 1 : -1;
		face = d.z >= 0 ? 4 : 5, out = mk(0, 0, s), right = mk(s, 0, 0), up = mk(0, 1, 0);
	}
	const double outward = dotv(d, out), u = dotv(d, right) / outward, v = dotv(d, up) / outward;
	int cells = (int) ceil(sqrt(V->star_count / 6.0));
	cells = cells < 1 ? 1 : cells;
	int column = (int) ((u * 0.5 + 0.5) * cells), row = (int) ((v * 0.5 + 0.5) * cells);
	column = column < 0 ? 0 : (column > cells - 1 ? cells - 1 : column);
	row = row < 0 ? 0 : (row > cells - 1 ? cells - 1 : row);
	uint64_t key = (face * 65536u + (uint64_t) row) * 65536u + (uint64_t) column;
	double draw[4];
	for (int k = 0; k < 4; ++k) {
		key = kp_mixed_bits(key + 0x9E3779B97F4A7C15ULL);
		draw[k] = (double) (key >> 11) * 0x1p-53;
	}
	const double across = (column + 0.2 + 0.6 * draw[0]) / cells * 2.0 - 1.0, down = (row + 0.2 + 0.6 * draw[1]) / cells * 2.0 - 1.0;
	const v3 star = unit(add(add(out, scl(right, across)), scl(up, down)));
	if (dotv(d, star) < cos(0.5 * V->star_angle)) return;
	double night = 1;
	if (J->sun_lamp != 0xFFFFFFFFu) night = 1 - smooth_share(-12.0 * PI / 180.0, -2.0 * PI / 180.0, J->sun_elevation_any);
	const double bright = V->star_strength * pow(draw[2], 6.0) * night, w = draw[3];
	out_rgb[0] = (0.75 * (1 - w) + 1.0 * w) * bright;
	out_rgb[1] = (0.85 * (1 - w) + 0.82 * w) * bright;
	out_rgb[2] = (1.0 * (1 - w) + 0.62 * w) * bright;
}

/* feature.cpp:30 skyAt: the gradient, or the air of a physical sky, and the
 * glow about the first sun (sky_layers.cpp:181 glowSeen) */
static spec sky_seen(const job* J, v3 d, const lanes* w) {
	const kp_view* V = J->view;
	spec sky;
	if (J->sky_air != NULL) {
		sky = air_seen(J->sky_air, V, J->lamps[J->sun_lamp].power, d, w);
	} else {
		double rgb[3];
		sky_colour(V, d, rgb);
		sky = spectrum(rgb, w);
	}
	if (J->glows) {
		const double above = smooth_share(-0.02, 0.02, d.z);
		double c = dotv(d, J->sun);
		c = c < -1 ? -1 : (c > 1 ? 1 : c);
		const double fade = smooth_share(-8.0 * PI / 180.0, 0.0, J->sun_elevation);
		const double falling = exp(-acos(c) / maxd(V->spread, 1e-6)) * fade * above;
		const double g[3] = { J->glow[0] * falling, J->glow[1] * falling, J->glow[2] * falling };
		sky = sadd(sky, spectrum(g, w));
	}
	if (V->stars && d.z > 0) {
		double rgb[3];
		starlight(J, d, rgb);
		sky = sadd(sky, spectrum(rgb, w));
	}
	return sky;
}

/* feature.cpp:133 lampTint: the first sun's light thinned by the air */
static spec lamp_tint(const job* J, uint32_t k, const lanes* w) {
	return J->sky_air != NULL && k == J->sun_lamp ? table_spectrum(J->sky_air->passed, w) : flat(1);
}

/* sky_map.cpp:138 chartedDirection, :144 chartAim: a direction from the
 * sky's chart (or a tenth of the time uniformly), its density and the sky's
 * radiance there over it */
static aim aim_sky(const kp_view* V, const double* chart, double u, double v, double part, double jitter_u, double jitter_v) {
	const double row_height = 2.0 / CHART_ROWS, column_width = 2 * PI / CHART_COLUMNS;
	double height, turn;
	if (part < CHART_EVEN) {
		height = 1 - 2 * u;
		turn = 2 * PI * v;
	} else {
		const int row = chart_found(chart, CHART_ROWS, u);
		const int column = chart_found(chart + CHART_ROWS + 1 + row * (CHART_COLUMNS + 1), CHART_COLUMNS, v);
		height = -1 + (row + jitter_u) * row_height;
		turn = (column + jitter_v) * column_width;
	}
	const double across = sqrt(maxd(1 - height * height, 0.0));
	/* sky_map.cpp:30 chartDirection with level +x, aside +y, up +z */
	const v3 toward = unit(add(add(scl(mk(1, 0, 0), across * cos(turn)), scl(mk(0, 1, 0), across * sin(turn))), scl(mk(0, 0, 1), height)));
	aim a;
	a.toward = toward;
	a.distance = INFINITY;
	a.density = chart_density(chart, toward);
	a.found = a.density > 0;
	double sky[3];
	sky_colour(V, toward, sky);
	for (int c = 0; c < 3; ++c) a.arriving[c] = a.found ? sky[c] / a.density : 0;
	return a;
}

/* material.cpp:345 bsdfAt: the leaf's albedo, mixed with the other leaf's by
 * the hit's share where a blend joins two leaves */
static const kp_material* material_in(const kp_material* materials, uint32_t count, const uint32_t* leaf_material, uint32_t leaf) {
	const uint32_t material = leaf != 0xFFFFFFFFu ? leaf_material[leaf] : 0;
	return &materials[material < count ? material : 0];
}

/* material.cpp:281 rampAt: the stops spread evenly over 0..1 */
static void ramp_at(const kp_material* m, double value, double rgb[3]) {
	const uint32_t n = m->stop_count;
	if (n <= 1) {
		for (int c = 0; c < 3; ++c) rgb[c] = m->stops ? m->stops[c] : m->albedo[c];
		return;
	}
	const double place = clampd(value, 0, 1) * (double) (n - 1);
	size_t lower = (size_t) place;
	if (lower > n - 2) lower = n - 2;
	const double share = place - (double) lower;
	for (int c = 0; c < 3; ++c) rgb[c] = m->stops[3 * lower + c] * (1 - share) + m->stops[3 * lower + 3 + c] * share;
}

/* material.cpp:292 placedVector: linear x (v - origin), or linear x v */
static v3 placed(const double* pl, v3 v, int offset) {
	const v3 d = offset ? sub(v, mk(pl[9], pl[10], pl[11])) : v;
	return mk(pl[0] * d.x + pl[1] * d.y + pl[2] * d.z, pl[3] * d.x + pl[4] * d.y + pl[5] * d.z, pl[6] * d.x + pl[7] * d.y + pl[8] * d.z);
}

/* material.cpp:314 albedoAt over :299 patternAt: a flat colour, or the ramp
 * at the pattern's value at the point and normal, in the painted leaf's
 * space unless the pattern is read in world space */
static void colour_at(const kp_material* m, const double* placements, uint32_t leaf, v3 point, v3 normal, double rgb[3]) {
	if (m->pattern.count == 0) {
		for (int c = 0; c < 3; ++c) rgb[c] = m->albedo[c];
		return;
	}
	const int local = !m->world && leaf != 0xFFFFFFFFu && placements != NULL;
	v3 p = point, n = normal;
	if (local) {
		const double* pl = placements + 12 * (size_t) leaf;
		p = placed(pl, point, 1);
		const v3 turned = placed(pl, normal, 0);
		const double size = len(turned);
		n = size > 0 ? scl(turned, 1 / size) : turned;
	}
	const double pt[3] = { p.x, p.y, p.z }, nv[3] = { n.x, n.y, n.z };
	double* regs = (double*) malloc(sizeof(double) * m->pattern.count);
	const double value = kp_eval_inputs(&m->pattern, pt, nv, m->pattern_arguments, regs);
	free(regs);
	ramp_at(m, value, rgb);
}

static void albedo_in(const kp_material* materials, uint32_t count, const uint32_t* leaf_material, const double* placements, const kp_hit* hit,
                      v3 normal, double rgb[3]) {
	const v3 point = mk(hit->point[0], hit->point[1], hit->point[2]);
	colour_at(material_in(materials, count, leaf_material, hit->leaf), placements, hit->leaf, point, normal, rgb);
	if (hit->other != 0xFFFFFFFFu && hit->share > 0) {
		double o[3];
		colour_at(material_in(materials, count, leaf_material, hit->other), placements, hit->other, point, normal, o);
		for (int c = 0; c < 3; ++c) rgb[c] = rgb[c] * (1 - (double) hit->share) + o[c] * (double) hit->share;
	}
}

static const kp_material* material_of_leaf(const job* J, uint32_t leaf) {
	return material_in(J->materials, J->view->material_count, J->leaf_material, leaf);
}

static void albedo_at(const job* J, const kp_hit* hit, v3 normal, double rgb[3]) {
	albedo_in(J->materials, J->view->material_count, J->leaf_material, J->placements, hit, normal, rgb);
}

void kp_albedos(const kp_material* materials, uint32_t material_count, const uint32_t* leaf_material, uint32_t leaf_count, const double* placements,
                uint32_t n, const uint32_t* leaf, const uint32_t* other, const float* share, const double* point, const double* normal, double* rgb) {
	(void) leaf_count;
	for (uint32_t i = 0; i < n; ++i) {
		kp_hit hit;
		memset(&hit, 0, sizeof hit);
		hit.leaf = leaf[i];
		hit.other = other[i];
		hit.share = share[i];
		for (int c = 0; c < 3; ++c) hit.point[c] = (float) point[3 * i + c];
		albedo_in(materials, material_count, leaf_material, placements, &hit, mk(normal[3 * i], normal[3 * i + 1], normal[3 * i + 2]), rgb + 3 * i);
	}
}

static void sample_pixel(job* J, kp_tracer* tracer, int x, int y, uint32_t index, double rgb[3]) {
	const kp_view* V = J->view;
	const uint64_t stream = J->seed_mix ^ kp_mixed_bits(((uint64_t) (uint32_t) x << 32) | (uint64_t) (uint32_t) y);
	lanes w;
	/* core/pixels.cpp:5 groupSample: with a split, the samples of a group
	 * share the first vertex's draws (path.cpp:37 sharedDraw): its
	 * wavelengths, camera ray and aim; the aim there counts once a group in
	 * the weights (weight.cpp:15 sharedAim) and each branch carries it
	 * (the group's sum is the reference's first branch's share times the
	 * split, trace.cpp:1570) */
	const uint32_t split = V->split > 1 ? V->split : 1, group = index / split;
	kp_sampled_wavelengths(kp_wavelength_share(kp_hashed(stream, ~(uint64_t) 0, 0), group), w.nm, w.density, w.basis);
	/* trace.cpp:105 filmDraw, :93 phasedDraw */
	const int factor = V->factor > 1 ? (int) V->factor : 1;
	const double column = factor > 1 ? (double) (V->phase % (uint32_t) factor) : 0, row = factor > 1 ? (double) (V->phase / (uint32_t) factor) : 0;
	const double px = factor > 1 ? x + (column + number(J->sobol, stream, group, 0, PIXEL_X)) / factor : x + number(J->sobol, stream, group, 0, PIXEL_X);
	const double py = factor > 1 ? y + (row + number(J->sobol, stream, group, 0, PIXEL_Y)) / factor : y + number(J->sobol, stream, group, 0, PIXEL_Y);
	const double u = 2 * px / V->width - 1, v = 1 - 2 * py / V->height;
	v3 heading = unit(add(add(J->forward, scl(J->right, u * J->reach * J->aspect)), scl(J->up, v * J->reach)));
	v3 from = J->eye;
	if (V->aperture > 0) {
		/* plugins/transport/paths/camera.cpp:14 cameraRay: from a point of the
		 * lens (math/random.cpp:48 concentricDisc) toward where the pinhole
		 * ray meets the plane in focus */
		const double focus = V->focus > 0 ? V->focus : len(sub(vd(V->target), J->eye));
		const double ahead = focus / maxd(dotv(heading, J->forward), 1e-9);
		const v3 sharp = add(J->eye, scl(heading, ahead));
		const double a = 2 * number(J->sobol, stream, group, 0, LENS_U) - 1, b = 2 * number(J->sobol, stream, group, 0, LENS_V) - 1;
		double du = 0, dv = 0;
		if (a != 0 || b != 0) {
			const int wide = fabs(a) > fabs(b);
			const double radius = wide ? a : b, angle = wide ? PI / 4 * (b / a) : PI / 2 - PI / 4 * (a / b);
			du = radius * cos(angle);
			dv = radius * sin(angle);
		}
		from = add(add(J->eye, scl(J->right, du * V->aperture)), scl(J->up, dv * V->aperture));
		heading = unit(sub(sharp, from));
	}
	kp_ray ray = ray_of(from, heading, INFINITY, NO_MATERIAL);
	spec T = flat(1), R = flat(0);
	double drawn = 0;
	int camera = 1, dispersed = 0, collisions = 0;
	uint32_t medium = NO_MATERIAL;
	for (int depth = 0;; ++depth) {
		kp_hit hit;
		kp_tracer_trace(tracer, &ray, &hit);
		const v3 origin = mk(ray.origin[0], ray.origin[1], ray.origin[2]);
		heading = mk(ray.direction[0], ray.direction[1], ray.direction[2]);
		const int found = hit.kind != 0;
		/* trace.cpp:250 stopOf: a leg inside a scattering body collides where
		 * a free flight -ln(1 - u) / scatter ends before its hit
		 * (scattering.cpp:61 scatteredAlong; u the event's Collision draw,
		 * path.cpp:28 dimensionOf: 2^22 + event) */
		int collided = 0;
		double collided_at = 0, flight = INFINITY;
		if (medium != NO_MATERIAL && J->materials[medium].scatter > 0) {
			flight = -log(1 - kp_hashed(stream, index, ((uint64_t) 1 << 22) + (uint64_t) depth)) / J->materials[medium].scatter;
			if (found && flight < len(sub(mk(hit.point[0], hit.point[1], hit.point[2]), from))) {
				collided = 1;
				collided_at = flight;
			}
		}
		/* trace.cpp:218 keptAlong of the walked leg: a scattering body's
		 * absorption reaches only as far as the drawn flight
		 * (feature.cpp:358 mediumAlong over collisionAlong's `at`) */
#define KEPT(d) kept_along(J, medium, mind((d), flight), &w)
		if (!camera) {
			const double limit = collided ? collided_at : (found ? hit.distance : INFINITY);
			for (uint32_t k = 0; k < V->lamp_count; ++k) {
				double reach;
				if (!meet_lamp(&J->lamps[k], origin, heading, limit, &reach)) continue;
				double wgt = 1;
				if (drawn > 0) {
					const double pa = aim_density(&J->lamps[k], from, heading, reach) / (depth == 1 ? split : 1);
					wgt = drawn * drawn / (drawn * drawn + pa * pa);
				}
				R = sadd(R, sscale(smul(smul(smul(T, KEPT(reach)), spectrum(J->lamps[k].radiance, &w)), lamp_tint(J, k, &w)), wgt * moon_lit(&J->lamps[k], J->has_sun, heading)));
			}
		}
		if (!found) {
			/* the sky met, weighed against aiming at it by its chart
			 * (trace.cpp:294 meetAimDensity, sampler.cpp:344 aimDensityAt) */
			const spec sky = sky_seen(J, heading, &w);
			double wgt = 1;
			if (drawn > 0 && J->chart != NULL) {
				const double pa = chart_density(J->chart, heading) / (depth == 1 ? split : 1);
				wgt = drawn * drawn / (drawn * drawn + pa * pa);
			}
			R = sadd(R, sscale(smul(smul(T, KEPT(INFINITY)), sky), wgt));
			break;
		}
		if (collided) {
			/* trace.cpp:502 collidedOn: the phase vertex at the collision
			 * (:474 phaseVertex), what the body kept up to it; a bending body
			 * is not aimed from (:579 aimsFromCollision), so it only scatters */
			const kp_material* body = &J->materials[medium];
			const v3 point = add(from, scl(heading, collided_at));
			T = smul(T, KEPT(collided_at));
			++collisions;
			/* weight.cpp:23 atDepthCap */
			if (depth + 1 - collisions >= V->surfaces || collisions >= V->collisions) break;
			/* material.cpp:1051 phaseCosine, :1059 phaseScatter */
			const double u = number(J->sobol, stream, index, depth, DIRECTION_U), v = number(J->sobol, stream, index, depth, DIRECTION_V);
			const double g = body->lean;
			double cosine = 1 - 2 * u;
			if (fabs(g) > 1e-3) {
				const double term = (1 - g * g) / (1 - g + 2 * g * u);
				cosine = (1 + g * g - term * term) / (2 * g);
				cosine = cosine < -1 ? -1 : (cosine > 1 ? 1 : cosine);
			}
			const double reach = sqrt(maxd(1 - cosine * cosine, 0)), angle = 2 * PI * v;
			const v3 incoming = to_world(basis_around(heading), mk(reach * cos(angle), reach * sin(angle), cosine));
			spec carried = T;
			if (depth >= 4) {
				const double survival = mind(0.95, smax(carried));
				if (!(number(J->sobol, stream, index, depth, SURVIVAL) < survival)) break;
				carried = sscale(carried, 1 / survival);
			}
			T = carried;
			drawn = 0;
			camera = 0;
			from = point;
			ray = ray_of(point, incoming, INFINITY, medium);
			continue;
		}
		const uint32_t material = hit.leaf != 0xFFFFFFFFu ? J->leaf_material[hit.leaf] : 0;
		const kp_material* m = &J->materials[material < V->material_count ? material : 0];
		const v3 point = mk(hit.point[0], hit.point[1], hit.point[2]);
		v3 normal = mk(hit.normal[0], hit.normal[1], hit.normal[2]);
		/* trace.cpp:529 stoodOn: the leg's body keeps its share */
		T = smul(T, KEPT(sqrt(dotv(sub(point, origin), sub(point, origin)))));
#undef KEPT
		/* trace.cpp:415 metGlow at the vertex: the glow bsdfAt
		 * (material.cpp:345) gives where the ray arrives from outside,
		 * mixed across a blend seam; not aimed at by the plain sampler, so
		 * the meet takes it whole (weight 1) */
		if (dotv(normal, heading) < 0) {
			double glow[3];
			for (int c = 0; c < 3; ++c) glow[c] = m->glow[c];
			if (hit.other != 0xFFFFFFFFu && hit.share > 0) {
				const kp_material* o = material_of_leaf(J, hit.other);
				for (int c = 0; c < 3; ++c) glow[c] = glow[c] * (1 - (double) hit.share) + o->glow[c] * (double) hit.share;
			}
			if (glow[0] > 0 || glow[1] > 0 || glow[2] > 0) R = sadd(R, smul(T, spectrum(glow, &w)));
		}
		if (dotv(normal, heading) >= 0) normal = scl(normal, -1);
		const double lift = BIAS + 2 * 1e-6;
		const int capped = depth + 1 - collisions >= V->surfaces || collisions >= V->collisions;
		const v3 out = scl(heading, -1);
		double rgb[3];
		albedo_at(J, &hit, normal, rgb);
		const shading s = shading_of(m, rgb, J->materials, normal, out, &w, medium);
		/* trace.cpp:583 aimable: from outside every body, or from inside
		 * the glass being crossed where it bends; trace.cpp:590 openSide:
		 * the side the line leaves by */
		const int bends = m->kind == 3 && s.within.v[0] != s.beyond.v[0];
		const int aimable = medium == NO_MATERIAL || (medium == material && bends);
		const v3 open = s.inside ? scl(normal, -1) : normal;
		if (!m->exact && aimable && (V->lamp_count > 0 || J->chart != NULL)) {
			const uint32_t aim_index = depth == 0 ? group : index;
			const double aim_count = depth == 0 ? 1.0 / split : 1.0;
			const double u0 = number(J->sobol, stream, aim_index, depth, LIGHT_U), v0 = number(J->sobol, stream, aim_index, depth, LIGHT_V);
			double choice = number(J->sobol, stream, aim_index, depth, PICK);
			double total = 0, picked = 0, chosen_dist = 0;
			spec chosen = flat(0);
			v3 chosen_dir = mk(0, 0, 1);
			/* the lamps, then a charted sky (sampler.cpp:312 skyAim) with its
			 * own draws past the per-event ones (path.cpp:22 dimensionOf:
			 * AimPart, AimJitterU, AimJitterV at 2^20 + 5 x event + 2, 3, 4) */
			/* sampler.cpp:171 selectLight, each_lamp_first.cpp:7: with
			 * --use sampler=each_lamp_first, at the first vertex each of
			 * the first four lamps whose offer is bright traces a line of
			 * its own, outside the reservoir (trace.cpp:935) */
			uint32_t owned = 0;
			for (uint32_t k = 0; k < V->lamp_count + (J->chart != NULL ? 1u : 0u); ++k) {
				const uint64_t plain = ((uint64_t) 1 << 20) + 5 * (uint64_t) depth;
				aim a = k < V->lamp_count ? aim_lamp(&J->lamps[k], point, u0, v0)
				                                : aim_sky(V, J->chart, u0, v0, kp_hashed(stream, aim_index, plain + 2), kp_hashed(stream, aim_index, plain + 3),
				                                          kp_hashed(stream, aim_index, plain + 4));
				if (!a.found) continue;
				if (k < V->lamp_count) {
					const double lit = moon_lit(&J->lamps[k], J->has_sun, a.toward);
					for (int c = 0; c < 3; ++c) a.arriving[c] *= lit;
				}
				const double facing = dotv(open, a.toward);
				if (facing <= 0 || a.distance <= 0) continue;
				const response f = respond(&s, out, a.toward, &w);
				double wgt = 1;
				if (a.density > 0) {
					const double pm = capped ? 0 : f.density;
					const double pa = a.density * aim_count;
					wgt = pa * pa / (pa * pa + pm * pm);
				}
				const spec arriving = k < V->lamp_count ? smul(spectrum(a.arriving, &w), lamp_tint(J, k, &w)) : spectrum(a.arriving, &w);
				const spec offer = sscale(smul(smul(T, f.value), arriving), facing * wgt);
				const double weight = smean(offer);
				if (!(weight > 0)) continue;
				if (V->each_lamp && depth == 0 && k < V->lamp_count && owned < 4) {
					++owned;
					const kp_ray own = ray_of(add(point, scl(open, lift)), a.toward, a.distance - lift, NO_MATERIAL);
					kp_hit blocked;
					kp_tracer_trace(tracer, &own, &blocked);
					if (blocked.kind == 0) R = sadd(R, offer);
					continue;
				}
				total += weight;
				const double keep = weight / total;
				if (choice < keep) {
					chosen = offer;
					picked = weight;
					chosen_dir = a.toward;
					chosen_dist = a.distance;
					choice = choice / keep;
				} else {
					choice = (choice - keep) / (1 - keep);
				}
			}
			if (picked > 0) {
				const kp_ray line = ray_of(add(point, scl(open, lift)), chosen_dir, chosen_dist - lift, NO_MATERIAL);
				kp_hit blocked;
				kp_tracer_trace(tracer, &line, &blocked);
				if (blocked.kind == 0) R = sadd(R, sscale(chosen, total / picked));
			}
		}
		if (capped) break;
		const scatter sc = sample(&s, out, &w, number(J->sobol, stream, index, depth, LOBE), number(J->sobol, stream, index, depth, SIDE), number(J->sobol, stream, index, depth, DIRECTION_U), number(J->sobol, stream, index, depth, DIRECTION_V), material, medium);
		const double side_of = dotv(sc.incoming, normal);
		const int below = sc.through ? side_of >= 0 : side_of <= 0;
		if (!sc.found || below) break;
		spec carried = smul(T, sc.weight);
		if (sc.dispersed && !dispersed) {
			carried.v[0] *= 4;
			carried.v[1] = carried.v[2] = carried.v[3] = 0;
			dispersed = 1;
		}
		if (depth >= 4) {
			const double survival = mind(0.95, smax(carried));
			if (!(number(J->sobol, stream, index, depth, SURVIVAL) < survival)) break;
			carried = sscale(carried, 1 / survival);
		}
		/* trace.cpp:956 aimedAlong: the next leg's meets are weighed against
		 * aiming where the scatter left by the open side of an aimable vertex */
		const int left_open = sc.through == (medium != NO_MATERIAL);
		const int aimed = !sc.delta && sc.density > 0 && left_open && aimable;
		if (sc.through) medium = sc.medium_after;
		T = carried;
		drawn = aimed ? sc.density : 0;
		camera = 0;
		from = point;
		ray = ray_of(add(point, scl(normal, side_of > 0 ? lift : -lift)), sc.incoming, INFINITY, medium);
	}
	kp_colour_of(w.nm, w.density, R.v, rgb);
}

static void* worker(void* arg) {
	job* J = (job*) arg;
	kp_tracer* tracer = kp_tracer_new(J->tree, J->leaf_material);
	/* work in runs of 16 pixels of a row, so a band of few rows still
	 * spreads over every thread */
	const int runs = (J->view->width + 15) / 16;
	for (;;) {
		pthread_mutex_lock(&J->lock);
		const int item = J->next++;
		pthread_mutex_unlock(&J->lock);
		if (item >= J->rows * runs) break;
		const int row = item / runs;
		const int y = J->row0 + row;
		const int x0 = (item % runs) * 16;
		const int x1 = x0 + 16 < J->view->width ? x0 + 16 : J->view->width;
		for (int x = x0; x < x1; ++x) {
			double sum[3] = { 0, 0, 0 };
			for (int k = 0; k < J->view->spp; ++k) {
				double rgb[3];
				sample_pixel(J, tracer, x, y, (uint32_t) k, rgb);
				for (int c = 0; c < 3; ++c) sum[c] += rgb[c];
			}
			double* out = J->sums + 3 * ((size_t) row * (size_t) J->view->width + (size_t) x);
			for (int c = 0; c < 3; ++c) out[c] = sum[c];
		}
	}
	kp_tracer_free(tracer);
	return NULL;
}

void kp_render_band(const kp_octree* tree, const uint32_t* leaf_material, const kp_material* materials, const kp_lamp* lamps, const kp_view* view,
                    const double* placements, int row0, int rows, int threads, double* sums) {
	job J;
	memset(&J, 0, sizeof J);
	J.tree = tree;
	J.leaf_material = leaf_material;
	J.materials = materials;
	for (uint32_t k = 0; k < view->lamp_count && k < 16; ++k) J.lamps[k] = lamp_of(&lamps[k]);
	J.has_sun = NULL;
	for (uint32_t k = 0; k < view->lamp_count && k < 16; ++k) {
		if (lamps[k].kind == 4) {
			J.sun = J.lamps[k].direction;
			if (len(vd(lamps[k].direction)) > 0) J.has_sun = &J.sun;
			break;
		}
	}
	J.view = view;
	J.row0 = row0;
	J.rows = rows;
	J.sums = sums;
	J.placements = placements;
	pthread_mutex_init(&J.lock, NULL);
	/* core/camera.cpp:9 lensOf */
	J.eye = vd(view->eye);
	J.forward = unit(sub(vd(view->target), J.eye));
	J.right = unit(crossv(J.forward, vd(view->up)));
	J.up = crossv(J.right, J.forward);
	J.reach = tan(view->fov / 2);
	J.aspect = (double) view->width / (double) view->height;
	J.seed_mix = kp_mixed_bits((uint64_t) (int64_t) view->seed);
	for (uint32_t k = 0; k < view->material_count; ++k) {
		const kp_material* m = &materials[k];
		if (m->kind == 3 && (m->absorb[0] > 0 || m->absorb[1] > 0 || m->absorb[2] > 0)) J.absorbs = 1;
	}
	double* chart = NULL;
	if (view->sky_map) {
		chart = (double*) malloc(sizeof(double) * CHART_DOUBLES);
		if (!sky_chart(view, lamps, chart)) {
			free(chart);
			chart = NULL;
		}
	}
	J.chart = chart;
	/* a physical sky lit by the first sun (atmosphere.cpp:308), the glow
	 * about the first sun (sky_layers.cpp:164 skyGlows) */
	air sky_air;
	J.sky_air = NULL;
	J.sun_lamp = 0xFFFFFFFFu;
	J.glows = 0;
	for (uint32_t k = 0; k < view->lamp_count && k < 16; ++k) {
		if (lamps[k].kind != 4) continue;
		J.sun_lamp = k;
		if (view->sky_kind == 1) {
			air_build(&sky_air, lamps[k].direction, view->haze);
			J.sky_air = &sky_air;
		}
		for (int c = 0; c < 3; ++c) J.glow[c] = view->glow[c] * view->strength;
		J.glows = J.glow[0] > 0 || J.glow[1] > 0 || J.glow[2] > 0;
		const v3 s = unit(vd(lamps[k].direction));
		J.sun = s;
		J.sun_elevation = asin(s.z < -1 ? -1 : (s.z > 1 ? 1 : s.z));
		J.sun_elevation_any = J.sun_elevation;
		break;
	}
	uint32_t* sobol = NULL;
	if (view->sobol) {
		sobol = (uint32_t*) malloc(sizeof(uint32_t) * KP_SOBOL_DIMENSIONS * 512);
		kp_sobol_tables(sobol);
	}
	J.sobol = sobol;
	if (threads < 1) threads = 1;
	pthread_t* pool = (pthread_t*) malloc(sizeof(pthread_t) * (size_t) threads);
	for (int t = 0; t < threads; ++t) pthread_create(&pool[t], NULL, worker, &J);
	for (int t = 0; t < threads; ++t) pthread_join(pool[t], NULL);
	free(pool);
	free(sobol);
	free(chart);
	if (J.sky_air != NULL) free(sky_air.air);
	pthread_mutex_destroy(&J.lock);
}
