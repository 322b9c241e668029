/*
 * Oracle temporal member: plugins/reconstruction/temporal/temporal.cpp
 * restated in C over double, for a film factor of 1 with a G-buffer (the
 * grid the reference runs before the a-trous denoiser: every drawn pixel is
 * a shown pixel, its light divided by its first surface's albedo).  Test
 * infrastructure (see kdn_port.h).
 *
 *   temporalFrame (:1001)     per pixel: the 3x3 neighbourhood of this
 *                             frame's light (:903 neighbourhoodOf), the
 *                             history (:605 historyFor: the pixel's own on a
 *                             still camera, else reprojected through the
 *                             G-buffer's plane, :584 surfacedHistory), and
 *                             the blend (:796 freshBlend, :836 heldBlend).
 */
#include "kdn_port.h"

#include <math.h>
#include <stddef.h>
#include <string.h>

#define NO_LEAF 0xFFFFFFFFu

/* temporal.cpp:16-24 */
static const double MOVING_CAP = 32, STILL_CAP = 256, YOUNG_LENGTH = 8;
static const double MOVING_SPREAD = 1.25, STILL_SPREAD = 6;
static const double DEPTH_SHARE = 0.03, NORMAL_COSINE = 0.9, ALBEDO_FLOOR = 1e-3;

typedef struct vec {
	double x, y, z;
} vec;

static vec mk(double x, double y, double z) {
	vec r = { x, y, z };
	return r;
}
static vec add(vec a, vec b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static vec sub(vec a, vec b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static vec scl(vec a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
static double dot(vec a, vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static double len(vec a) { return sqrt(dot(a, a)); }

/* :307 temporalCamera */
typedef struct camera {
	vec eye, forward, corner, across, down, across_inverse, down_inverse;
	double width, height;
} camera;

static camera camera_of(const double* l, int width, int height) {
	camera c;
	const vec eye = mk(l[0], l[1], l[2]), forward = mk(l[3], l[4], l[5]), right = mk(l[6], l[7], l[8]), up = mk(l[9], l[10], l[11]);
	const double reach = l[12], sideways = l[12] * l[13];
	c.eye = eye;
	c.forward = forward;
	c.across = scl(right, 2 * sideways / (double) width);
	c.down = scl(up, -2 * reach / (double) height);
	c.corner = add(sub(forward, scl(right, sideways)), scl(up, reach));
	c.across_inverse = scl(c.across, 1 / dot(c.across, c.across));
	c.down_inverse = scl(c.down, 1 / dot(c.down, c.down));
	c.width = width;
	c.height = height;
	return c;
}

static vec film_heading(const camera* c, double x, double y) { return add(add(c->corner, scl(c->across, x)), scl(c->down, y)); }

typedef struct plane {
	uint32_t leaf;
	vec point, normal;
	double reach;
} plane;

static plane sky_plane(void) {
	plane p;
	memset(&p, 0, sizeof p);
	p.leaf = NO_LEAF;
	return p;
}

static int sky_surface(const kp_surface* s) { return s->leaf == NO_LEAF || !isfinite(s->distance); }

/* :358 planeThrough */
static plane plane_through(const kp_surface* s, vec eye, vec heading) {
	if (sky_surface(s)) return sky_plane();
	plane p;
	p.leaf = s->leaf;
	p.point = add(eye, scl(heading, (double) s->distance / len(heading)));
	p.normal = mk(s->normal[0], s->normal[1], s->normal[2]);
	p.reach = DEPTH_SHARE * (double) s->distance;
	return p;
}

static int same_leaf(uint32_t a, uint32_t b, int recounted) { return recounted ? ((a == NO_LEAF) == (b == NO_LEAF)) : a == b; }

/* :397 onPlane */
static int on_plane(const plane* p, const plane* other, int recounted) {
	if (!same_leaf(other->leaf, p->leaf, recounted)) return 0;
	if (p->leaf == NO_LEAF) return 1;
	if (dot(other->normal, p->normal) < NORMAL_COSINE) return 0;
	return fabs(dot(sub(other->point, p->point), p->normal)) <= p->reach;
}

/* :208 lightingDivisor, :224 sampleLight */
static double divisor(double albedo) { return albedo < ALBEDO_FLOOR ? 1 : albedo; }

static void sample_light(const double* light, const kp_surface* first, size_t k, double out[3]) {
	for (int c = 0; c < 3; ++c) out[c] = light[3 * k + c] / divisor((double) first[k].albedo[c]);
}

static double luminance(const double c[3]) { return 0.2126 * c[0] + 0.7152 * c[1] + 0.0722 * c[2]; }

/* :870 sampleSum, :882 joinedSums */
typedef struct tsum {
	double sum[3], squares[3];
	size_t closest;
	double nearest, farthest;
} tsum;

static tsum sample_sum(const double* light, const kp_surface* first, size_t k) {
	tsum s;
	double c[3];
	sample_light(light, first, k, c);
	for (int i = 0; i < 3; ++i) {
		s.sum[i] = c[i];
		s.squares[i] = c[i] * c[i];
	}
	s.closest = k;
	s.nearest = (double) first[k].distance;
	s.farthest = isfinite(s.nearest) ? s.nearest : 0;
	return s;
}

static tsum joined(tsum a, tsum b) {
	tsum r;
	const int closer = b.nearest < a.nearest;
	for (int i = 0; i < 3; ++i) {
		r.sum[i] = a.sum[i] + b.sum[i];
		r.squares[i] = a.squares[i] + b.squares[i];
	}
	r.closest = closer ? b.closest : a.closest;
	r.nearest = closer ? b.nearest : a.nearest;
	r.farthest = a.farthest < b.farthest ? b.farthest : a.farthest;
	return r;
}

typedef struct near {
	double mean[3], deviation[3];
	size_t closest;
	double spread;
} near;

static size_t clamped(int x, int y, int w, int h) {
	x = x < 0 ? 0 : (x > w - 1 ? w - 1 : x);
	y = y < 0 ? 0 : (y > h - 1 ? h - 1 : y);
	return (size_t) y * (size_t) w + (size_t) x;
}

/* :893 columnSum, :912 rowNeighbourhoods, :903 neighbourhoodOf */
static tsum column_sum(const double* light, const kp_surface* first, int x, int y, int w, int h) {
	const tsum middle = joined(sample_sum(light, first, clamped(x, y, w, h)), sample_sum(light, first, clamped(x, y - 1, w, h)));
	return joined(middle, sample_sum(light, first, clamped(x, y + 1, w, h)));
}

static near neighbourhood(const double* light, const kp_surface* first, int x, int y, int w, int h) {
	const tsum centre = column_sum(light, first, x, y, w, h);
	const tsum left = column_sum(light, first, x - 1 < 0 ? 0 : x - 1, y, w, h);
	const tsum right = column_sum(light, first, x + 1 > w - 1 ? w - 1 : x + 1, y, w, h);
	const tsum all = joined(joined(centre, left), right);
	near n;
	for (int c = 0; c < 3; ++c) {
		n.mean[c] = all.sum[c] * (1.0 / 9);
		const double mean = all.sum[c] / 9;
		const double var = all.squares[c] / 9 - mean * mean;
		n.deviation[c] = sqrt(var > 0 ? var : 0);
	}
	n.closest = all.closest;
	n.spread = isfinite(all.nearest) ? all.farthest - all.nearest : 0;
	return n;
}

typedef struct history {
	int found;
	double colour[3], moment;
	float length;
	double albedo[3];
} history;

/* :410 placeBefore */
static int place_before(const camera* before, vec along, double* x, double* y) {
	const double ahead = dot(along, before->forward);
	if (!(ahead > 0)) return 0;
	const double scale = 1 / ahead;
	*x = dot(along, before->across_inverse) * scale + 0.5 * before->width;
	*y = dot(along, before->down_inverse) * scale + 0.5 * before->height;
	return *x >= 0 && *x < before->width && *y >= 0 && *y < before->height;
}

/* core/camera.cpp:51 filmCentre of this frame's film and of the state
 * before's (temporal.cpp:187 temporalCentre): where in a grid pixel its
 * G-buffer ray passes */
typedef struct centres {
	double now_x, now_y, before_x, before_y;
} centres;

/* :378 lastPlane */
static plane last_plane(const camera* before, const centres* c, const kp_tpixel* last, int x, int y) {
	const vec heading = film_heading(before, x + c->before_x, y + c->before_y);
	if (last->leaf == NO_LEAF || !isfinite(last->distance)) return sky_plane();
	plane p;
	p.leaf = last->leaf;
	p.point = add(before->eye, scl(heading, (double) last->distance / len(heading)));
	p.normal = mk(last->normal[0], last->normal[1], last->normal[2]);
	p.reach = 0;
	return p;
}

/* :584 surfacedHistory with :495 fetchedHistory (bilinear taps over the
 * pixels before whose surface lies on this pixel's plane) */
static history surfaced_history(const camera* now, const camera* before, const centres* c, const kp_tpixel* last, const kp_surface* centre, int x, int y,
                                int w, int h, int recounted) {
	history out;
	memset(&out, 0, sizeof out);
	const vec heading = film_heading(now, x + c->now_x, y + c->now_y);
	const plane p = plane_through(&centre[(size_t) y * (size_t) w + (size_t) x], now->eye, heading);
	const vec along = p.leaf == NO_LEAF ? heading : sub(p.point, before->eye);
	double px, py;
	if (!place_before(before, along, &px, &py)) return out;
	const double ax = px - c->before_x, ay = py - c->before_y;
	const int lx = (int) floor(ax), ly = (int) floor(ay);
	const double tx = ax - lx, ty = ay - ly;
	double sum[3] = { 0, 0, 0 }, albedo[3] = { 0, 0, 0 }, moment = 0, weight = 0;
	float length = 0;
	for (int j = 0; j < 2; ++j) {
		for (int i = 0; i < 2; ++i) {
			const int cx = lx + i, cy = ly + j;
			const double wt = (i == 0 ? 1 - tx : tx) * (j == 0 ? 1 - ty : ty);
			if (!(wt > 0 && cx >= 0 && cx < w && cy >= 0 && cy < h)) continue;
			const kp_tpixel* l = &last[(size_t) cy * (size_t) w + (size_t) cx];
			const plane lp = last_plane(before, c, l, cx, cy);
			if (!(l->length > 0 && on_plane(&p, &lp, recounted))) continue;
			for (int c = 0; c < 3; ++c) {
				sum[c] += l->colour[c] * wt;
				albedo[c] += l->albedo[c] * wt;
			}
			moment += l->moment * wt;
			length += (float) ((double) l->length * wt);
			weight += wt;
		}
	}
	if (!(weight > 0)) return out;
	out.found = 1;
	for (int c = 0; c < 3; ++c) {
		out.colour[c] = sum[c] * (1 / weight);
		out.albedo[c] = albedo[c] * (1 / weight);
	}
	out.moment = moment / weight;
	out.length = (float) ((double) length / weight);
	return out;
}

/* :711 fillShare against a sample's plane along its pixel centre */
static int sample_on_plane(const plane* p, const camera* now, const centres* c, const kp_surface* first, size_t k, int w) {
	const int x = (int) (k % (size_t) w), y = (int) (k / (size_t) w);
	const plane sp = plane_through(&first[k], now->eye, film_heading(now, x + c->now_x, y + c->now_y));
	return on_plane(p, &sp, 0);
}

/* :754 jointFilled: the pixel's own light if its sample lies on the
 * G-buffer's plane, else those of the 3x3 that do, else its own */
static void joint_filled(const camera* now, const centres* c, const double* light, const kp_surface* first, const kp_surface* centre, int x, int y, int w,
                         int h, double out[3]) {
	const size_t k = (size_t) y * (size_t) w + (size_t) x;
	const plane p = plane_through(&centre[k], now->eye, film_heading(now, x + c->now_x, y + c->now_y));
	if (sample_on_plane(&p, now, c, first, k, w)) {
		sample_light(light, first, k, out);
		return;
	}
	double sum[3] = { 0, 0, 0 }, weight = 0;
	for (int dy = -1; dy <= 1; ++dy) {
		for (int dx = -1; dx <= 1; ++dx) {
			const size_t j = clamped(x + dx, y + dy, w, h);
			if (!sample_on_plane(&p, now, c, first, j, w)) continue;
			double c[3];
			sample_light(light, first, j, c);
			for (int i = 0; i < 3; ++i) sum[i] += c[i];
			weight += 1;
		}
	}
	if (weight > 0) {
		for (int i = 0; i < 3; ++i) out[i] = sum[i] * (1 / weight);
		return;
	}
	sample_light(light, first, k, out);
}

void kp_temporal(int width, int height, int moved, int recounted, int kept, const int film[4], const double lens_now[14], const double lens_before[14],
                 const double* light, const kp_surface* first, const kp_surface* centre, const kp_tpixel* before, kp_tpixel* after, float* image) {
	const camera now = camera_of(lens_now, width, height);
	const camera prev = camera_of(lens_before, width, height);
	/* core/camera.cpp:51 filmCentre: film = factor, phase now; factor, phase before */
	const int fn = film[0] > 1 ? film[0] : 1, fb = film[2] > 1 ? film[2] : 1;
	const centres cs = { ((fn > 1 ? film[1] % fn : 0) + 0.5) / fn, ((fn > 1 ? film[1] / fn : 0) + 0.5) / fn, ((fb > 1 ? film[3] % fb : 0) + 0.5) / fb,
		                 ((fb > 1 ? film[3] / fb : 0) + 0.5) / fb };
	const double cap = moved ? MOVING_CAP : STILL_CAP;
	for (int y = 0; y < height; ++y) {
		for (int x = 0; x < width; ++x) {
			const size_t k = (size_t) y * (size_t) width + (size_t) x;
			const near nb = neighbourhood(light, first, x, y, width, height);
			/* :244 aimedSurface: the sample's first surface is the G-buffer's */
			const uint32_t sampled = sky_surface(&first[k]) ? NO_LEAF : first[k].leaf;
			const uint32_t shown = sky_surface(&centre[k]) ? NO_LEAF : centre[k].leaf;
			const int aimed = sampled == shown;
			history hist;
			memset(&hist, 0, sizeof hist);
			if (kept) {
				if (!moved) {
					const kp_tpixel* l = &before[k];
					if (l->length > 0) {
						hist.found = 1;
						memcpy(hist.colour, l->colour, sizeof hist.colour);
						hist.moment = l->moment;
						hist.length = l->length;
						memcpy(hist.albedo, l->albedo, sizeof hist.albedo);
					}
				} else {
					hist = surfaced_history(&now, &prev, &cs, before, centre, x, y, width, height, recounted);
				}
			}
			double colour[3], moment;
			float length;
			if (!hist.found) {
				/* :796 freshBlend */
				if (aimed) sample_light(light, first, k, colour);
				else joint_filled(&now, &cs, light, first, centre, x, y, width, height, colour);
				const double l = luminance(colour);
				moment = l * l;
				length = aimed ? 1.0f : 0.0f;
			} else {
				/* :836 heldBlend with :810 heldColour (clamped to the neighbourhood while young or moving) */
				const float held_length = (float) ((double) hist.length < cap ? (double) hist.length : cap);
				double held[3];
				if (!moved && !((double) hist.length < YOUNG_LENGTH)) {
					memcpy(held, hist.colour, sizeof held);
				} else {
					const double spread = moved ? MOVING_SPREAD : STILL_SPREAD;
					for (int c = 0; c < 3; ++c) {
						const double reach = spread * nb.deviation[c];
						const double lo = nb.mean[c] - reach, hi = nb.mean[c] + reach;
						held[c] = hist.colour[c] < lo ? lo : (hist.colour[c] > hi ? hi : hist.colour[c]);
					}
				}
				if (!aimed) {
					memcpy(colour, held, sizeof colour);
					moment = hist.moment;
					length = held_length;
				} else {
					double sample[3];
					sample_light(light, first, k, sample);
					const double l = luminance(sample);
					const double base = 1.0 / ((double) held_length + 1);
					const double alpha = base > 1.0 / cap ? base : 1.0 / cap;
					for (int c = 0; c < 3; ++c) colour[c] = held[c] * (1 - alpha) + sample[c] * alpha;
					moment = hist.moment * (1 - alpha) + l * l * alpha;
					length = (float) (held_length + 1.0f < cap ? held_length + 1.0f : cap);
				}
			}
			/* :865 surfacedPixel: what the pixel shows is the G-buffer's */
			kp_tpixel* o = &after[k];
			memcpy(o->colour, colour, sizeof colour);
			o->moment = moment;
			o->length = length;
			o->distance = centre[k].distance;
			o->leaf = centre[k].leaf;
			for (int c = 0; c < 3; ++c) {
				o->normal[c] = centre[k].normal[c];
				o->albedo[c] = centre[k].albedo[c];
				/* :220 shownLight */
				image[3 * k + c] = (float) (colour[c] * divisor(o->albedo[c]));
			}
		}
	}
}
