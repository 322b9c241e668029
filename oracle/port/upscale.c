/*
 * The oracle's upscale member: plugins/reconstruction/upscale/upscale.cpp
 * upscaledFrame restated in C for one frame at a film factor above 1, with
 * the reference's own number types (tones in float, positions, lenses and
 * the history's colours in double) so that it answers as the reference does
 * to the bit.  Test infrastructure: only tests/ and the benchmark's CPU leg
 * run it.
 *
 * Each shown pixel gathers the drawn frame's 3x3 samples around it twice: a
 * sharp gather (Gaussian weights, exp(-8 d^2) in shown pixels, :575) and a
 * Catmull-Rom fill (:244 catmullRom), in a luma / orange / green tone
 * (:179 toneOf, tone-mapped by 1 / (1 + max)); the history is the frame
 * before's shown pixels where this pixel's nearest surface was seen
 * (:357 seenFrom), read by a five-tap Catmull-Rom over bilinear taps
 * (:453 historyAt), kept where the depth there matches (:418 sameDepth),
 * clamped to the 3x3 box's mean and deviation (:481 clampedHistory) and
 * blended toward the sharp gather (:497 blendedTone).
 */
#include "kdn_port.h"

#include <float.h>
#include <math.h>
#include <stddef.h>
#include <stdlib.h>

/* upscale.cpp:17-34 */
#define CEILING 60000.0f
#define FLOOR_ 1e-4f
#define SHARP 8.0
#define ALPHA 0.5f
#define ALPHA_SETTLE 1.0f
#define ALPHA_FAST 1.0f
#define ALPHA_LEAST 1e-5f
#define ALPHA_MOVING 0.15f
#define FAST 8.0
#define CLAMP_MOVING 1.25f
#define CLAMP_STILL 6.0f
#define STILL 1.0
#define STILL_MARGIN 1.0f
#define DEPTH_SHARE 0.03f
#define SPREAD_SHARE 0.25f
#define LEAST_WEIGHT 1e-6f

typedef struct tone {
	float l, o, g;
} tone;

static tone t_add(tone a, tone b) { return (tone) { a.l + b.l, a.o + b.o, a.g + b.g }; }
static tone t_sub(tone a, tone b) { return (tone) { a.l - b.l, a.o - b.o, a.g - b.g }; }
static tone t_mul(tone a, float s) { return (tone) { a.l * s, a.o * s, a.g * s }; }
static float minf_(float a, float b) { return b < a ? b : a; }
static float maxf_(float a, float b) { return a < b ? b : a; }
static tone t_min(tone a, tone b) { return (tone) { minf_(a.l, b.l), minf_(a.o, b.o), minf_(a.g, b.g) }; }
static tone t_max(tone a, tone b) { return (tone) { maxf_(a.l, b.l), maxf_(a.o, b.o), maxf_(a.g, b.g) }; }
static tone t_sq(tone a) { return (tone) { a.l * a.l, a.o * a.o, a.g * a.g }; }
static tone t_root(tone a) { return (tone) { sqrtf(maxf_(a.l, 0.0f)), sqrtf(maxf_(a.o, 0.0f)), sqrtf(maxf_(a.g, 0.0f)) }; }
static tone t_clamp(tone a, tone lo, tone hi) { return t_min(t_max(a, lo), hi); }
static tone t_mix(tone a, tone b, float s) { return t_add(a, t_mul(t_sub(b, a), s)); }
static tone t_spread(tone a, float s) { return (tone) { a.l + s, a.o + s, a.g + s }; }

/* :179 toneOf */
static tone tone_of(double red_, double green_, double blue_) {
	const float red = minf_((float) red_, CEILING);
	const float green = minf_((float) green_, CEILING);
	const float blue = minf_((float) blue_, CEILING);
	const float scale = 1 / (1 + maxf_(red, maxf_(green, blue)));
	const float r = red * scale, g = green * scale, b = blue * scale;
	return (tone) { 0.25f * r + 0.5f * g + 0.25f * b, 0.5f * r - 0.5f * b, -0.25f * r + 0.5f * g - 0.25f * b };
}

/* :190 untonedColour */
static void untoned(tone t, double out[3]) {
	const float r = maxf_(t.l + t.o - t.g, 0.0f);
	const float g = maxf_(t.l + t.g, 0.0f);
	const float b = maxf_(t.l - t.o - t.g, 0.0f);
	const float scale = 1 / maxf_(1 - maxf_(r, maxf_(g, b)), FLOOR_);
	out[0] = (double) (r * scale);
	out[1] = (double) (g * scale);
	out[2] = (double) (b * scale);
}

/* :244 catmullRom */
static double catmull_rom(double t) {
	const double a = fabs(t);
	if (a < 1) return (1.5 * a - 2.5) * a * a + 1;
	if (a < 2) return ((-0.5 * a + 2.5) * a - 4) * a + 2;
	return 0;
}

typedef struct sample {
	tone t;
	float depth;
} sample;

typedef struct stats {
	tone mean, deviation, least, most;
	float closest, farthest;
} stats;

typedef struct axis {
	int taps[3];
	float sharp[3], fill[3];
	int toward, box;
} axis;

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (hi < v ? hi : v); }

/* :267 upscaleGridSample, :273 upscaleStatsAt */
static stats stats_at(const sample* s, int w, int h, int x, int y) {
	stats st;
	st.mean = (tone) { 0, 0, 0 };
	st.deviation = (tone) { 0, 0, 0 };
	st.least = (tone) { FLT_MAX, FLT_MAX, FLT_MAX };
	st.most = (tone) { -FLT_MAX, -FLT_MAX, -FLT_MAX };
	st.closest = INFINITY;
	st.farthest = 0;
	tone squares = { 0, 0, 0 };
	for (int dy = -1; dy <= 1; ++dy) {
		for (int dx = -1; dx <= 1; ++dx) {
			const sample* p = &s[(size_t) clampi(y + dy, 0, h - 1) * (size_t) w + (size_t) clampi(x + dx, 0, w - 1)];
			st.mean = t_add(st.mean, p->t);
			squares = t_add(squares, t_sq(p->t));
			st.least = t_min(st.least, p->t);
			st.most = t_max(st.most, p->t);
			st.closest = minf_(st.closest, p->depth);
			if (p->depth < INFINITY) st.farthest = maxf_(st.farthest, p->depth);
		}
	}
	st.mean = t_mul(st.mean, 1.0f / 9);
	st.deviation = t_root(t_sub(t_mul(squares, 1.0f / 9), t_sq(st.mean)));
	return st;
}

/* :564 towardSpot, :568 upscaleAxis */
static axis axis_of(int factor, double jitter, int count, int shown) {
	const double internal = ((double) shown + 0.5) / (double) factor;
	const int nearest = (int) floor(internal - jitter);
	const double first = (double) nearest + 0.5 + jitter - internal;
	axis a;
	for (int d = 0; d < 3; ++d) {
		const int at = clampi(nearest + d - 1, 0, count - 1);
		const double offset = ((double) at + 0.5 + jitter - internal) * (double) factor;
		a.taps[d] = at;
		a.sharp[d] = (float) exp(-SHARP * offset * offset);
		a.fill[d] = (float) catmull_rom(first + (double) (d - 1));
	}
	const double centre = (double) a.taps[1] + 0.5 + jitter - internal;
	const int toward = centre > 0 ? -1 : (centre < 0 ? 1 : 0);
	a.toward = clampi(a.taps[1] + toward, 0, count - 1);
	a.box = nearest + 1;
	return a;
}

typedef struct lens {
	double eye[3], forward[3], right[3], up[3], reach, aspect;
	int width, height;
} lens;

static lens lens_of(const double v[14], int w, int h) {
	lens l;
	for (int k = 0; k < 3; ++k) {
		l.eye[k] = v[k];
		l.forward[k] = v[3 + k];
		l.right[k] = v[6 + k];
		l.up[k] = v[9 + k];
	}
	l.reach = v[12];
	l.aspect = v[13];
	l.width = w;
	l.height = h;
	return l;
}

static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* :342 upscaleHeading */
static void heading_of(const lens* l, double x, double y, double out[3]) {
	const double u = 2 * x / (double) l->width - 1;
	const double v = 1 - 2 * y / (double) l->height;
	for (int k = 0; k < 3; ++k) out[k] = l->forward[k] + l->right[k] * (u * l->reach * l->aspect) + l->up[k] * (v * l->reach);
	const double size = sqrt(dot3(out, out));
	if (size > 0) {
		for (int k = 0; k < 3; ++k) out[k] = out[k] / size;
	}
}

typedef struct seen {
	int inside;
	double x, y;
	float depth;
} seen;

/* :357 seenFrom */
static seen seen_from(const lens* before, const double along[3], float depth) {
	seen s = { 0, 0, 0, 0 };
	const double ahead = dot3(along, before->forward);
	if (!(ahead > 1e-9)) return s;
	const double u = dot3(along, before->right) / (ahead * before->reach * before->aspect);
	const double v = dot3(along, before->up) / (ahead * before->reach);
	const double x = (u + 1) * 0.5 * (double) before->width;
	const double y = (1 - v) * 0.5 * (double) before->height;
	if (!(x >= 0 && x < (double) before->width && y >= 0 && y < (double) before->height)) return s;
	s.inside = 1;
	s.x = x;
	s.y = y;
	s.depth = depth;
	return s;
}

typedef struct history {
	const double* colour; /* x3 */
	const float* depth;
	int w, h;
} history;

static size_t hpix(const history* hs, int x, int y) { return (size_t) clampi(y, 0, hs->h - 1) * (size_t) hs->w + (size_t) clampi(x, 0, hs->w - 1); }

/* :409 depthMatches, :416 sameDepth */
static int depth_matches(float last, float depth, float slack) {
	if (!(depth < INFINITY)) return !(last < INFINITY);
	return fabsf(last - depth) <= DEPTH_SHARE * depth + slack;
}

static int same_depth(const history* hs, const seen* s, float slack) {
	const int x = (int) floor(s->x - 0.5), y = (int) floor(s->y - 0.5);
	for (int dy = 0; dy <= 1; ++dy) {
		for (int dx = 0; dx <= 1; ++dx) {
			if (depth_matches(hs->depth[hpix(hs, x + dx, y + dy)], s->depth, slack)) return 1;
		}
	}
	return 0;
}

/* :428 historyShare, :432 historyIndex, :436 historyAcross, :442 historyDown, :448 bilinearHistory */
static double h_share(double at) { return at - 0.5 - floor(at - 0.5); }
static int h_index(double at) { return (int) floor(at - 0.5); }

static void h_across(const history* hs, double x, int y, double out[3]) {
	const double share = h_share(x);
	const int column = h_index(x);
	const double* a = hs->colour + 3 * hpix(hs, column, y);
	const double* b = hs->colour + 3 * hpix(hs, column + 1, y);
	for (int c = 0; c < 3; ++c) out[c] = a[c] * (1 - share) + b[c] * share;
}

static void h_down(const history* hs, int x, double y, double out[3]) {
	const double share = h_share(y);
	const int row = h_index(y);
	const double* a = hs->colour + 3 * hpix(hs, x, row);
	const double* b = hs->colour + 3 * hpix(hs, x, row + 1);
	for (int c = 0; c < 3; ++c) out[c] = a[c] * (1 - share) + b[c] * share;
}

static void h_bilinear(const history* hs, double x, double y, double out[3]) {
	const double share = h_share(y);
	const int row = h_index(y);
	double a[3], b[3];
	h_across(hs, x, row, a);
	h_across(hs, x, row + 1, b);
	for (int c = 0; c < 3; ++c) out[c] = a[c] * (1 - share) + b[c] * share;
}

typedef struct taps {
	int before;
	double middle;
	int after;
	double middle_weight, before_weight, after_weight;
} taps;

/* :460 upscaleTaps */
static taps taps_at(double at) {
	const double centre = floor(at - 0.5) + 0.5;
	const double f = at - centre;
	const double w0 = f * (-0.5 + f * (1 - 0.5 * f));
	const double w1 = 1 + f * f * (-2.5 + 1.5 * f);
	const double w2 = f * (0.5 + f * (2 - 1.5 * f));
	const double w3 = f * f * (-0.5 + 0.5 * f);
	taps t;
	t.before = (int) (centre - 1.5);
	t.middle = centre + w2 / (w1 + w2);
	t.after = (int) (centre + 1.5);
	t.middle_weight = w1 + w2;
	t.before_weight = w0;
	t.after_weight = w3;
	return t;
}

/* :476 historyAt */
static void history_at(const history* hs, const seen* s, double out[3]) {
	const taps across = taps_at(s->x), down = taps_at(s->y);
	double top[3], left[3], middle[3], right[3], bottom[3];
	h_across(hs, across.middle, down.before, top);
	h_down(hs, across.before, down.middle, left);
	h_bilinear(hs, across.middle, down.middle, middle);
	h_down(hs, across.after, down.middle, right);
	h_across(hs, across.middle, down.after, bottom);
	const double wt = across.middle_weight * down.before_weight, wl = across.before_weight * down.middle_weight;
	const double wm = across.middle_weight * down.middle_weight, wr = across.after_weight * down.middle_weight;
	const double wb = across.middle_weight * down.after_weight;
	const double ends = down.before_weight + down.middle_weight + down.after_weight;
	const double total = across.middle_weight * ends + down.middle_weight * (across.before_weight + across.after_weight);
	for (int c = 0; c < 3; ++c) {
		const double sum = (top[c] * wt + left[c] * wl + middle[c] * wm + right[c] * wr + bottom[c] * wb) * (1 / total);
		out[c] = sum < 0.0 ? 0.0 : sum;
	}
}

void kp_upscale(int width, int height, int factor, int phase, int moved, int kept, int settling, const double lens_now[14], const double lens_before[14],
                const float* internal, const float* distance, const double* before_colour, const float* before_depth, double* colour, float* depth,
                float* image) {
	const int dw = width / factor, dh = height / factor;
	const size_t drawn = (size_t) dw * (size_t) dh;
	/* :224 upscaleSamples: the tones and the G-buffer's depth (sky where
	 * no G-buffer is given or the distance is not finite) */
	sample* samples = (sample*) malloc(sizeof(sample) * drawn);
	for (size_t k = 0; k < drawn; ++k) {
		samples[k].t = tone_of((double) internal[3 * k], (double) internal[3 * k + 1], (double) internal[3 * k + 2]);
		samples[k].depth = distance != NULL && isfinite(distance[k]) ? distance[k] : INFINITY;
	}
	/* :665 upscaleJitter */
	const double jx = ((double) (phase % factor) + 0.5) / (double) factor - 0.5;
	const double jy = ((double) (phase / factor) + 0.5) / (double) factor - 0.5;
	const lens now = lens_of(lens_now, width, height), prev = lens_of(lens_before, width, height);
	const history hs = { before_colour, before_depth, width, height };
	for (int y = 0; y < height; ++y) {
		const axis row = axis_of(factor, jy, dh, y);
		for (int x = 0; x < width; ++x) {
			const axis column = axis_of(factor, jx, dw, x);
			/* :313 upscaleBoxAt: the 3x3 box around the nearest sample */
			const stats st = stats_at(samples, dw, dh, column.box - 1, row.box - 1);
			/* :317 upscaleGather */
			tone sharp = { 0, 0, 0 }, fill = { 0, 0, 0 };
			float sharp_weight = 0, fill_weight = 0;
			for (int dy = 0; dy < 3; ++dy) {
				for (int dx = 0; dx < 3; ++dx) {
					const tone t = samples[(size_t) row.taps[dy] * (size_t) dw + (size_t) column.taps[dx]].t;
					const float near = column.sharp[dx] * row.sharp[dy];
					const float spread = column.fill[dx] * row.fill[dy];
					sharp = t_add(sharp, t_mul(t, near));
					fill = t_add(fill, t_mul(t, spread));
					sharp_weight += near;
					fill_weight += spread;
				}
			}
			fill = t_clamp(t_mul(fill, 1 / fill_weight), st.least, st.most);
			/* :515 upscaledTone */
			tone out = fill;
			if (kept) {
				double direction[3];
				heading_of(&now, (double) x + 0.5, (double) y + 0.5, direction);
				seen s;
				if (!(st.closest < INFINITY)) {
					s = seen_from(&prev, direction, INFINITY);
				} else {
					double along[3];
					for (int k = 0; k < 3; ++k) along[k] = now.eye[k] + direction[k] * (double) st.closest - prev.eye[k];
					s = seen_from(&prev, along, (float) sqrt(dot3(along, along)));
				}
				/* :511 upscaleSlack */
				const float slack = minf_(st.farthest - st.closest, SPREAD_SHARE * st.closest);
				if (s.inside && same_depth(&hs, &s, slack)) {
					/* :497 blendedTone */
					const double mx = s.x - ((double) x + 0.5), my = s.y - ((double) y + 0.5);
					const double moved_by = sqrt(mx * mx + my * my);
					double hc[3];
					history_at(&hs, &s, hc);
					const tone history_tone = tone_of(hc[0], hc[1], hc[2]);
					const float motion = (float) (moved_by / STILL < 1.0 ? moved_by / STILL : 1.0);
					/* :481 clampedHistory */
					const float spread = CLAMP_STILL + (CLAMP_MOVING - CLAMP_STILL) * motion;
					const float margin = STILL_MARGIN * (1 - motion);
					const tone low = t_spread(t_sub(st.mean, t_mul(st.deviation, spread)), -margin);
					const tone high = t_spread(t_add(st.mean, t_mul(st.deviation, spread)), margin);
					tone last;
					if (!(motion > 0)) {
						last = t_clamp(history_tone, low, high);
					} else {
						/* :469 nearestBox */
						const int bx = column.taps[1], by = row.taps[1];
						const tone a = samples[(size_t) by * (size_t) dw + (size_t) bx].t;
						const tone b = samples[(size_t) by * (size_t) dw + (size_t) column.toward].t;
						const tone c = samples[(size_t) row.toward * (size_t) dw + (size_t) bx].t;
						const tone e = samples[(size_t) row.toward * (size_t) dw + (size_t) column.toward].t;
						const tone least = t_min(t_min(a, b), t_min(c, e));
						const tone most = t_max(t_max(a, b), t_max(c, e));
						const tone tight_low = t_mix(low, t_max(low, least), motion);
						const tone tight_high = t_mix(high, t_min(high, most), motion);
						last = t_clamp(history_tone, tight_low, tight_high);
					}
					const float speed = (float) (moved_by / FAST < 1.0 ? moved_by / FAST : 1.0);
					const float base = settling ? ALPHA_SETTLE : ALPHA;
					float alpha = (base + (ALPHA_FAST - base) * speed) * sharp_weight;
					alpha = alpha < ALPHA_LEAST ? ALPHA_LEAST : (alpha > 1.0f ? 1.0f : alpha);
					const tone sharp_tone = t_mul(sharp, 1 / maxf_(sharp_weight, LEAST_WEIGHT));
					const tone blend = t_mix(last, sharp_tone, alpha);
					out = t_mix(blend, fill, ALPHA_MOVING * speed);
				}
			}
			const size_t at = (size_t) y * (size_t) width + (size_t) x;
			double linear[3];
			untoned(out, linear);
			for (int c = 0; c < 3; ++c) {
				colour[3 * at + c] = linear[c];
				image[3 * at + c] = (float) linear[c];
			}
			depth[at] = st.closest;
		}
	}
	free(samples);
}

/* plugins/reconstruction/upsample/upsample.cpp: the drawn frame (drawn
 * size, RGB float) to the shown size (width x height) by bilinear taps in
 * float, the taps (:15 upsampleTap) from each shown pixel's centre in drawn
 * pixels, clamped to the drawn frame. */
typedef struct utap {
	int first, second;
	float share;
} utap;

static utap upsample_tap(int shown, int factor, int drawn) {
	const double centre = ((double) shown + 0.5) / (double) factor - 0.5;
	const double clamped = centre < 0.0 ? 0.0 : ((double) (drawn - 1) < centre ? (double) (drawn - 1) : centre);
	utap t;
	t.first = (int) clamped;
	t.second = t.first + 1 < drawn - 1 ? t.first + 1 : drawn - 1;
	t.share = (float) (clamped - (double) t.first);
	return t;
}

void kp_upsample(int width, int height, int factor, const float* drawn, float* shown) {
	const int dw = width / factor, dh = height / factor;
	for (int y = 0; y < height; ++y) {
		const utap row = upsample_tap(y, factor, dh);
		const float* upper = drawn + (size_t) row.first * (size_t) dw * 3;
		const float* lower = drawn + (size_t) row.second * (size_t) dw * 3;
		for (int x = 0; x < width; ++x) {
			const utap column = upsample_tap(x, factor, dw);
			for (int c = 0; c < 3; ++c) {
				/* :41 blendedChannel */
				const float a = upper[3 * column.first + c], b = upper[3 * column.second + c];
				const float d = lower[3 * column.first + c], e = lower[3 * column.second + c];
				const float top = a + (b - a) * column.share;
				const float bottom = d + (e - d) * column.share;
				shown[((size_t) y * (size_t) width + (size_t) x) * 3 + c] = top + (bottom - top) * row.share;
			}
		}
	}
}
