/*
 * Oracle denoiser: the reference's SVGF-like a-trous filter
 * (plugins/reconstruction/atrous/atrous.cpp) restated in C, single precision
 * where the reference keeps floats.  Test infrastructure (see kdn_port.h).
 *
 *   preparedDenoise (:148)   guides (point, normal, plane offset, reach) and
 *                            demodulated light with its history variance;
 *   estimatedChunk  (:376)   a 7x7 spatial variance for young pixels;
 *   filteredChunk   (:411)   4 passes of the 5x5 B3 spline at steps 1,2,4,8,
 *                            edge-stopped by normal^128, plane distance and
 *                            luminance over a 3x3-prefiltered deviation;
 *   remodulatedImage (:461)  times the albedo, faded toward the history by
 *                            its length.
 */
#include "kdn_port.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NO_LEAF 0xFFFFFFFFu

static const float spline[5] = { 1.0f / 16, 1.0f / 4, 3.0f / 8, 1.0f / 4, 1.0f / 16 };
static const float gauss3[3] = { 0.25f, 0.5f, 0.25f };

/* atrous.cpp:31 quickExp: 2^(x log2 e) from a fitted quadratic mantissa */
static float quick_exp(float x) {
	const float t = (x > -30.0f ? x : -30.0f) * 1.44269504f;
	const float whole = floorf(t);
	const float f = t - whole;
	const float power = 1 + f * (0.66023f + f * 0.33977f);
	int32_t bits;
	memcpy(&bits, &power, 4);
	bits += (int32_t) whole * (1 << 23);
	float value;
	memcpy(&value, &bits, 4);
	return x > -30.0f ? value : 0.0f;
}

static float luma(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

typedef struct lights {
	float *r, *g, *b, *lum, *var;
} lights;

typedef struct guides {
	float *x, *y, *z, *nx, *ny, *nz, *offset, *reach, *sky;
} guides;

static double divisor_of(double a) { return a < 1e-3 ? 1 : a; }

static void alloc_lights(lights* l, size_t n) {
	l->r = calloc(n, 4);
	l->g = calloc(n, 4);
	l->b = calloc(n, 4);
	l->lum = calloc(n, 4);
	l->var = calloc(n, 4);
}

static void free_lights(lights* l) {
	free(l->r);
	free(l->g);
	free(l->b);
	free(l->lum);
	free(l->var);
}

typedef struct sums {
	float r, g, b, var, sq, w;
} sums;

/* atrous.cpp:260-300: weight of tap q for centre p */
static float tap_weight(const guides* G, const lights* L, size_t p, size_t q, float inv_plane, float inv_dev, float kernel) {
	const float facing = G->nx[p] * G->nx[q] + G->ny[p] * G->ny[q] + G->nz[p] * G->nz[q] + G->sky[p] * G->sky[q];
	float power = facing > 0.5f ? facing : 0.0f;
	for (int n = 0; n < 7; ++n) power *= power;
	const float along = G->x[q] * G->nx[p] + G->y[q] * G->ny[p] + G->z[q] * G->nz[p];
	const float plane = fabsf(along - G->offset[p]) * inv_plane;
	const float apart = fabsf(L->lum[q] - L->lum[p]) * inv_dev;
	return kernel * power * quick_exp(-plane - apart);
}

void kp_denoise(int width, int height, int demodulated, const double lens[14], const double* colour, const double* moment, const float* length,
                const float* distance, const double* normal, const uint32_t* leaf, const double* albedo, float* out) {
	const size_t n = (size_t) width * (size_t) height;
	guides G;
	float** gf[9] = { &G.x, &G.y, &G.z, &G.nx, &G.ny, &G.nz, &G.offset, &G.reach, &G.sky };
	for (int k = 0; k < 9; ++k) *gf[k] = calloc(n, 4);
	lights L, S;
	alloc_lights(&L, n);
	alloc_lights(&S, n);
	/* atrous.cpp:55 denoiseCamera: the heading through each pixel's centre */
	const double sideways = lens[12] * lens[13];
	double corner[3], across[3], down[3];
	for (int a = 0; a < 3; ++a) {
		corner[a] = lens[3 + a] - lens[6 + a] * sideways + lens[9 + a] * lens[12];
		across[a] = lens[6 + a] * (2 * sideways / (double) width);
		down[a] = lens[9 + a] * (-2 * lens[12] / (double) height);
	}
	for (int y = 0; y < height; ++y) {
		for (int x = 0; x < width; ++x) {
			const size_t p = (size_t) y * (size_t) width + (size_t) x;
			const int sky = leaf[p] == NO_LEAF || !isfinite(distance[p]) || !(distance[p] > 0);
			if (sky) {
				G.x[p] = G.y[p] = G.z[p] = G.nx[p] = G.ny[p] = G.nz[p] = G.offset[p] = G.reach[p] = 0;
				G.sky[p] = 1;
			} else {
				double h[3];
				for (int a = 0; a < 3; ++a) h[a] = corner[a] + across[a] * (x + 0.5) + down[a] * (y + 0.5);
				const double hl = sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
				double pt[3];
				for (int a = 0; a < 3; ++a) pt[a] = h[a] * ((double) distance[p] / hl);
				G.x[p] = (float) pt[0];
				G.y[p] = (float) pt[1];
				G.z[p] = (float) pt[2];
				G.nx[p] = (float) normal[3 * p];
				G.ny[p] = (float) normal[3 * p + 1];
				G.nz[p] = (float) normal[3 * p + 2];
				G.offset[p] = (float) (pt[0] * normal[3 * p] + pt[1] * normal[3 * p + 1] + pt[2] * normal[3 * p + 2]);
				G.reach[p] = (float) (1 / (0.02 * (double) distance[p]));
				G.sky[p] = 0;
			}
			double dv[3] = { 1, 1, 1 };
			if (!demodulated) {
				for (int c = 0; c < 3; ++c) dv[c] = divisor_of(albedo[3 * p + c]);
			}
			L.r[p] = (float) (colour[3 * p] / dv[0]);
			L.g[p] = (float) (colour[3 * p + 1] / dv[1]);
			L.b[p] = (float) (colour[3 * p + 2] / dv[2]);
			L.lum[p] = luma(L.r[p], L.g[p], L.b[p]);
			if (!(length[p] >= 4)) {
				L.var[p] = -1;
			} else {
				const double l = 0.2126 * colour[3 * p] + 0.7152 * colour[3 * p + 1] + 0.0722 * colour[3 * p + 2];
				const double scale = 0.2126 * dv[0] + 0.7152 * dv[1] + 0.0722 * dv[2];
				const double spread = moment[p] - l * l > 0 ? moment[p] - l * l : 0.0;
				L.var[p] = (float) (spread / ((double) length[p] * scale * scale));
			}
		}
	}
	/* estimatedChunk: the 7x7 variance of young pixels, unguided by luminance */
	for (int y = 0; y < height; ++y) {
		for (int x = 0; x < width; ++x) {
			const size_t p = (size_t) y * (size_t) width + (size_t) x;
			S.r[p] = L.r[p];
			S.g[p] = L.g[p];
			S.b[p] = L.b[p];
			S.lum[p] = L.lum[p];
			S.var[p] = L.var[p];
			if (!(L.var[p] < 0)) continue;
			sums s = { 0, 0, 0, 0, 0, 0 };
			for (int j = -3; j <= 3; ++j) {
				for (int i = -3; i <= 3; ++i) {
					const int qx = x + i, qy = y + j;
					if (qy < 0 || qy >= height || qx < 0 || qx >= width) continue;
					const size_t q = (size_t) qy * (size_t) width + (size_t) qx;
					const float w = tap_weight(&G, &L, p, q, G.reach[p] * 1.0f, 0.0f, 1.0f);
					s.r += w * L.r[q];
					s.g += w * L.g[q];
					s.b += w * L.b[q];
					s.var += w * w * L.var[q];
					s.w += w;
					s.sq += w * L.lum[q] * L.lum[q];
				}
			}
			if (!(s.w > 0)) {
				S.var[p] = 0;
			} else {
				const float mean = luma(s.r, s.g, s.b) / s.w;
				const float v = s.sq / s.w - mean * mean;
				S.var[p] = v > 0.0f ? v : 0.0f;
			}
		}
	}
	lights T = L;
	L = S;
	S = T;
	/* filteredChunk x4 */
	for (int pass = 0; pass < 4; ++pass) {
		const int step = 1 << pass;
		for (int y = 0; y < height; ++y) {
			for (int x = 0; x < width; ++x) {
				const size_t p = (size_t) y * (size_t) width + (size_t) x;
				/* prefilteredDeviation: 3x3 Gaussian of the variance */
				float vs = 0, vw = 0;
				for (int j = 0; j < 3; ++j) {
					for (int i = 0; i < 3; ++i) {
						const int qx = x + i - 1, qy = y + j - 1;
						if (qy < 0 || qy >= height || qx < 0 || qx >= width) continue;
						const size_t q = (size_t) qy * (size_t) width + (size_t) qx;
						const float k = gauss3[i] * gauss3[j];
						vs += k * L.var[q];
						vw += k;
					}
				}
				const float deviation = sqrtf(vs / vw);
				const float inv_dev = 1 / (4.0f * deviation + 1e-4f + 1e-3f * L.lum[p]);
				const float inv_plane = G.reach[p] * (1 / (float) step);
				sums s = { 0, 0, 0, 0, 0, 0 };
				for (int j = -2; j <= 2; ++j) {
					for (int i = -2; i <= 2; ++i) {
						const int qx = x + i * step, qy = y + j * step;
						if (qy < 0 || qy >= height || qx < 0 || qx >= width) continue;
						const size_t q = (size_t) qy * (size_t) width + (size_t) qx;
						const float w = tap_weight(&G, &L, p, q, inv_plane, inv_dev, spline[i + 2] * spline[j + 2]);
						s.r += w * L.r[q];
						s.g += w * L.g[q];
						s.b += w * L.b[q];
						s.var += w * w * L.var[q];
						s.w += w;
					}
				}
				S.r[p] = L.r[p];
				S.g[p] = L.g[p];
				S.b[p] = L.b[p];
				S.lum[p] = L.lum[p];
				S.var[p] = L.var[p];
				if (s.w > 0) {
					const float scale = 1 / s.w;
					S.r[p] = s.r * scale;
					S.g[p] = s.g * scale;
					S.b[p] = s.b * scale;
					S.lum[p] = luma(S.r[p], S.g[p], S.b[p]);
					S.var[p] = s.var * scale * scale;
				}
			}
		}
		T = L;
		L = S;
		S = T;
	}
	/* remodulatedImage */
	for (size_t p = 0; p < n; ++p) {
		double dv[3], held[3];
		for (int c = 0; c < 3; ++c) {
			dv[c] = divisor_of(albedo[3 * p + c]);
			held[c] = demodulated ? colour[3 * p + c] * dv[c] : colour[3 * p + c];
		}
		const double share = 1 / (1 + (double) length[p] / 8);
		const float f[3] = { L.r[p], L.g[p], L.b[p] };
		for (int c = 0; c < 3; ++c) out[3 * p + c] = (float) ((double) f[c] * dv[c] * share + held[c] * (1 - share));
	}
	for (int k = 0; k < 9; ++k) free(*gf[k]);
	free_lights(&L);
	free_lights(&S);
}
