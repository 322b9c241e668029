/*
 * Oracle numbers, wavelengths and colour: the counter-based generator of
 * math/random.cpp and the tables of math/colour.cpp / math/spectrum.cpp,
 * restated.  Test infrastructure only (see kdn_port.h).
 */
#include "kdn_port.h"

#include <math.h>
#include <pthread.h>

#define SHORTEST 380.0
#define LONGEST 700.0
#define TABLE_STEP 5.0
#define TABLE_SIZE 65
#define TABLE_SLICES (TABLE_SIZE - 1)
#define EVEN_SHARE 0.3
#define CUTS 256

/* math/random.cpp:8 mixedBits (splitmix64 finaliser) */
uint64_t kp_mixed_bits(uint64_t v) {
	v += 0x9E3779B97F4A7C15ULL;
	v = (v ^ (v >> 30)) * 0xBF58476D1CE4E5B9ULL;
	v = (v ^ (v >> 27)) * 0x94D049BB133111EBULL;
	return v ^ (v >> 31);
}

/* math/random.cpp:15 unitOf */
double kp_unit_of(uint64_t bits) { return (double) (bits >> 11) * 0x1p-53; }

/* math/random.cpp:19 hashedNumber */
double kp_hashed(uint64_t stream, uint64_t index, uint64_t coordinate) {
	return kp_unit_of(kp_mixed_bits(stream + kp_mixed_bits(index + kp_mixed_bits(coordinate))));
}

static double clampd(double x, double lo, double hi) { return x < lo ? lo : (hi < x ? hi : x); }

/* math/colour.cpp:99-113 the fitted CIE curves */
static double skewed(double nm, double peak, double below, double above) {
	const double width = nm < peak ? below : above;
	const double o = (nm - peak) / width;
	return exp(-0.5 * o * o);
}
static double fit_x(double nm) { return 1.056 * skewed(nm, 599.8, 37.9, 31.0) + 0.362 * skewed(nm, 442.0, 16.0, 26.7) - 0.065 * skewed(nm, 501.1, 20.4, 26.2); }
static double fit_y(double nm) { return 0.821 * skewed(nm, 568.8, 46.9, 40.5) + 0.286 * skewed(nm, 530.9, 16.3, 31.1); }
static double fit_z(double nm) { return 1.217 * skewed(nm, 437.0, 11.8, 36.0) + 0.681 * skewed(nm, 459.0, 26.0, 13.8); }

static void linear_of(double x, double y, double z, double rgb[3]) {
	rgb[0] = 3.2406 * x - 1.5372 * y - 0.4986 * z;
	rgb[1] = -0.9689 * x + 1.8758 * y + 0.0415 * z;
	rgb[2] = 0.0557 * x - 0.2040 * y + 1.0570 * z;
}

static double cx[TABLE_SIZE], cy[TABLE_SIZE], cz[TABLE_SIZE], white[3], cuts[CUTS + 1];
static pthread_once_t once = PTHREAD_ONCE_INIT;

/* math/colour.cpp:121-196 tabledCurves, seenResponse, sliceShares, cutsOf */
static void build_tables(void) {
	double sx = 0, sy = 0, sz = 0;
	for (int s = 0; s < TABLE_SIZE; ++s) {
		const double nm = SHORTEST + TABLE_STEP * s;
		cx[s] = fit_x(nm);
		cy[s] = fit_y(nm);
		cz[s] = fit_z(nm);
		const int edge = s == 0 || s == TABLE_SIZE - 1;
		const double w = (edge ? 0.5 : 1.0) * TABLE_STEP;
		sx = sx + cx[s] * w;
		sy = sy + cy[s] * w;
		sz = sz + cz[s] * w;
	}
	linear_of(sx, sy, sz, white);
	double seen[TABLE_SIZE];
	for (int s = 0; s < TABLE_SIZE; ++s) {
		double rgb[3];
		linear_of(cx[s], cy[s], cz[s], rgb);
		seen[s] = fabs(rgb[0] / white[0]) + fabs(rgb[1] / white[1]) + fabs(rgb[2] / white[2]);
	}
	double total = 0;
	for (int s = 0; s < TABLE_SLICES; ++s) total += seen[s] + seen[s + 1];
	double shares[TABLE_SLICES], before[TABLE_SLICES + 1];
	for (int s = 0; s < TABLE_SLICES; ++s) shares[s] = (1 - EVEN_SHARE) * (seen[s] + seen[s + 1]) / total + EVEN_SHARE / TABLE_SLICES;
	before[0] = 0;
	for (int s = 0; s < TABLE_SLICES; ++s) before[s + 1] = before[s] + shares[s];
	int slice = 0;
	for (int i = 0; i <= CUTS; ++i) {
		const double u = (double) i / CUTS * before[TABLE_SLICES];
		while (slice < TABLE_SLICES - 1 && before[slice + 1] <= u) ++slice;
		const double along = clampd((u - before[slice]) / shares[slice], 0.0, 1.0);
		cuts[i] = SHORTEST + TABLE_STEP * (slice + along);
	}
	cuts[0] = SHORTEST;
	cuts[CUTS] = LONGEST;
}

static void tables(void) { pthread_once(&once, build_tables); }

/* math/colour.cpp:236 sampledWavelengths */
static double basis_red(double nm);
static double basis_green(double nm);
static double basis_blue(double nm);

void kp_sampled_wavelengths(double u, double nanometres[4], double density[4], double basis[12]) {
	tables();
	for (int lane = 0; lane < 4; ++lane) {
		const double raw = u + 0.25 * lane;
		const double turned = raw >= 1 ? raw - 1 : raw;
		const double place = turned * CUTS;
		const int index = (int) place < CUTS - 1 ? (int) place : CUTS - 1;
		const double width = cuts[index + 1] - cuts[index];
		const double nm = cuts[index] + (place - index) * width;
		const double cap = nextafter(LONGEST, SHORTEST);
		/* the reference stores the lanes as float (math/spectrum.cpp:62) */
		const double kept = nm < cap ? nm : cap;
		nanometres[lane] = (double) (float) kept;
		density[lane] = (double) (float) (1 / (CUTS * width));
		/* math/spectrum.cpp:62 wavelengthsAt: basis from the double, kept as float */
		basis[lane] = (double) (float) basis_red(kept);
		basis[4 + lane] = (double) (float) basis_green(kept);
		basis[8 + lane] = (double) (float) basis_blue(kept);
	}
}

/* math/colour.cpp:252 wavelengthShare */
double kp_wavelength_share(double start, uint32_t index) {
	const double turned = (double) index * 0.6180339887498949 + start;
	return turned - floor(turned);
}

/* math/spectrum.cpp:42-60 the smooth basis curves */
static double smooth_rise(double nm, double lo, double hi) {
	const double b = clampd((nm - lo) / (hi - lo), 0.0, 1.0);
	return b * b * (3 - 2 * b);
}
static double basis_red(double nm) { return smooth_rise(nm, 575.0, 605.0); }
static double basis_blue(double nm) { return 1 - smooth_rise(nm, 445.0, 530.0); }
static double basis_green(double nm) { return (1 - basis_blue(nm)) * (1 - basis_red(nm)); }

/* math/colour.cpp:69-96 leastChannel, mostChannel, spectrumOf */
void kp_spectrum_of(const double rgb[3], const double basis[12], double out[4]) {
	int least;
	if (rgb[0] <= rgb[1] && rgb[0] <= rgb[2]) least = 0;
	else least = rgb[1] <= rgb[0] && rgb[1] <= rgb[2] ? 1 : 2;
	const int first = least == 0 ? 1 : 0;
	const int second = least == 2 ? 1 : 2;
	const int most = rgb[first] <= rgb[second] ? second : first;
	const int middle = 3 - least - most;
	const double base = rgb[least];
	const double low = rgb[middle] - base;
	const double high = rgb[most] - rgb[middle];
	for (int lane = 0; lane < 4; ++lane) {
		out[lane] = base + low * (1 - basis[4 * least + lane]) + high * basis[4 * most + lane];
	}
}

static double table_at(const double* curve, double nm) {
	const double slot = (nm - SHORTEST) / TABLE_STEP;
	int below = (int) slot;
	below = below < 0 ? 0 : (below > TABLE_SIZE - 2 ? TABLE_SIZE - 2 : below);
	const double blend = clampd(slot - below, 0.0, 1.0);
	return curve[below] + blend * (curve[below + 1] - curve[below]);
}

/* math/colour.cpp:213 colourOf */
void kp_colour_of(const double nanometres[4], const double density[4], const double spectrum[4], double rgb[3]) {
	tables();
	double x = 0, y = 0, z = 0;
	for (int lane = 0; lane < 4; ++lane) {
		if (density[lane] <= 0) continue;
		const double w = spectrum[lane] / density[lane];
		const double nm = nanometres[lane];
		x = x + table_at(cx, nm) * w;
		y = y + table_at(cy, nm) * w;
		z = z + table_at(cz, nm) * w;
	}
	double lin[3];
	linear_of(x / 4, y / 4, z / 4, lin);
	for (int c = 0; c < 3; ++c) rgb[c] = lin[c] / white[c];
}

/* ---- --use sampler=sobol (plugins/sampler/sobol/sobol.cpp): an
 * Owen-scrambled Sobol sequence for the first 28 dimensions of a path's
 * draws.  Direction numbers from Joe and Kuo's published primitive
 * polynomials and initial numbers (dimension 0: van der Corput), the index
 * shuffled and the points scrambled by the Laine-Karras permutation
 * (Burley 2020), seeds hashed by Wellons' lowbias32. ---- */
static uint32_t sobol_stirred(uint32_t v) {
	v ^= v >> 16;
	v *= 0x7FEB352DU;
	v ^= v >> 15;
	v *= 0x846CA68BU;
	return v ^ (v >> 16);
}

static uint32_t sobol_reversed(uint32_t v) {
	uint32_t r = 0;
	for (int b = 0; b < 32; ++b) r |= ((v >> b) & 1U) << (31 - b);
	return r;
}

static uint32_t sobol_reversed16(uint32_t v) { return sobol_reversed(v & 0xFFFFU) >> 16; }

static uint32_t laine_karras(uint32_t v, uint32_t seed) {
	v += seed;
	v ^= v * 0x6C50B47CU;
	v ^= v * 0xB82F1E52U;
	v ^= v * 0xC7AFE638U;
	return v ^ (v * 0x8D22F6E6U);
}

void kp_sobol_tables(uint32_t* out) {
	static const int degree[KP_SOBOL_DIMENSIONS] = { 0, 1, 2, 3, 3, 4, 4, 5, 5, 5, 5, 5, 5, 6, 6, 6, 6, 6, 6, 7, 7, 7, 7, 7, 7, 7, 7, 7 };
	static const int inner[KP_SOBOL_DIMENSIONS] = { 0, 0, 1, 1, 2, 1, 4, 2, 4, 7, 11, 13, 14, 1, 13, 16, 19, 22, 25, 1, 4, 7, 8, 14, 19, 21, 28, 31 };
	static const uint32_t initial[KP_SOBOL_DIMENSIONS][7] = {
		{ 1 }, { 1 }, { 1, 3 }, { 1, 3, 1 }, { 1, 1, 1 }, { 1, 1, 3, 3 }, { 1, 3, 5, 13 }, { 1, 1, 5, 5, 17 }, { 1, 1, 5, 5, 5 }, { 1, 1, 7, 11, 19 },
		{ 1, 1, 5, 1, 1 }, { 1, 1, 1, 3, 11 }, { 1, 3, 5, 5, 31 }, { 1, 3, 3, 9, 7, 49 }, { 1, 1, 1, 15, 21, 21 }, { 1, 3, 1, 13, 27, 49 },
		{ 1, 1, 1, 15, 7, 5 }, { 1, 3, 1, 15, 13, 25 }, { 1, 1, 5, 5, 19, 61 }, { 1, 3, 7, 11, 23, 15, 103 }, { 1, 3, 7, 13, 13, 15, 69 },
		{ 1, 1, 3, 13, 7, 35, 63 }, { 1, 3, 5, 9, 1, 25, 53 }, { 1, 3, 1, 13, 9, 35, 107 }, { 1, 3, 1, 5, 27, 61, 31 }, { 1, 1, 5, 11, 19, 41, 61 },
		{ 1, 3, 5, 3, 3, 13, 69 }, { 1, 1, 7, 13, 1, 19, 1 },
	};
	for (int d = 0; d < KP_SOBOL_DIMENSIONS; ++d) {
		uint32_t m[16];
		for (int bit = 0; bit < 16; ++bit) {
			const int s = degree[d];
			if (s == 0) {
				m[bit] = 1;
			} else if (bit < s) {
				m[bit] = initial[d][bit];
			} else {
				/* Bratley and Fox's recurrence */
				uint32_t v = m[bit - s] ^ (m[bit - s] << s);
				for (int k = 1; k < s; ++k) {
					if ((inner[d] >> (s - 1 - k)) & 1) v ^= m[bit - k] << k;
				}
				m[bit] = v;
			}
		}
		for (uint32_t byte = 0; byte < 256; ++byte) {
			uint32_t low = 0, high = 0;
			for (int bit = 0; bit < 16; ++bit) {
				const uint32_t column = sobol_reversed(m[bit] << (31 - bit));
				if (((byte >> bit) & 1U) != 0) low ^= column;
				if ((((byte << 8) >> bit) & 1U) != 0) high ^= column;
			}
			out[d * 512 + byte] = low;
			out[d * 512 + 256 + byte] = high;
		}
	}
}

/* sobol.cpp:140 sobolNumber: the number of dimension `dimension` (below 28)
 * of sample `index` of the pixel stream `stream` */
double kp_sobol_number(const uint32_t* tables, uint64_t stream, uint32_t index, uint32_t dimension) {
	const uint32_t own = dimension < KP_SOBOL_SHARED ? 0U : 0x68E31DA4U;
	const uint32_t place = sobol_reversed16(laine_karras(sobol_reversed16(index), sobol_stirred((uint32_t) (stream >> 32) + own)) & 0xFFFFU);
	const uint32_t seed = sobol_stirred((uint32_t) (stream >> 32) + dimension * 0xA136AAADU + 0x2545F491U);
	const uint32_t* column = tables + (size_t) (dimension < KP_SOBOL_SHARED ? dimension : dimension - KP_SOBOL_SHARED) * 512;
	const uint32_t value = column[place & 0xFFU] ^ column[256 + ((place >> 8) & 0xFFU)];
	return (double) sobol_reversed(laine_karras(value, seed)) * 0x1p-32;
}
