// Host construction of the wavelength and colour tables (math/colour.cpp:99-196).
#include "spectral.h"

#include <algorithm>
#include <cmath>

namespace kdn {

namespace {

double skewed(double nm, double peak, double below, double above) {
	const double width = nm < peak ? below : above;
	const double o     = (nm - peak) / width;
	return std::exp(-0.5 * o * o);
}

// The three multi-lobe fits of the CIE 1931 observer the reference tables.
double fitX(double nm) { return 1.056 * skewed(nm, 599.8, 37.9, 31.0) + 0.362 * skewed(nm, 442.0, 16.0, 26.7) - 0.065 * skewed(nm, 501.1, 20.4, 26.2); }
double fitY(double nm) { return 0.821 * skewed(nm, 568.8, 46.9, 40.5) + 0.286 * skewed(nm, 530.9, 16.3, 31.1); }
double fitZ(double nm) { return 1.217 * skewed(nm, 437.0, 11.8, 36.0) + 0.681 * skewed(nm, 459.0, 26.0, 13.8); }

void toLinear(double x, double y, double z, double rgb[3]) {
	rgb[0] = 3.2406 * x - 1.5372 * y - 0.4986 * z;
	rgb[1] = -0.9689 * x + 1.8758 * y + 0.0415 * z;
	rgb[2] = 0.0557 * x - 0.2040 * y + 1.0570 * z;
}

} // namespace

void buildSpectralTables(SpectralTables& out) {
	constexpr double step   = 5.0;
	constexpr int slices    = kTableSize - 1;
	constexpr double evenly = 0.3;
	double cx[kTableSize], cy[kTableSize], cz[kTableSize];
	double sx = 0, sy = 0, sz = 0;
	for (int s = 0; s < kTableSize; ++s) {
		const double nm = kShortest + step * s;
		cx[s]           = fitX(nm);
		cy[s]           = fitY(nm);
		cz[s]           = fitZ(nm);
		const double w  = (s == 0 || s == kTableSize - 1 ? 0.5 : 1.0) * step;
		sx += cx[s] * w;
		sy += cy[s] * w;
		sz += cz[s] * w;
	}
	double white[3];
	toLinear(sx, sy, sz, white);
	// the density of the hero wavelength: a share of the summed absolute
	// response of the three channels per slice, mixed with a flat share
	double seen[kTableSize];
	for (int s = 0; s < kTableSize; ++s) {
		double rgb[3];
		toLinear(cx[s], cy[s], cz[s], rgb);
		seen[s] = std::fabs(rgb[0] / white[0]) + std::fabs(rgb[1] / white[1]) + std::fabs(rgb[2] / white[2]);
	}
	double total = 0;
	for (int s = 0; s < slices; ++s) total += seen[s] + seen[s + 1];
	double shares[slices], before[slices + 1];
	before[0] = 0;
	for (int s = 0; s < slices; ++s) {
		shares[s]     = (1 - evenly) * (seen[s] + seen[s + 1]) / total + evenly / slices;
		before[s + 1] = before[s] + shares[s];
	}
	int slice = 0;
	double cuts[kCuts + 1];
	for (int i = 0; i <= kCuts; ++i) {
		const double u = double(i) / kCuts * before[slices];
		while (slice < slices - 1 && before[slice + 1] <= u) ++slice;
		const double along = std::clamp((u - before[slice]) / shares[slice], 0.0, 1.0);
		cuts[i]            = kShortest + step * (slice + along);
	}
	cuts[0]     = kShortest;
	cuts[kCuts] = kLongest;
	for (int s = 0; s < kTableSize; ++s) {
		out.cie[0][s] = float(cx[s]);
		out.cie[1][s] = float(cy[s]);
		out.cie[2][s] = float(cz[s]);
	}
	for (int c = 0; c < 3; ++c) out.white[c] = float(white[c]);
	for (int i = 0; i <= kCuts; ++i) out.cuts[i] = cuts[i];
}

} // namespace kdn
