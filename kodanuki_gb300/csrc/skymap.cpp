// The sky chart of `--use sampler=sky_map`, built on the host
// (plugins/sampler/sky_map/sky_map.cpp:99 chartedSky).
#include "skymap.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace kdn {

namespace {

// light.cpp:582 gradientColour's channel mean at a height (the cosine to +z)
double brightnessAt(const SkyGradient& sky, double height) {
	const double* far  = height >= 0 ? sky.zenith : sky.ground;
	const double share = std::sqrt(std::abs(height));
	double mean        = 0;
	for (int c = 0; c < 3; ++c) mean += sky.horizon[c] * (1 - share) + far[c] * share;
	return std::max(mean / 3, 0.0);
}

} // namespace

bool buildSkyChart(const SkyGradient& sky, const ChartLamp* lamps, uint32_t lampCount, const double middle[3], double* chart) {
	const double rowHeight = 2.0 / kChartRows;
	// sky_map.cpp:42 cellWeights at each cell's middle direction
	std::vector<double> weights(size_t(kChartRows) * kChartColumns);
	for (int row = 0; row < kChartRows; ++row) {
		const double height = -1 + (double(row) + 0.5) * rowHeight;
		for (int column = 0; column < kChartColumns; ++column) {
			// sky_map.cpp:30 chartDirection's cosine to the sky's up is the
			// row's height (level and aside lie in the horizon), so a gradient
			// sky's cells of a row weigh alike
			weights[size_t(row) * kChartColumns + column] = brightnessAt(sky, height);
		}
	}
	double total = 0;
	for (double w : weights) total += w;
	if (!(total > 0)) return false;
	// sky_map.cpp:67 filledChart over :54 runOfRow
	double* rows  = chart;
	double* cells = chart + kChartRows + 1;
	rows[0]       = 0;
	for (int row = 0; row < kChartRows; ++row) {
		double* run = cells + row * kChartCells;
		run[0]      = 0;
		for (int column = 0; column < kChartColumns; ++column) run[column + 1] = run[column] + weights[size_t(row) * kChartColumns + column];
		const double held = run[kChartColumns];
		for (int column = 1; column <= kChartColumns; ++column) run[column] = held > 0 ? run[column] / held : double(column) / kChartColumns;
		rows[row + 1] = rows[row] + held / total;
	}
	rows[kChartRows]        = 1;
	const double brightness = total / double(kChartRows * kChartColumns);
	// sky_map.cpp:83 lampSent, :94 outshone: the lamps' light reaching the
	// region's middle against the sky's over the sphere
	double lit = 0;
	for (uint32_t k = 0; k < lampCount; ++k) {
		const ChartLamp& l = lamps[k];
		// a directional light, a sun or a moon sends its power's mean from afar
		if (l.kind == 1 || l.kind == 4 || l.kind == 5) {
			lit += std::max((l.power[0] + l.power[1] + l.power[2]) / 3, 0.0);
			continue;
		}
		double place[3], apart = 0;
		for (int a = 0; a < 3; ++a) {
			place[a]        = l.kind == 3 ? l.at[a] + (l.along[a] + l.across[a]) * 0.5 : l.at[a];
			const double d  = place[a] - middle[a];
			apart += d * d;
		}
		const double mean    = std::max((l.power[0] + l.power[1] + l.power[2]) / 3, 0.0);
		const double emitted = (l.kind == 3 ? kChartPi : 4 * kChartPi) * mean;
		lit += emitted / (4 * kChartPi * std::max(apart, 1e-12));
	}
	return !(lit > 5 * 4 * kChartPi * brightness);
}

} // namespace kdn
