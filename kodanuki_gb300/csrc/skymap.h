// `--use sampler=sky_map` (plugins/sampler/sky_map/sky_map.cpp): the sky
// aimed at by a chart of its brightness over directions, 64 rows of equal
// height (the cosine to the sky's up, -1..1) by 128 columns of equal turn,
// each cell's share of the sky's channel-mean brightness, mixed with 10%
// uniform directions; the sky is left uncharted (only met) where the lamps
// outshine it five times over as seen from the middle of the scene's
// region.  The host builds the chart in double as the reference does; the
// device reads it in double where it searches it.
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define KDN_HD __host__ __device__
#else
#define KDN_HD
#endif

namespace kdn {

constexpr int kChartRows = 64, kChartColumns = 128;
constexpr int kChartCells  = kChartColumns + 1; // a row's run of shares
constexpr double kChartEven = 0.1;              // sky_map.cpp:16 evenShare
// the chart as the device reads it: the rows' run (kChartRows + 1), then
// each row's run of its columns (kChartRows x kChartCells)
constexpr int kChartDoubles = kChartRows + 1 + kChartRows * kChartCells;

struct SkyGradient {
	double zenith[3], horizon[3], ground[3];
};

struct ChartLamp {
	uint32_t kind; // sdf/scene.h LightKind
	double at[3], along[3], across[3], power[3];
};

// sky_map.cpp:99 chartedSky: the chart, or false where the sky is dark or
// the lamps outshine it (it is then only met).  The sky's up is +z
// (light.cpp:98 lightsOf), so the chart's level and aside are +x and +y.
bool buildSkyChart(const SkyGradient& sky, const ChartLamp* lamps, uint32_t lampCount, const double middle[3], double* chart);

constexpr double kChartPi = 3.14159265358979323846;

// sky_map.cpp:153 chartDensity: the solid-angle density of drawing `toward`
KDN_HD inline double chartDensity(const double* chart, double x, double y, double z) {
	const double rowHeight = 2.0 / kChartRows, columnWidth = 2 * kChartPi / kChartColumns;
	const double height = z < -1.0 ? -1.0 : (z > 1.0 ? 1.0 : z);
	const double angle  = std::atan2(y, x);
	const double turn   = angle < 0 ? angle + 2 * kChartPi : angle;
	int row             = int((height + 1) / rowHeight);
	int column          = int(turn / columnWidth);
	row                 = row < kChartRows - 1 ? row : kChartRows - 1;
	column              = column < kChartColumns - 1 ? column : kChartColumns - 1;
	const double* run   = chart + kChartRows + 1 + row * kChartCells;
	const double held   = (chart[row + 1] - chart[row]) * (run[column + 1] - run[column]);
	return kChartEven / (4 * kChartPi) + (1 - kChartEven) * held / (rowHeight * columnWidth);
}

// sky_map.cpp:131 foundIn: the cell whose run passes `target` first
KDN_HD inline int chartFound(const double* run, int count, double target) {
	int lo = 0, hi = count; // the first of run[1..count] above target, as std::upper_bound
	while (lo < hi) {
		const int mid = (lo + hi) / 2;
		if (target < run[1 + mid]) hi = mid;
		else lo = mid + 1;
	}
	return lo < count - 1 ? lo : count - 1;
}

} // namespace kdn
