// The tables of a physical sky, marched on the host in double
// (plugins/feature/atmosphere/atmosphere.cpp).  The constants are the
// reference's: the planet and the air's top (km), the scale heights of the
// air and the haze, the haze's lean and albedo, the march's steps.
#include "atmosphere.h"

#include <algorithm>
#include <cmath>

namespace kdn {

namespace {

constexpr double kPi         = 3.14159265358979323846;
constexpr double kPlanet     = 6360.0;
constexpr double kAirTop     = 6420.0;
constexpr double kEyeHeight  = 0.001;
constexpr double kAirScale   = 8.0;
constexpr double kHazeScale  = 1.2;
constexpr double kHazeLean   = 0.76;
constexpr double kHazeAlbedo = 0.9;
constexpr int kViewSteps     = 40;
constexpr int kSunSteps      = 12;
constexpr int kRings         = 32;
constexpr int kSpokes        = 64;

struct P {
	double x, y, z;
};
P operator+(P a, P b) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
P operator-(P a, P b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
P operator*(P a, double s) { return { a.x * s, a.y * s, a.z * s }; }
double dot(P a, P b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
P unit(P a) { return a * (1.0 / std::sqrt(dot(a, a))); }
P of(const double* v) { return { v[0], v[1], v[2] }; }
void put(double* out, P v) { out[0] = v.x, out[1] = v.y, out[2] = v.z; }

// the two densities a point holds, and their sums along a way
struct Depth {
	double air, haze;
};

double wavelengthOf(int colour) { return 380.0 + 320.0 * double(colour) / double(kAirColours - 1); }

// Rayleigh's fall with the fourth power of the wavelength, 33.1e-3 / km at 440 nm
double airScatter(double nm) {
	const double r = 440.0 / nm;
	return 33.1e-3 * r * r * r * r;
}

double hazeScatter(double nm, double haze) { return 0.004 * haze * haze * std::pow(550.0 / nm, 1.3); }

// where a way from inside a shell of a radius leaves it
double leaving(P from, P toward, double radius) {
	const double along = dot(from, toward);
	return -along + std::sqrt(std::max(along * along - (dot(from, from) - radius * radius), 0.0));
}

bool groundAhead(P from, P toward) {
	const double along = dot(from, toward);
	const double under = along * along - (dot(from, from) - kPlanet * kPlanet);
	return under >= 0.0 && -along - std::sqrt(under) > 0.0;
}

Depth densityAt(P at) {
	const double height = std::max(std::sqrt(dot(at, at)) - kPlanet, 0.0);
	return { std::exp(-height / kAirScale), std::exp(-height / kHazeScale) };
}

// the densities summed toward the sun to the air's top, the steps closer
// near the start (squared spacing)
Depth towardSun(P from, P sun) {
	const double reach = leaving(from, sun, kAirTop);
	Depth sum { 0, 0 };
	for (int k = 0; k < kSunSteps; ++k) {
		const double near = double(k) / kSunSteps, far = double(k + 1) / kSunSteps, mid = (double(k) + 0.5) / kSunSteps;
		const Depth d     = densityAt(from + sun * (reach * mid * mid));
		const double span = reach * (far * far - near * near);
		sum.air += d.air * span;
		sum.haze += d.haze * span;
	}
	return sum;
}

// One view from the eye: at each step lit by the sun, what the air and the
// haze there scatter, thinned along the way in and the way to the sun.
void marchView(P view, P sun, double haze, double* air, double* dust) {
	const P eye        = { 0.0, 0.0, kPlanet + kEyeHeight };
	const double reach = leaving(eye, view, kAirTop);
	Depth seen { 0, 0 };
	for (int k = 0; k < kViewSteps; ++k) {
		const double near = double(k) / kViewSteps, far = double(k + 1) / kViewSteps, mid = (double(k) + 0.5) / kViewSteps;
		const double span = reach * (far * far - near * near);
		const P at        = eye + view * (reach * mid * mid);
		const Depth there = densityAt(at);
		seen.air += there.air * span * 0.5;
		seen.haze += there.haze * span * 0.5;
		if (!groundAhead(at, sun)) {
			const Depth lit = towardSun(at, sun);
			const Depth crossed { seen.air + lit.air, seen.haze + lit.haze };
			for (int c = 0; c < kAirColours; ++c) {
				const double nm        = wavelengthOf(c);
				const double scattered = hazeScatter(nm, haze);
				const double thinned   = std::exp(-(airScatter(nm) * crossed.air + scattered / kHazeAlbedo * crossed.haze));
				air[c] += thinned * there.air * span * airScatter(nm);
				dust[c] += thinned * there.haze * span * scattered;
			}
		}
		seen.air += there.air * span * 0.5;
		seen.haze += there.haze * span * 0.5;
	}
}

double airPhase(double c) { return 3.0 / (16.0 * kPi) * (1.0 + c * c); }

double hazePhase(double c) {
	const double g2 = kHazeLean * kHazeLean;
	return 3.0 / (8.0 * kPi) * (1.0 - g2) * (1.0 + c * c) / ((2.0 + g2) * std::pow(1.0 + g2 - 2.0 * kHazeLean * c, 1.5));
}

// a table's value at fractional (row, column, colour), trilinear
double tableAt(const double* table, double row, double column, double colour) {
	const int r = std::min(int(row), kAirHeights - 2), b = std::min(int(column), kAirBearings - 2), l = std::min(int(colour), kAirColours - 2);
	const double fr = std::clamp(row - r, 0.0, 1.0), fb = std::clamp(column - b, 0.0, 1.0), fl = std::clamp(colour - l, 0.0, 1.0);
	double sum = 0.0;
	for (int dr = 0; dr < 2; ++dr) {
		for (int db = 0; db < 2; ++db) {
			for (int dl = 0; dl < 2; ++dl) {
				const double w = (dr ? fr : 1 - fr) * (db ? fb : 1 - fb) * (dl ? fl : 1 - fl);
				sum += w * table[((r + dr) * kAirBearings + b + db) * kAirColours + l + dl];
			}
		}
	}
	return sum;
}

} // namespace

void buildAtmosphere(const double sunDirection[3], double haze, AirFrame& frame, double* air, double* hazeTable, double* passed, double* landing) {
	const P up  = { 0, 0, 1 };
	const P sun = unit(of(sunDirection));
	// the level direction toward the sun's bearing (atmosphere.cpp:240)
	const P flat  = sun - up * dot(sun, up);
	const P level = std::sqrt(dot(flat, flat)) < 1e-9 ? P { 1, 0, 0 } : unit(flat);
	const P aside = { up.y * level.z - up.z * level.y, up.z * level.x - up.x * level.z, up.x * level.y - up.y * level.x };
	put(frame.up, up);
	put(frame.sun, sun);
	put(frame.level, level);
	put(frame.aside, aside);
	const P sunLocal = { dot(sun, level), dot(sun, aside), dot(sun, up) };
	std::fill(air, air + kAirTable, 0.0);
	std::fill(hazeTable, hazeTable + kAirTable, 0.0);
	// rows of height (squared spacing to the zenith), columns of bearing 0..pi
	for (int row = 0; row < kAirHeights; ++row) {
		const double along  = double(row) / double(kAirHeights - 1);
		const double height = 0.5 * kPi * along * along;
		for (int column = 0; column < kAirBearings; ++column) {
			const double bearing = kPi * double(column) / double(kAirBearings - 1);
			const P view         = { std::cos(height) * std::cos(bearing), std::cos(height) * std::sin(bearing), std::sin(height) };
			const int first      = (row * kAirBearings + column) * kAirColours;
			marchView(view, sunLocal, haze, air + first, hazeTable + first);
		}
	}
	// what of the sun passes straight down to the eye (zero with the sun below)
	const P eye         = { 0.0, 0.0, kPlanet + kEyeHeight };
	const Depth straight = towardSun(eye, sunLocal);
	const bool set       = groundAhead(eye, sunLocal);
	for (int c = 0; c < kAirColours; ++c) {
		const double nm = wavelengthOf(c);
		passed[c]       = set ? 0.0 : std::exp(-(airScatter(nm) * straight.air + hazeScatter(nm, haze) / kHazeAlbedo * straight.haze));
	}
	// what lands on the ground: the sky over the hemisphere, cosine-weighted,
	// plus the sun overhead
	for (int c = 0; c < kAirColours; ++c) landing[c] = 0.0;
	for (int ring = 0; ring < kRings; ++ring) {
		const double rise = (double(ring) + 0.5) / kRings;
		const double flatness = std::sqrt(1.0 - rise * rise);
		for (int spoke = 0; spoke < kSpokes; ++spoke) {
			const double turn = 2.0 * kPi * (double(spoke) + 0.5) / kSpokes;
			const P toward    = level * (flatness * std::cos(turn)) + aside * (flatness * std::sin(turn)) + up * rise;
			const double h    = std::asin(std::clamp(dot(toward, up), -1.0, 1.0));
			const double b    = std::abs(std::atan2(dot(toward, aside), dot(toward, level)));
			const double row  = std::sqrt(std::max(h, 0.0) / (0.5 * kPi)) * double(kAirHeights - 1);
			const double col  = b / kPi * double(kAirBearings - 1);
			const double cosine = dot(toward, sun);
			for (int c = 0; c < kAirColours; ++c) {
				const double sky = airPhase(cosine) * tableAt(air, row, col, double(c)) + hazePhase(cosine) * tableAt(hazeTable, row, col, double(c));
				landing[c] += sky * rise * (2.0 * kPi / (kRings * kSpokes));
			}
		}
	}
	const double overhead = std::max(dot(sun, up), 0.0);
	for (int c = 0; c < kAirColours; ++c) landing[c] += passed[c] * overhead;
}

} // namespace kdn
