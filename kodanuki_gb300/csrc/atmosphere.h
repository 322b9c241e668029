// The air of a physical sky (`sky physical`, plugins/feature/atmosphere):
// sunlight scattered once toward the eye by the air (Rayleigh, sharply
// bluer) and by the haze (Mie-like, grey, forward), over a planet of
// 6360 km with its air to 6420 km.  What each scatters toward the eye
// before its phase is tabled by height, bearing from the sun and
// wavelength (48 x 32 x 33, marched on the host in double once a sun and a
// haze); the phase, sharp about the sun, is applied where the sky is met.
// Below the horizon the sky shows the ground, lit by the sun and the sky
// (the landing table); the sun itself reaches the ground thinned by the
// air (the passed table).
#pragma once

#include <cstdint>

namespace kdn {

constexpr int kAirHeights  = 48;
constexpr int kAirBearings = 32;
constexpr int kAirColours  = 33; // math/spectrum.h tablePlaces: 380..700 nm
constexpr int kAirTable    = kAirHeights * kAirBearings * kAirColours;

// The sky's frame: up, the sun, and the level and aside directions about
// the sun's bearing (atmosphere.cpp:240 levelFrame).
struct AirFrame {
	double up[3], sun[3], level[3], aside[3];
};

// atmosphere.cpp:308 atmosphereOf for a sun direction and a haze: the
// frame, the air's and the haze's tables (kAirTable each, [row][column]
// [colour]), what of the sun passes to the ground and what lands on it
// (kAirColours each).
void buildAtmosphere(const double sunDirection[3], double haze, AirFrame& frame, double* air, double* hazeTable, double* passed, double* landing);

} // namespace kdn
