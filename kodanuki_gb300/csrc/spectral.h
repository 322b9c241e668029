// Wavelength and colour tables shared by host and device.
//
// The host builds them in double exactly as the reference does
// (math/colour.cpp:121-196: the fitted CIE curves tabled every 5 nm over
// 380-700 nm, the white point, and 256 equal-probability cuts of the
// wavelength density), then the frame copies them to constant memory.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define KDN_HD __host__ __device__
#else
#define KDN_HD
#endif

namespace kdn {

constexpr int kTableSize = 65;
constexpr int kCuts      = 256;
constexpr double kShortest = 380.0;
constexpr double kLongest  = 700.0;

struct SpectralTables {
	float cie[3][kTableSize]; // x, y, z
	float white[3];
	double cuts[kCuts + 1]; // kept in double: a lane is drawn in double and stored as float, as the reference does
};

void buildSpectralTables(SpectralTables& out);

// math/random.cpp:8 mixedBits
KDN_HD inline uint64_t mixedBits(uint64_t v) {
	v += 0x9E3779B97F4A7C15ULL;
	v = (v ^ (v >> 30)) * 0xBF58476D1CE4E5B9ULL;
	v = (v ^ (v >> 27)) * 0x94D049BB133111EBULL;
	return v ^ (v >> 31);
}

// math/random.cpp:19 hashedNumber, as the 53-bit integer it scales.
KDN_HD inline uint64_t hashedBits(uint64_t stream, uint64_t index, uint64_t coordinate) {
	return mixedBits(stream + mixedBits(index + mixedBits(coordinate))) >> 11;
}

} // namespace kdn
