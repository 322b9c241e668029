// The numbers of `--use sampler=sobol` (plugins/sampler/sobol/sobol.cpp,
// drawn by plugins/transport/paths/sampler.cpp:16 numberAt): the first 28
// dimensions of a path's draws (a pixel's four, then three events of
// eight) come from a Sobol sequence, Owen-scrambled per pixel stream:
//   - the sample index is shuffled by a nested uniform scramble of its 16
//     low bits (Burley, "Practical Hash-based Owen Scrambling", JCGT 2020:
//     the Laine-Karras permutation between two bit reversals), seeded by the
//     stream's high word and, for the dimensions past the first six, a
//     second constant, so those restart the sequence's dimensions from 0;
//   - the dimension's Sobol point at that place, from direction numbers
//     built from the primitive polynomials and initial numbers of Joe and
//     Kuo (2008), read through two 256-entry tables of the place's bytes;
//   - the point's bits Laine-Karras scrambled with a seed of the stream and
//     the dimension, reversed, and scaled by 2^-32.
// The seeds' hash is Wellons' "lowbias32" integer hash.  Host and device
// share these functions; the tables are built on the host.
#pragma once

#include <cstddef>
#include <cstdint>

#ifdef __CUDACC__
#define KDN_HD __host__ __device__
#else
#define KDN_HD
#endif

namespace kdn {

constexpr uint32_t kSobolDimensions = 28; // sobol.h:13 sobolDimensions
constexpr uint32_t kSobolShared     = 6;  // sobol.h:21 sharedCoordinates
constexpr uint32_t kSobolTableWords = kSobolDimensions * 2 * 256;

KDN_HD inline uint32_t sobolStirred(uint32_t v) {
	v ^= v >> 16;
	v *= 0x7FEB352DU;
	v ^= v >> 15;
	v *= 0x846CA68BU;
	return v ^ (v >> 16);
}

KDN_HD inline uint32_t sobolReversed(uint32_t v) {
#ifdef __CUDA_ARCH__
	return __brev(v);
#else
	v = (v << 16) | (v >> 16);
	v = ((v & 0x00FF00FFU) << 8) | ((v & 0xFF00FF00U) >> 8);
	v = ((v & 0x0F0F0F0FU) << 4) | ((v & 0xF0F0F0F0U) >> 4);
	v = ((v & 0x33333333U) << 2) | ((v & 0xCCCCCCCCU) >> 2);
	return ((v & 0x55555555U) << 1) | ((v & 0xAAAAAAAAU) >> 1);
#endif
}

// the 16 low bits reversed
KDN_HD inline uint32_t sobolReversed16(uint32_t v) { return sobolReversed(v & 0xFFFFU) >> 16; }

// the Laine-Karras permutation (Burley 2020)
KDN_HD inline uint32_t laineKarras(uint32_t v, uint32_t seed) {
	v += seed;
	v ^= v * 0x6C50B47CU;
	v ^= v * 0xB82F1E52U;
	v ^= v * 0xC7AFE638U;
	return v ^ (v * 0x8D22F6E6U);
}

// sobol.cpp:121 pairPlace: the sample's shuffled place in the sequence
KDN_HD inline uint32_t sobolPlace(uint64_t stream, uint32_t index, uint32_t dimension) {
	const uint32_t own  = dimension < kSobolShared ? 0U : 0x68E31DA4U;
	const uint32_t seed = sobolStirred(uint32_t(stream >> 32) + own);
	return sobolReversed16(laineKarras(sobolReversed16(index), seed) & 0xFFFFU);
}

// sobol.cpp:130 placedNumber as its 32 bits (the number is bits * 2^-32)
KDN_HD inline uint32_t sobolBits(const uint32_t* tables, uint64_t stream, uint32_t index, uint32_t dimension) {
	const uint32_t place   = sobolPlace(stream, index, dimension);
	const uint32_t seed    = sobolStirred(uint32_t(stream >> 32) + dimension * 0xA136AAADU + 0x2545F491U);
	const uint32_t* column = tables + std::size_t(dimension < kSobolShared ? dimension : dimension - kSobolShared) * 512;
	const uint32_t value   = column[place & 0xFFU] ^ column[256 + ((place >> 8) & 0xFFU)];
	return sobolReversed(laineKarras(value, seed));
}

// The byte tables of the 28 dimensions: [dimension][low byte, high byte][256].
void buildSobolTables(uint32_t* out);

} // namespace kdn
