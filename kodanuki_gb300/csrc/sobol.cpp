// The Sobol byte tables of `--use sampler=sobol` (plugins/sampler/sobol/
// sobol.cpp:112 builtTable), built on the host.
#include "sobol.h"

namespace kdn {

namespace {

// A dimension's primitive polynomial (its degree and the bits of its inner
// coefficients) and initial direction numbers: dimension 0 is the van der
// Corput sequence (every direction number 1), the others the first 27 of
// Joe and Kuo's published set (new-joe-kuo-6.21201), which the reference's
// table holds too: the points must be the same.
struct Primitive {
	int degree;
	int inner;
	uint32_t initial[7];
};

constexpr Primitive kPrimitives[kSobolDimensions] = {
	{ 0, 0, { 1, 1, 1, 1, 1, 1, 1 } },   { 1, 0, { 1 } },
	{ 2, 1, { 1, 3 } },                  { 3, 1, { 1, 3, 1 } },
	{ 3, 2, { 1, 1, 1 } },               { 4, 1, { 1, 1, 3, 3 } },
	{ 4, 4, { 1, 3, 5, 13 } },           { 5, 2, { 1, 1, 5, 5, 17 } },
	{ 5, 4, { 1, 1, 5, 5, 5 } },         { 5, 7, { 1, 1, 7, 11, 19 } },
	{ 5, 11, { 1, 1, 5, 1, 1 } },        { 5, 13, { 1, 1, 1, 3, 11 } },
	{ 5, 14, { 1, 3, 5, 5, 31 } },       { 6, 1, { 1, 3, 3, 9, 7, 49 } },
	{ 6, 13, { 1, 1, 1, 15, 21, 21 } },  { 6, 16, { 1, 3, 1, 13, 27, 49 } },
	{ 6, 19, { 1, 1, 1, 15, 7, 5 } },    { 6, 22, { 1, 3, 1, 15, 13, 25 } },
	{ 6, 25, { 1, 1, 5, 5, 19, 61 } },   { 7, 1, { 1, 3, 7, 11, 23, 15, 103 } },
	{ 7, 4, { 1, 3, 7, 13, 13, 15, 69 } }, { 7, 7, { 1, 1, 3, 13, 7, 35, 63 } },
	{ 7, 8, { 1, 3, 5, 9, 1, 25, 53 } }, { 7, 14, { 1, 3, 1, 13, 9, 35, 107 } },
	{ 7, 19, { 1, 3, 1, 5, 27, 61, 31 } }, { 7, 21, { 1, 1, 5, 11, 19, 41, 61 } },
	{ 7, 28, { 1, 3, 5, 3, 3, 13, 69 } }, { 7, 31, { 1, 1, 7, 13, 1, 19, 1 } },
};

constexpr int kBits = 16;

// The 16 direction numbers m_1..m_16 of a dimension: the initial ones, then
// Bratley and Fox's recurrence over the polynomial's coefficients.
void directions(const Primitive& p, uint32_t m[kBits]) {
	for (int bit = 0; bit < kBits; ++bit) {
		if (p.degree == 0) {
			m[bit] = p.initial[0];
			continue;
		}
		if (bit < p.degree) {
			m[bit] = p.initial[bit];
			continue;
		}
		uint32_t v = m[bit - p.degree] ^ (m[bit - p.degree] << p.degree);
		for (int k = 1; k < p.degree; ++k) {
			if ((p.inner >> (p.degree - 1 - k)) & 1) v ^= m[bit - k] << k;
		}
		m[bit] = v;
	}
}

// The point of a place's set bits: the direction numbers as 32-bit
// fractions, each bit reversed, summed by XOR.
uint32_t pointBits(const uint32_t m[kBits], uint32_t place) {
	uint32_t value = 0;
	for (int bit = 0; bit < kBits; ++bit) {
		if ((place >> bit) & 1U) value ^= sobolReversed(m[bit] << (31 - bit));
	}
	return value;
}

} // namespace

void buildSobolTables(uint32_t* out) {
	for (uint32_t d = 0; d < kSobolDimensions; ++d) {
		uint32_t m[kBits];
		directions(kPrimitives[d], m);
		for (uint32_t byte = 0; byte < 256; ++byte) {
			out[d * 512 + byte]       = pointBits(m, byte);
			out[d * 512 + 256 + byte] = pointBits(m, byte << 8);
		}
	}
}

} // namespace kdn
