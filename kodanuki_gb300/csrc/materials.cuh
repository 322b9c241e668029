// BSDFs of the transport kernels (plugins/transport/paths/material/
// material.cpp and material/microfacet.cpp), in FP32 over the four
// hero-wavelength lanes:
//  - matte: Lambert (material.cpp:406 matteValue, :1173 matteScatter);
//  - metal: GGX facets with Schlick's Fresnel plus the lobe that gives back
//    what single scattering loses, read off the finish's escape table
//    (material.cpp:649 viewedMetal, energy.cpp:120 escapeAt);
//  - plastic: a Lambert body under a GGX coat of index 1.5
//    (material.cpp:661 viewedPlastic, :440 plasticShare);
//  - glass, smooth: exact mirror and passage by Fresnel, per lane where the
//    glass disperses (Cauchy), the passage bent by the hero lane's index
//    (material.cpp:1300 exactGlassScatter, feature/dispersion);
//  - glass, rough: GGX facets mirrored or bent (Walter et al. 2007), per
//    lane, plus the broad lobe that gives back what single scattering
//    loses, read off the finish's boundary tables (material.cpp:884
//    glassReflection, :986 glassPassage, :1328 glassScatter, energy.cpp:284
//    lossAt, :317 boundaryAt).
// Films are refused by the host.
#pragma once

#include "frame.h"

#include <cuda_runtime.h>

namespace kdn {

constexpr float kPiF     = 3.14159265358979f;
constexpr float kCoatIndex = 1.5f;        // material.cpp:10 coatIndex
constexpr float kCoatRatio = 1.0f / kCoatIndex;

struct Frame {
	float3 t, b, n;
	__device__ float3 toWorld(float3 v) const {
		return make_float3(t.x * v.x + b.x * v.y + n.x * v.z, t.y * v.x + b.y * v.y + n.y * v.z, t.z * v.x + b.z * v.y + n.z * v.z);
	}
	__device__ float3 toLocal(float3 v) const {
		return make_float3(t.x * v.x + t.y * v.y + t.z * v.z, b.x * v.x + b.y * v.y + b.z * v.z, n.x * v.x + n.y * v.y + n.z * v.z);
	}
};

// An orthonormal frame about a unit vector (Duff et al., "Building an
// Orthonormal Basis, Revisited", JCGT 2017).
__device__ __forceinline__ Frame frameAround(float3 n) {
	const float sign = copysignf(1.0f, n.z);
	const float a    = -1.0f / (sign + n.z);
	const float b    = n.x * n.y * a;
	Frame f;
	f.t = make_float3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
	f.b = make_float3(b, sign + n.y * n.y * a, -n.y);
	f.n = n;
	return f;
}

__device__ __forceinline__ float dotF(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 scaleF(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 addF(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 subF(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 unitF(float3 a) { return scaleF(a, 1.0f / sqrtf(dotF(a, a))); }
__device__ __forceinline__ float4 flat4(float v) { return make_float4(v, v, v, v); }
__device__ __forceinline__ float4 lin4(float4 a, float sa, float4 b, float sb) { return make_float4(a.x * sa + b.x * sb, a.y * sa + b.y * sb, a.z * sa + b.z * sb, a.w * sa + b.w * sb); }
__device__ __forceinline__ float lane4(float4 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w)); }

// math/vector.cpp:45 mirrored
__device__ __forceinline__ float3 mirrorOf(float3 v, float3 n) { return subF(scaleF(n, 2.0f * dotF(v, n)), v); }

// ---- microfacet.cpp ----
__device__ __forceinline__ float facetDistribution(float cosine, float width) {
	if (cosine <= 0.0f) return 0.0f;
	const float sq    = width * width;
	const float lower = cosine * cosine * (sq - 1.0f) + 1.0f;
	return sq / (kPiF * lower * lower);
}

__device__ __forceinline__ float smithVisibility(float leaving, float arriving, float width) {
	const float sq    = width * width;
	const float first = arriving * sqrtf(sq + (1.0f - sq) * leaving * leaving);
	const float second = leaving * sqrtf(sq + (1.0f - sq) * arriving * arriving);
	const float total = first + second;
	return total > 0.0f ? 0.5f / total : 0.0f;
}

__device__ __forceinline__ float smithMasking(float cosine, float width) {
	const float sq    = width * width;
	const float under = cosine + sqrtf(sq + (1.0f - sq) * cosine * cosine);
	return under > 0.0f ? 2.0f * cosine / under : 0.0f;
}

__device__ __forceinline__ float3 halfwayOf(float3 o, float3 i, float3 n) {
	const float3 total = addF(o, i);
	const float size   = sqrtf(dotF(total, total));
	return size > 1e-12f ? scaleF(total, 1.0f / size) : n;
}

// microfacet.cpp:67 visibleFacet: a facet drawn by its visible area from the
// outgoing direction (stretch, draw on the hemisphere seen from it, unstretch).
__device__ float3 visibleFacet(const Frame& f, float3 outgoing, float width, float u, float v) {
	const float3 local     = f.toLocal(outgoing);
	const float3 stretched = unitF(make_float3(width * local.x, width * local.y, local.z));
	const float flat       = stretched.x * stretched.x + stretched.y * stretched.y;
	const float3 first     = flat > 1e-12f ? scaleF(make_float3(-stretched.y, stretched.x, 0.0f), rsqrtf(flat)) : make_float3(1.0f, 0.0f, 0.0f);
	const float3 second    = make_float3(stretched.y * first.z - stretched.z * first.y, stretched.z * first.x - stretched.x * first.z, stretched.x * first.y - stretched.y * first.x);
	const float reach      = sqrtf(u);
	const float angle      = 2.0f * kPiF * v;
	const float across     = reach * cosf(angle);
	const float lean       = 0.5f * (1.0f + stretched.z);
	const float along      = (1.0f - lean) * sqrtf(fmaxf(1.0f - across * across, 0.0f)) + lean * reach * sinf(angle);
	const float height     = sqrtf(fmaxf(1.0f - across * across - along * along, 0.0f));
	const float3 raised    = addF(addF(scaleF(first, across), scaleF(second, along)), scaleF(stretched, height));
	const float3 unstretched = unitF(make_float3(width * raised.x, width * raised.y, fmaxf(raised.z, 1e-12f)));
	return f.toWorld(unstretched);
}

// microfacet.cpp:94 dielectricReflectance, ratio = index before / index after.
__device__ __forceinline__ float dielectricReflectance(float cosine, float ratio) {
	const float leftover = 1.0f - ratio * ratio * (1.0f - cosine * cosine);
	if (leftover <= 0.0f) return 1.0f;
	const float onward = sqrtf(leftover);
	const float perp   = (ratio * cosine - onward) / (ratio * cosine + onward);
	const float par    = (ratio * onward - cosine) / (ratio * onward + cosine);
	return 0.5f * (perp * perp + par * par);
}

// ---- thin films: a layer `thickness` nm deep of index `index` between an
// outside and a beneath index, thin enough that the light off its two faces
// interferes (material.cpp:106-172) ----

// material.cpp:143 bentCosine: the cosine past a crossing from index
// `before` into `after`, -1 where the crossing reflects totally
__device__ __forceinline__ float bentCosine(float before, float facing, float after) {
	const float sine = before / after * sqrtf(fmaxf(1.0f - facing * facing, 0.0f));
	return sine >= 1.0f ? -1.0f : sqrtf(1.0f - sine * sine);
}

// material.cpp:136 airySum: the reflectance of the two faces' amplitudes
// summed over every round trip inside the layer, `shift` the cosine of the
// phase one round trip adds
__device__ __forceinline__ float airySum(float front, float back, float shift) {
	const float both   = front * back;
	const float top    = front * front + back * back + 2.0f * both * shift;
	const float bottom = 1.0f + both * both + 2.0f * both * shift;
	return bottom > 0.0f ? fminf(fmaxf(top / bottom, 0.0f), 1.0f) : 1.0f;
}

// material.cpp:148 filmReflectance at one wavelength: the mean of the two
// polarisations' Airy sums over the front face (outside into the layer) and
// the back face (the layer into beneath), their amplitudes as
// material.cpp:129 faceAmplitude; 1 where either face reflects totally.
// The film functions are called, not inlined, so that the shading of
// unfilmed surfaces keeps its registers.
__device__ __noinline__ float filmReflectance(float thickness, float index, float facing, float nm, float outside, float beneath) {
	const float inside = bentCosine(outside, facing, index);
	const float beyond = inside < 0.0f ? -1.0f : bentCosine(index, inside, beneath);
	if (inside < 0.0f || beyond < 0.0f) return 1.0f;
	const float nearPerp = (outside * facing - index * inside) / (outside * facing + index * inside);
	const float nearPar  = (index * facing - outside * inside) / (index * facing + outside * inside);
	const float farPerp  = (index * inside - beneath * beyond) / (index * inside + beneath * beyond);
	const float farPar   = (beneath * inside - index * beyond) / (beneath * inside + index * beyond);
	const float shift    = cosf(4.0f * kPiF * index * thickness * inside / nm);
	return 0.5f * (airySum(nearPerp, farPerp, shift) + airySum(nearPar, farPar, shift));
}

// material.cpp:515 stackedFilm: a film in air over a reflector of
// reflectance `under` (a metal's facets), the light held between them
// summed
__device__ __forceinline__ float stackedFilm(float thickness, float index, float facing, float nm, float under) {
	if (!(thickness > 0.0f)) return under;
	const float front = filmReflectance(thickness, index, facing, nm, 1.0f, 1.0f);
	const float held  = fminf(fmaxf(under, 0.0f), 1.0f);
	const float room  = 1.0f - front * held;
	if (!(room > 1e-9f)) return 1.0f;
	return front + (1.0f - front) * (1.0f - front) * held / room;
}

// material.cpp:528 coatFacing: a plastic's coat at the cosine `onto` under
// its film (the film in air over the coat's index)
__device__ __forceinline__ float filmedCoatFacing(float thickness, float index, float onto, float nm) {
	return filmReflectance(thickness, index, onto, nm, 1.0f, kCoatIndex);
}

// material.cpp:592 metalTwice under a film: microfacet.cpp:116
// averagedFresnel `average` at the lanes, under the film facing straight on
__device__ __noinline__ float4 filmedMetalTwice(float4 average, float escapeAverage, float thickness, float index, float4 nm) {
	float t[4];
	for (int k = 0; k < 4; ++k) {
		const float flat = stackedFilm(thickness, index, 1.0f, lane4(nm, k), lane4(average, k));
		t[k]             = flat * flat * escapeAverage / (1.0f - flat * (1.0f - escapeAverage));
	}
	return make_float4(t[0], t[1], t[2], t[3]);
}

// material.cpp:651 viewedMetal's facet colour under a film: `face` (Schlick
// at the lanes) under the film at the cosine `onto`
__device__ __noinline__ float4 filmedMetalFace(float4 face, float onto, float thickness, float index, float4 nm) {
	return make_float4(stackedFilm(thickness, index, onto, nm.x, face.x), stackedFilm(thickness, index, onto, nm.y, face.y),
	                   stackedFilm(thickness, index, onto, nm.z, face.z), stackedFilm(thickness, index, onto, nm.w, face.w));
}

// material.cpp:661 viewedPlastic under a filmed coat: each lane's coat
// (:543 filmCoating, :604 laneCoats) at its own wavelength; `albedo` the
// body's colour at the lanes, `left`/`came` the escapes of the two
// directions, `facets` the facet term, `lost` material.cpp:620 lostOf
__device__ __noinline__ float4 filmedPlastic(float4 albedo, float left, float came, float escapeAverage, float onto, float facets, float lost, float thickness,
                                             float index, float4 nm) {
	float v[4];
	for (int k = 0; k < 4; ++k) {
		const float nmk     = lane4(nm, k);
		const float faced   = filmedCoatFacing(thickness, index, 1.0f, nmk);
		const float front   = faced + (1.0f - faced) / 21.0f;
		const float twice   = front * front * escapeAverage / (1.0f - front * (1.0f - escapeAverage));
		const float room    = 1.0f - front * escapeAverage;
		const float through = room > 1e-6f ? (1.0f - front * left) * (1.0f - front * came) / room : 0.0f;
		v[k] = lane4(albedo, k) / kPiF * through + filmedCoatFacing(thickness, index, onto, nmk) * facets + twice * lost;
	}
	return make_float4(v[0], v[1], v[2], v[3]);
}

// material.cpp:797 laneReflectance of a filmed glass at the four lanes
__device__ __noinline__ float4 filmedLanes(float thickness, float index, float cosine, float4 nm, float4 within, float4 beyond) {
	return make_float4(filmReflectance(thickness, index, cosine, nm.x, within.x, beyond.x), filmReflectance(thickness, index, cosine, nm.y, within.y, beyond.y),
	                   filmReflectance(thickness, index, cosine, nm.z, within.z, beyond.z), filmReflectance(thickness, index, cosine, nm.w, within.w, beyond.w));
}

// energy.cpp:120 escapeAt
__device__ __forceinline__ float escapeAt(const float* table, float cosine) {
	const float place = fminf(fmaxf(cosine, 0.0f), 1.0f) * 32.0f - 0.5f;
	const int lower   = min(max(int(floorf(place)), 0), 31);
	const int upper   = min(lower + 1, 31);
	const float share = fminf(fmaxf(place - float(lower), 0.0f), 1.0f);
	return table[lower] * (1.0f - share) + table[upper] * share;
}

// What a vertex's BSDF needs, worked out once per vertex (material.cpp:580
// roughViewed for the rough kinds).
struct Shading {
	uint32_t kind;
	float3 normal;
	Frame frame;
	float4 albedo;   // albedo at the lanes
	float leaving;   // cosine of the outgoing direction
	float left;      // escapeAt(leaving)
	float share;     // chance of the facet lobe when sampling
	float masking;   // smithMasking(leaving)
	float4 twice;    // metal: the colour light keeps over many bounces
	float4 within, beyond; // glass: index on either side, per lane
	bool parted;     // the lanes answer apart (a dispersing or filmed glass)
	bool inside;     // glass: the vertex is seen from inside the body
	float width;     // glass: GGX width of the facets
	const float* boundary; // rough glass that loses much: its boundary tables
	float filmThickness, filmIndex; // the film it wears (thickness 0: none)
	float4 nm;       // the lanes' wavelengths
};

struct Response {
	float4 value;
	float density;
};

struct Scatter {
	bool found;
	bool through;
	bool delta;
	bool dispersed;
	float3 incoming;
	float4 weight;     // value * |cosine| / density, or the kept share of an exact side
	float density;
	uint32_t mediumAfter;
};

// math/spectrum.cpp:42-60: the smooth basis curves RGB is upsampled by.
__device__ __forceinline__ float smoothRise(float nm, float lo, float hi) {
	const float b = fminf(fmaxf((nm - lo) / (hi - lo), 0.0f), 1.0f);
	return b * b * (3.0f - 2.0f * b);
}

__device__ __forceinline__ float basisOf(int channel, float nm) {
	const float red  = smoothRise(nm, 575.0f, 605.0f);
	const float blue = 1.0f - smoothRise(nm, 445.0f, 530.0f);
	return channel == 0 ? red : (channel == 2 ? blue : (1.0f - blue) * (1.0f - red));
}

// math/colour.cpp:85 spectrumOf: an RGB colour at the four lanes, from its
// least channel, the rise to the middle one and the rise to the most one.
__device__ __forceinline__ float4 spectrumOf(float r, float g, float b, float4 nm) {
	const float c[3] = { r, g, b };
	int least;
	if (r <= g && r <= b) least = 0;
	else least = (g <= r && g <= b) ? 1 : 2;
	const int first  = least == 0 ? 1 : 0;
	const int second = least == 2 ? 1 : 2;
	const int most   = c[first] <= c[second] ? second : first;
	const int middle = 3 - least - most;
	const float base = c[least];
	const float low  = c[middle] - base;
	const float high = c[most] - c[middle];
	const float lanes[4] = { nm.x, nm.y, nm.z, nm.w };
	float out[4];
	for (int k = 0; k < 4; ++k) out[k] = base + low * (1.0f - basisOf(least, lanes[k])) + high * basisOf(most, lanes[k]);
	return make_float4(out[0], out[1], out[2], out[3]);
}

// feature/dispersion/dispersion.cpp cauchyIndex: A + B / lambda^2, lambda in micrometres.
__device__ __forceinline__ float4 laneIndices(const DeviceMaterial& m, float4 nm) {
	if (m.dispersion == 0.0f) return flat4(m.index);
	const float l0 = nm.x * 1e-3f, l1 = nm.y * 1e-3f, l2 = nm.z * 1e-3f, l3 = nm.w * 1e-3f;
	return make_float4(m.index + m.dispersion / (l0 * l0), m.index + m.dispersion / (l1 * l1), m.index + m.dispersion / (l2 * l2), m.index + m.dispersion / (l3 * l3));
}

__device__ __forceinline__ float plasticShare(const DeviceMaterial& m, float leaving) {
	const float face  = dielectricReflectance(leaving, kCoatRatio);
	const float share = face / fmaxf(face + (1.0f - face) * m.body, 1e-12f);
	return fminf(fmaxf(share, 0.25f), 0.9f);
}

// rgb: the albedo at the hit (the material's, or mixed across a blend seam).
// Films: the frame's scene wears a thin film somewhere; without, the film
// fields are the constant 0 and every film branch folds away.
template <bool Films>
__device__ __forceinline__ Shading surfaceOf(const DeviceMaterial& m, float3 rgb, float3 normal, float3 outgoing, float4 nm, uint32_t medium, const DeviceMaterial* all,
                                             const float* boundaries) {
	Shading s;
	s.kind    = m.kind;
	s.normal  = normal;
	s.frame   = frameAround(normal);
	s.albedo  = spectrumOf(rgb.x, rgb.y, rgb.z, nm);
	s.leaving = dotF(normal, outgoing);
	s.left    = 0.0f;
	s.share   = 0.0f;
	s.masking = 0.0f;
	s.twice   = flat4(0.0f);
	s.within  = flat4(1.0f);
	s.beyond  = flat4(1.0f);
	s.parted  = false;
	s.inside  = medium != kNoMaterial;
	s.width   = m.width;
	s.boundary = (m.kind == 3 && m.losesMuch && boundaries != nullptr) ? boundaries + size_t(m.boundaryFirst) * kBoundaryFloats : nullptr;
	s.filmThickness = Films ? m.filmThickness : 0.0f;
	s.filmIndex     = Films ? m.filmIndex : 1.0f;
	s.nm            = nm;
	if (m.kind == 1 || m.kind == 2) {
		s.left    = escapeAt(m.escape, s.leaving);
		s.share   = m.kind == 2 ? m.facetShare : (s.leaving <= 0.0f ? 0.0f : plasticShare(m, s.leaving));
		s.masking = smithMasking(s.leaving, m.width);
		if (m.kind == 2) {
			// microfacet.cpp:116 averagedFresnel under the film facing
			// straight on, then material.cpp:592 metalTwice
			const float4 avg = lin4(s.albedo, 1.0f - 1.0f / 21.0f, flat4(1.0f), 1.0f / 21.0f);
			const float e    = m.escapeAverage;
			if (s.filmThickness > 0.0f) {
				s.twice = filmedMetalTwice(avg, e, s.filmThickness, s.filmIndex, nm);
			} else {
				const float a[4] = { avg.x, avg.y, avg.z, avg.w };
				float t[4];
				for (int k = 0; k < 4; ++k) t[k] = a[k] * a[k] * e / (1.0f - a[k] * (1.0f - e));
				s.twice = make_float4(t[0], t[1], t[2], t[3]);
			}
		}
	} else if (m.kind == 3) {
		// material.cpp:328 sidesOf with feature/dispersion's per-lane
		// indices (dispersion.cpp:60 dispersedSides); a filmed glass answers
		// each lane at its own wavelength (dispersion.cpp:38 filmedSides)
		if (medium != kNoMaterial) {
			const DeviceMaterial& body = all[medium];
			s.within = laneIndices(body, nm);
			s.parted = body.dispersion != 0.0f;
		} else {
			s.beyond = laneIndices(m, nm);
			s.parted = m.dispersion != 0.0f;
		}
		s.parted = s.parted || s.filmThickness > 0.0f;
	}
	return s;
}

// material.cpp:620 lostOf
__device__ __forceinline__ float lostOf(const DeviceMaterial& m, float left, float came) {
	const float room = 1.0f - m.escapeAverage;
	if (room <= 1e-6f) return 0.0f;
	return (1.0f - left) * (1.0f - came) / (kPiF * room);
}

// ---- rough glass ----
struct TableRow {
	int lower, upper;
	float share;
};

// energy.cpp:255 rowOf: the place of the indices' ratio among the rows (1 to 3)
__device__ __forceinline__ TableRow rowOf(float near, float far) {
	const float ratio = fmaxf(near, far) / fminf(near, far);
	const float place = (fminf(ratio, 3.0f) - 1.0f) / 2.0f * float(kBoundaryRatios - 1);
	TableRow r;
	r.lower = min(max(int(floorf(place)), 0), kBoundaryRatios - 1);
	r.upper = min(r.lower + 1, kBoundaryRatios - 1);
	r.share = fminf(fmaxf(place - float(r.lower), 0.0f), 1.0f);
	return r;
}

__device__ __forceinline__ float blendedRow(const float* v, TableRow r) { return v[r.lower] * (1.0f - r.share) + v[r.upper] * r.share; }

struct Loss {
	float back, through, share;
};

// energy.cpp:284 lossAt (its back, through and share)
__device__ Loss lossAt(const float* b, float near, float far) {
	const TableRow row   = rowOf(near, far);
	const float* tail    = b + 2 * kBoundaryRatios * kBoundaryViews;
	const float rarer    = blendedRow(tail, row);
	const float denser   = blendedRow(tail + kBoundaryRatios, row);
	const float share    = blendedRow(tail + 2 * kBoundaryRatios, row);
	const bool fromRarer = near <= far;
	const float nearAvg  = fromRarer ? rarer : denser;
	const float farAvg   = fromRarer ? denser : rarer;
	Loss l { 0.0f, 0.0f, 0.0f };
	const float nearLost = 1.0f - nearAvg, denserLost = 1.0f - denser;
	if (!(nearLost > 1e-9f) || !(denserLost > 1e-9f)) return l;
	const float turned = (far / near) * (far / near);
	l.through          = fromRarer ? share / denserLost : share / denserLost * turned;
	const float given  = fminf(l.through * (1.0f - farAvg), 1.0f);
	l.back             = (1.0f - given) / nearLost;
	l.share            = given;
	return l;
}

// energy.cpp:309 rowAt, :317 boundaryAt, material.cpp:780 lossLeft
__device__ __forceinline__ float rowAt(const float* table, int row, float cosine) {
	const float place = fminf(fmaxf(cosine, 0.0f), 1.0f) * float(kBoundaryViews) - 0.5f;
	const int lower   = min(max(int(floorf(place)), 0), kBoundaryViews - 1);
	const int upper   = min(lower + 1, kBoundaryViews - 1);
	const float share = fminf(fmaxf(place - float(lower), 0.0f), 1.0f);
	return table[row * kBoundaryViews + lower] * (1.0f - share) + table[row * kBoundaryViews + upper] * share;
}

__device__ float lossLeft(const float* b, float near, float far, float cosine) {
	const TableRow row  = rowOf(near, far);
	const float* table  = near <= far ? b : b + kBoundaryRatios * kBoundaryViews;
	const float reached = rowAt(table, row.lower, cosine) * (1.0f - row.share) + rowAt(table, row.upper, cosine) * row.share;
	return fmaxf(1.0f - reached, 0.0f);
}

struct Broad {
	float share, through;
};

// material.cpp:789 broadOf over the hero lane's indices
__device__ __forceinline__ Broad broadOf(const Shading& s, float leaving) {
	Broad w { 0.0f, 0.0f };
	if (s.boundary != nullptr) {
		w.share   = fminf(fmaxf(lossLeft(s.boundary, s.within.x, s.beyond.x, leaving), 0.0f), 1.0f);
		w.through = lossAt(s.boundary, s.within.x, s.beyond.x).share;
	}
	return w;
}

// material.cpp:797 laneReflectance (Fresnel, or the film between the two
// sides at lane k's wavelength), :814 laneReflectances, :821 reflectChance
__device__ __forceinline__ float laneReflectance(const Shading& s, float cosine, int k) {
	const float within = lane4(s.within, k), beyond = lane4(s.beyond, k);
	if (!(s.filmThickness > 0.0f)) return dielectricReflectance(cosine, within / beyond);
	return filmReflectance(s.filmThickness, s.filmIndex, cosine, lane4(s.nm, k), within, beyond);
}

__device__ __forceinline__ float4 laneReflectances(const Shading& s, float cosine) {
	if (s.filmThickness > 0.0f) return filmedLanes(s.filmThickness, s.filmIndex, cosine, s.nm, s.within, s.beyond); // a filmed glass is parted
	if (!s.parted) return flat4(laneReflectance(s, cosine, 0));
	return make_float4(laneReflectance(s, cosine, 0), laneReflectance(s, cosine, 1), laneReflectance(s, cosine, 2), laneReflectance(s, cosine, 3));
}

__device__ __forceinline__ float reflectChance(const Shading& s, float cosine) {
	if (!s.parted) return laneReflectance(s, cosine, 0);
	const float4 r = laneReflectances(s, cosine);
	return 0.25f * (r.x + r.y + r.z + r.w);
}

// material.cpp:836 reflectanceAcross: from the denser side, Fresnel (or the
// film, :825 filmedFromDenser) of the arriving cosine
__device__ __forceinline__ float reflectanceAcross(const Shading& s, float leaving, float arriving, int k) {
	const float within = lane4(s.within, k), beyond = lane4(s.beyond, k);
	if (within <= beyond) return laneReflectance(s, leaving, k);
	if (s.filmThickness > 0.0f) return filmReflectance(s.filmThickness, s.filmIndex, arriving, lane4(s.nm, k), beyond, within);
	return dielectricReflectance(arriving, beyond / within);
}

// material.cpp:846 backLoss, :850 throughLoss, :859 givenBack
__device__ float4 givenBack(const Shading& s, float leaving, float arriving, bool through) {
	if (s.boundary == nullptr) return flat4(0.0f);
	const int lanes = s.parted ? 4 : 1;
	float g[4]      = { 0.0f, 0.0f, 0.0f, 0.0f };
	for (int k = 0; k < lanes; ++k) {
		const float near = lane4(s.within, k), far = lane4(s.beyond, k);
		const Loss l     = lossAt(s.boundary, near, far);
		g[k] = through ? l.through * lossLeft(s.boundary, near, far, leaving) * lossLeft(s.boundary, far, near, -arriving) / kPiF
		               : l.back * lossLeft(s.boundary, near, far, leaving) * lossLeft(s.boundary, near, far, arriving) / kPiF;
	}
	return s.parted ? make_float4(g[0], g[1], g[2], g[3]) : flat4(g[0]);
}

// material.cpp:884 glassReflection
__device__ Response glassReflection(const Shading& s, float3 outgoing, float3 incoming, float leaving, float arriving) {
	const float3 facet  = halfwayOf(outgoing, incoming, s.normal);
	const float onto    = dotF(outgoing, facet);
	const float4 each   = laneReflectances(s, fmaxf(onto, 0.0f));
	const float lobe    = onto > 0.0f ? facetDistribution(dotF(s.normal, facet), s.width) : 0.0f;
	const float back    = s.parted ? 0.25f * (each.x + each.y + each.z + each.w) : each.x;
	const float facets  = lobe * smithMasking(leaving, s.width) / (4.0f * leaving);
	const Broad wide    = broadOf(s, leaving);
	Response r;
	r.value   = lin4(each, lobe * smithVisibility(leaving, arriving, s.width), givenBack(s, leaving, arriving, false), 1.0f);
	r.density = (1.0f - wide.share) * back * facets + wide.share * (1.0f - wide.through) * arriving / kPiF;
	return r;
}

// material.cpp:947 lanePassage over :925 bentFacet: what lane k sends
// through the facet that bends the outgoing into the incoming direction,
// and (lane 0) the density of drawing it
__device__ void lanePassage(const Shading& s, float3 outgoing, float3 incoming, float leaving, float arriving, int k, float& sent, float& facets) {
	sent = facets     = 0.0f;
	const float near  = lane4(s.within, k), far = lane4(s.beyond, k);
	const float3 sum  = addF(scaleF(outgoing, near), scaleF(incoming, far));
	const float size  = sqrtf(dotF(sum, sum));
	if (!(size > 1e-12f)) return;
	const float3 facet = scaleF(sum, (dotF(sum, s.normal) < 0.0f ? -1.0f : 1.0f) / size);
	const float into   = dotF(incoming, facet);
	if (dotF(outgoing, facet) <= 0.0f || into >= 0.0f) return;
	const float stretch = far * far * -into / (size * size);
	if (stretch <= 0.0f) return;
	const float onto = dotF(outgoing, facet);
	const float lobe = facetDistribution(dotF(s.normal, facet), s.width) * onto * stretch;
	const float kept = 1.0f - reflectanceAcross(s, onto, -into, k);
	sent             = kept * lobe * 4.0f * smithVisibility(leaving, -arriving, s.width);
	facets           = (1.0f - reflectChance(s, onto)) * lobe * smithMasking(leaving, s.width) / leaving;
}

// material.cpp:986 glassPassage
__device__ Response glassPassage(const Shading& s, float3 outgoing, float3 incoming, float leaving, float arriving) {
	const int lanes = s.parted ? 4 : 1;
	float sent[4]   = { 0.0f, 0.0f, 0.0f, 0.0f };
	float facets    = 0.0f;
	for (int k = 0; k < lanes; ++k) {
		float f;
		lanePassage(s, outgoing, incoming, leaving, arriving, k, sent[k], f);
		if (k == 0) facets = f;
	}
	const Broad wide = broadOf(s, leaving);
	const float4 bent = s.parted ? make_float4(sent[0], sent[1], sent[2], sent[3]) : flat4(sent[0]);
	Response r;
	r.value   = lin4(bent, 1.0f, givenBack(s, leaving, arriving, true), 1.0f);
	r.density = (1.0f - wide.share) * facets + wide.share * wide.through * -arriving / kPiF;
	return r;
}

// The value and density of the BSDF for one pair of directions
// (material.cpp:1076 respondBsdf / :710 roughViewedAnswer).
__device__ __forceinline__ Response respond(const Shading& s, const DeviceMaterial& m, float3 outgoing, float3 incoming, float4 nm) {
	Response r;
	r.value              = flat4(0.0f);
	const float arriving = dotF(s.normal, incoming);
	if (s.kind == 0) {
		r.density = fmaxf(arriving, 0.0f) / kPiF;
		if (s.leaving > 0.0f && arriving > 0.0f) r.value = lin4(s.albedo, 1.0f / kPiF, flat4(0.0f), 0.0f);
		return r;
	}
	if (s.kind == 3) {
		// material.cpp:1002 glassResponse: exact glass answers no direction
		// not drawn by it
		r.density = 0.0f;
		if (s.leaving <= 0.0f || m.exact) return r;
		return arriving < 0.0f ? glassPassage(s, outgoing, incoming, s.leaving, arriving) : glassReflection(s, outgoing, incoming, s.leaving, arriving);
	}
	const float cosineDensity = fmaxf(arriving, 0.0f) / kPiF;
	if (s.leaving <= 0.0f || arriving <= 0.0f) {
		// material.cpp:447 roughDensity of a shadowed pair
		r.density = (s.kind == 1 && s.leaving <= 0.0f) ? 0.0f : (1.0f - s.share) * cosineDensity;
		return r;
	}
	const float3 h     = halfwayOf(outgoing, incoming, s.normal);
	const float tilt   = dotF(s.normal, h);
	const float D      = facetDistribution(tilt, m.width);
	const float came   = escapeAt(m.escape, arriving);
	const float ontoRaw = dotF(outgoing, h);
	const float onto   = fmaxf(ontoRaw, 0.0f);
	const float facets = D * smithVisibility(s.leaving, arriving, m.width);
	const float lost   = lostOf(m, s.left, came);
	if (s.kind == 2) {
		// material.cpp:651 viewedMetal: Schlick per channel, then to lanes
		// (spectrumOf is linear in a shift toward white), under the film
		const float rest = powf(fminf(fmaxf(1.0f - onto, 0.0f), 1.0f), 5.0f);
		float4 face      = lin4(s.albedo, 1.0f - rest, flat4(1.0f), rest);
		if (s.filmThickness > 0.0f) face = filmedMetalFace(face, onto, s.filmThickness, s.filmIndex, s.nm);
		r.value = lin4(face, facets, s.twice, lost);
	} else if (!(s.filmThickness > 0.0f)) {
		// material.cpp:661 viewedPlastic
		const float through = m.coatRoom > 1e-6f ? (1.0f - m.coatFront * s.left) * (1.0f - m.coatFront * came) / m.coatRoom : 0.0f;
		const float coated  = dielectricReflectance(onto, kCoatRatio) * facets + m.coatTwice * lost;
		r.value             = lin4(s.albedo, through / kPiF, flat4(1.0f), coated);
	} else {
		r.value = filmedPlastic(s.albedo, s.left, came, m.escapeAverage, onto, facets, lost, s.filmThickness, s.filmIndex, s.nm);
	}
	const float facetDensity = ontoRaw <= 0.0f ? 0.0f : D * s.masking / (4.0f * s.leaving);
	r.density                = s.share * facetDensity + (1.0f - s.share) * cosineDensity;
	return r;
}

__device__ __forceinline__ Scatter noScatter() {
	Scatter out;
	out.found       = false;
	out.through     = false;
	out.delta       = false;
	out.dispersed   = false;
	out.incoming    = make_float3(0.0f, 0.0f, 1.0f);
	out.weight      = flat4(0.0f);
	out.density     = 0.0f;
	out.mediumAfter = kNoMaterial;
	return out;
}

// material.cpp:1398 sampleBsdf
__device__ __forceinline__ Scatter sampleSurface(const Shading& s, const DeviceMaterial& m, float3 outgoing, float4 nm, float lobe, float side, float u, float v, uint32_t material, uint32_t medium) {
	Scatter out = noScatter();
	if (s.kind == 0) {
		const float reach  = sqrtf(u);
		const float angle  = 2.0f * kPiF * v;
		const float height = sqrtf(fmaxf(1.0f - u, 0.0f));
		out.incoming       = s.frame.toWorld(make_float3(reach * cosf(angle), reach * sinf(angle), height));
		out.density        = fmaxf(dotF(s.normal, out.incoming), 0.0f) / kPiF;
		out.found          = out.density > 0.0f;
		out.weight         = s.albedo;
		return out;
	}
	if (s.kind == 1 || s.kind == 2) {
		// material.cpp:1198 roughScatter
		if (s.leaving <= 0.0f) return out;
		const bool facetLobe = lobe < s.share;
		const float3 facet   = visibleFacet(s.frame, outgoing, m.width, u, v);
		float3 incoming;
		if (facetLobe) {
			incoming = mirrorOf(outgoing, facet);
		} else {
			const float reach  = sqrtf(u);
			const float angle  = 2.0f * kPiF * v;
			const float height = sqrtf(fmaxf(1.0f - u, 0.0f));
			incoming           = s.frame.toWorld(make_float3(reach * cosf(angle), reach * sinf(angle), height));
		}
		const float arriving = dotF(s.normal, incoming);
		if ((facetLobe && dotF(outgoing, facet) <= 0.0f) || arriving <= 0.0f) return out;
		const Response r = respond(s, m, outgoing, incoming, nm);
		if (r.density <= 0.0f) return out;
		out.found    = true;
		out.incoming = incoming;
		out.density  = r.density;
		out.weight   = lin4(r.value, fabsf(arriving) / r.density, flat4(0.0f), 0.0f);
		return out;
	}
	if (!m.exact) {
		// material.cpp:1328 glassScatter: the broad lobe (cosine about either
		// side, :1236 broadChoice) or a visible facet, mirrored or bent by the
		// hero lane (:1246 facetChoice)
		const float leaving = s.leaving;
		if (leaving <= 0.0f) return out;
		const Broad wide = broadOf(s, leaving);
		bool found = true, reflected;
		float3 incoming;
		if (lobe < wide.share) {
			reflected          = side >= wide.through;
			const Frame around = frameAround(reflected ? s.normal : scaleF(s.normal, -1.0f));
			const float reach  = sqrtf(u);
			const float angle  = 2.0f * kPiF * v;
			const float height = sqrtf(fmaxf(1.0f - u, 0.0f));
			incoming           = around.toWorld(make_float3(reach * cosf(angle), reach * sinf(angle), height));
		} else {
			const float3 facet = visibleFacet(s.frame, outgoing, s.width, u, v);
			const float onto   = dotF(outgoing, facet);
			if (onto <= 0.0f) return out;
			reflected = side < reflectChance(s, onto);
			if (reflected) {
				incoming = mirrorOf(outgoing, facet);
			} else {
				const float ratio    = s.within.x / s.beyond.x;
				const float leftover = 1.0f - ratio * ratio * (1.0f - onto * onto);
				found                = leftover > 0.0f;
				incoming             = found ? subF(scaleF(subF(scaleF(facet, onto), outgoing), ratio), scaleF(facet, sqrtf(leftover))) : make_float3(0.0f, 0.0f, 0.0f);
			}
		}
		const float arriving = dotF(s.normal, incoming);
		if (!found || (reflected ? arriving <= 0.0f : arriving >= 0.0f)) return out;
		const Response r = reflected ? glassReflection(s, outgoing, incoming, leaving, arriving) : glassPassage(s, outgoing, incoming, leaving, arriving);
		if (r.density <= 0.0f) return out;
		out.found       = true;
		out.incoming    = incoming;
		out.density     = r.density;
		out.weight      = lin4(r.value, fabsf(arriving) / r.density, flat4(0.0f), 0.0f);
		out.through     = !reflected;
		out.dispersed   = out.through && s.parted && s.within.x != s.beyond.x;
		out.mediumAfter = out.through ? (medium != kNoMaterial ? kNoMaterial : material) : kNoMaterial;
		return out;
	}
	// material.cpp:1300 exactGlassScatter
	if (s.leaving <= 0.0f) return out;
	float refl[4];
	if (s.filmThickness > 0.0f) {
		const float4 r = filmedLanes(s.filmThickness, s.filmIndex, s.leaving, s.nm, s.within, s.beyond);
		refl[0] = r.x, refl[1] = r.y, refl[2] = r.z, refl[3] = r.w;
	} else {
		for (int k = 0; k < 4; ++k) refl[k] = dielectricReflectance(s.leaving, lane4(s.within, k) / lane4(s.beyond, k));
		if (!s.parted) refl[1] = refl[2] = refl[3] = refl[0];
	}
	const float chance   = s.parted ? 0.25f * (refl[0] + refl[1] + refl[2] + refl[3]) : refl[0];
	const float ratio    = s.within.x / s.beyond.x;
	const float leftover = 1.0f - ratio * ratio * (1.0f - s.leaving * s.leaving);
	const bool passed    = leftover > 0.0f;
	out.delta            = true;
	out.found            = true;
	out.density          = 0.0f;
	if (side < chance || !passed) {
		const float c  = passed ? chance : 1.0f;
		out.incoming   = mirrorOf(outgoing, s.normal);
		out.weight     = make_float4(refl[0] / c, refl[1] / c, refl[2] / c, refl[3] / c);
		out.through    = false;
		return out;
	}
	const float c        = 1.0f - chance;
	out.incoming         = subF(scaleF(subF(scaleF(s.normal, s.leaving), outgoing), ratio), scaleF(s.normal, sqrtf(leftover)));
	out.weight           = make_float4((1.0f - refl[0]) / c, (1.0f - refl[1]) / c, (1.0f - refl[2]) / c, (1.0f - refl[3]) / c);
	out.through          = true;
	out.dispersed        = s.parted && s.within.x != s.beyond.x;
	out.mediumAfter      = medium != kNoMaterial ? kNoMaterial : material;
	return out;
}

} // namespace kdn
