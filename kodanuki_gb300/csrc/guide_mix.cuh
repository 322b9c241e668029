// The learned guide's mixture of eight von Mises-Fisher lobes, as the
// transport reads it: per query 40 floats, lobe j at 5j holding its weight,
// its concentration and its mean direction.  Density and sampling follow
// Jakob 2012 ("Numerically stable sampling of the von Mises-Fisher
// distribution on S2"): v(w) = k / (2 pi (1 - e^-2k)) exp(k (mu . w - 1)).
#pragma once

#include "guide.h"

#include <cuda_runtime.h>

namespace kdn {

__device__ __forceinline__ float vmfDensity(float kappa, float cosine) {
	return kappa / (6.283185307179586f * (1.0f - __expf(-2.0f * kappa))) * __expf(kappa * (cosine - 1.0f));
}

__device__ __forceinline__ float mixtureDensity(const float* lobes, float3 w) {
	float q = 0.0f;
#pragma unroll
	for (int j = 0; j < kGuideLobes; ++j) {
		const float* L = lobes + 5 * j;
		q += L[0] * vmfDensity(L[1], L[2] * w.x + L[3] * w.y + L[4] * w.z);
	}
	return q;
}

// A direction of the mixture: the lobe by its weight (u), then the vMF by
// inverting its cosine (du) and a turn about the mean (dv).
__device__ __forceinline__ float3 mixtureSample(const float* lobes, float u, float du, float dv) {
	int j     = kGuideLobes - 1;
	float cdf = 0.0f;
	for (int i = 0; i < kGuideLobes; ++i) {
		cdf += lobes[5 * i];
		if (u < cdf) {
			j = i;
			break;
		}
	}
	const float* L = lobes + 5 * j;
	const float k  = L[1];
	const float3 m = make_float3(L[2], L[3], L[4]);
	float w        = 1.0f + __logf(du + (1.0f - du) * __expf(-2.0f * k)) / k;
	w              = fminf(fmaxf(w, -1.0f), 1.0f);
	const float s  = sqrtf(fmaxf(0.0f, 1.0f - w * w));
	const float phi = 6.283185307179586f * dv;
	float3 t        = fabsf(m.x) > 0.9f ? make_float3(0.0f, 1.0f, 0.0f) : make_float3(1.0f, 0.0f, 0.0f);
	float3 a        = make_float3(m.y * t.z - m.z * t.y, m.z * t.x - m.x * t.z, m.x * t.y - m.y * t.x);
	const float al  = rsqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
	a               = make_float3(a.x * al, a.y * al, a.z * al);
	const float3 b  = make_float3(m.y * a.z - m.z * a.y, m.z * a.x - m.x * a.z, m.x * a.y - m.y * a.x);
	float sp, cp;
	__sincosf(phi, &sp, &cp);
	return make_float3(w * m.x + s * (cp * a.x + sp * b.x), w * m.y + s * (cp * a.y + sp * b.y), w * m.z + s * (cp * a.z + sp * b.z));
}

} // namespace kdn
