// Device evaluation of a leaf's kept programs (sdf/program.cpp:57 runStep),
// in single precision.
//
//  - evalSlots: the march's form.  Values live in register slots held in
//    shared memory, one column per thread: slot s of thread t is at
//    slots[s * blockDim.x + t], so a warp's accesses to one slot hit 32
//    consecutive banks.
//  - evalDual:  the value and gradient (forward mode, sdf/numbers.cpp:440
//    Dual) over the same slots, 4 floats a slot.
//  - evalSsa:   every step's value kept by step number, for the walk back from
//    the result that names the source leaf (sdf/program.cpp:478).
#pragma once

#include "world.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

// The march form's interpreter compiles for the host too, where
// kdn_world_march runs it to check the march form against the programs.
#define KDN_HD __host__ __device__ __forceinline__

namespace kdn {

KDN_HD float floatOfBits(uint32_t bits) {
#ifdef __CUDA_ARCH__
	return __uint_as_float(bits);
#else
	float f;
	std::memcpy(&f, &bits, sizeof f);
	return f;
#endif
}

KDN_HD float smoothMinF(float a, float b, float r) {
	const float blend = fmaxf(r - fabsf(a - b), 0.0f) / r;
	return fminf(a, b) - blend * blend * r * 0.25f;
}

KDN_HD float truthF(bool b) { return b ? 1.0f : 0.0f; }

// The march's square root: the hardware's approximate one on the device
// (PTX sqrt.approx.f32, relative error within 2^-22), correctly rounded on
// the host.
KDN_HD float marchSqrt(float x) {
#ifdef __CUDA_ARCH__
	float r;
	asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
	return r;
#else
	return sqrtf(x);
#endif
}

KDN_HD float stepValue(uint8_t op, float a, float b, float c, float value, const float p[3]) {
	switch (op) {
		case OpConstant: return value;
		case OpArgument: return 0.0f;
		case OpPointX: return p[0];
		case OpPointY: return p[1];
		case OpPointZ: return p[2];
		case OpNormalX: case OpNormalY: case OpNormalZ: return 0.0f;
		case OpAdd: return a + b;
		case OpSubtract: return a - b;
		case OpMultiply: return a * b;
		case OpDivide: return a / b;
		case OpNegate: return -a;
		case OpSqrt: return sqrtf(a);
		case OpAbs: return fabsf(a);
		case OpFloor: return floorf(a);
		case OpSin: return sinf(a);
		case OpCos: return cosf(a);
		case OpSign: return a > 0.0f ? 1.0f : (a < 0.0f ? -1.0f : 0.0f);
		case OpAtan2: return atan2f(a, b);
		case OpPow: return powf(a, b);
		case OpMin: return b < a ? b : a;
		case OpMax: return a < b ? b : a;
		case OpSmin: return smoothMinF(a, b, c);
		case OpPosSq: {
			const float q = fmaxf(a, 0.0f);
			return q * q;
		}
		case OpLess: return truthF(a < b);
		case OpLessEq: return truthF(a <= b);
		case OpEqual: return truthF(a == b);
		case OpNotEqual: return truthF(a != b);
		case OpAnd: return truthF(a != 0.0f && b != 0.0f);
		case OpOr: return truthF(a != 0.0f || b != 0.0f);
		case OpNot: return truthF(a == 0.0f);
		case OpSelect: return a != 0.0f ? b : c;
		default: return 0.0f;
	}
}

// The reserved slots of a thread's column: 0, 1 and -1 once, the point at
// each new point.
KDN_HD void setConstants(float* slots, uint32_t stride) {
	slots[SlotZero * stride]     = 0.0f;
	slots[SlotOne * stride]      = 1.0f;
	slots[SlotMinusOne * stride] = -1.0f;
}

KDN_HD void setPoint(float* slots, uint32_t stride, const float p[3]) {
	slots[SlotX * stride] = p[0];
	slots[SlotY * stride] = p[1];
	slots[SlotZ * stride] = p[2];
}

// One step of the march form (world.h MarchStep): r = post(fma(a, b, c), w)
// with the post operations worked out together and the step's picked, so
// the lanes of a warp on different steps do not split; a rare step runs the
// reference operation.  Writes the result to its slot and returns it.
KDN_HD float marchStep(const MarchStep& s, float* slots, uint32_t stride) {
	slots[SlotImm * stride] = s.value;
	const float a = slots[s.a * stride], b = slots[s.b * stride], c = slots[s.c * stride];
	float r;
	if (s.op >= kMarchRare) {
		const float p[3] = { slots[SlotX * stride], slots[SlotY * stride], slots[SlotZ * stride] };
		r                = stepValue(uint8_t(s.op - kMarchRare), a, b, c, s.value, p);
	} else {
		const float w = slots[s.w * stride];
		const float f = fmaf(a, b, c);
		const float q = fmaxf(f, 0.0f);
		// the smooth minimum of radius r = value: min - max(r - |f - w|, 0)^2 * 0.25 / r
		const float m = fmaxf(s.value - fabsf(f - w), 0.0f);
		r             = f;
		r             = s.op == PostSqrt ? marchSqrt(f) : r;
		r             = s.op == PostAbs ? fabsf(f) : r;
		r             = s.op == PostPosSq ? q * q : r;
		r             = s.op == PostMin ? (w < f ? w : f) : r;
		r             = s.op == PostMax ? (f < w ? w : f) : r;
		r             = s.op == PostSminK ? fminf(f, w) - m * m * s.quarter : r;
	}
	slots[s.dst * stride] = r;
	return r;
}

// One program at one point; slots is this thread's column base (stride
// blockDim.x), with the constants set.  Returns the program's value.
KDN_HD float evalSlots(const MarchStep* __restrict__ code, uint32_t count, uint32_t resultSlot, float* slots, uint32_t stride, const float p[3]) {
	setPoint(slots, stride, p);
	for (uint32_t i = 0; i < count; ++i) marchStep(code[i], slots, stride);
	return slots[resultSlot * stride];
}

struct DualF {
	float v, g0, g1, g2;
};

__device__ __forceinline__ DualF dualConst(float v) { return { v, 0.0f, 0.0f, 0.0f }; }
__device__ __forceinline__ DualF chain1(DualF a, float f, float d) { return { f, d * a.g0, d * a.g1, d * a.g2 }; }
__device__ __forceinline__ DualF chain2(DualF a, DualF b, float f, float fa, float fb) {
	return { f, fa * a.g0 + fb * b.g0, fa * a.g1 + fb * b.g1, fa * a.g2 + fb * b.g2 };
}

// sdf/numbers.cpp:440-590 the Dual operations.
__device__ __forceinline__ DualF dualStep(uint8_t op, DualF a, DualF b, DualF c, float value, const float p[3]) {
	switch (op) {
		case OpConstant: return dualConst(value);
		case OpPointX: return { p[0], 1.0f, 0.0f, 0.0f };
		case OpPointY: return { p[1], 0.0f, 1.0f, 0.0f };
		case OpPointZ: return { p[2], 0.0f, 0.0f, 1.0f };
		case OpAdd: return chain2(a, b, a.v + b.v, 1.0f, 1.0f);
		case OpSubtract: return chain2(a, b, a.v - b.v, 1.0f, -1.0f);
		case OpMultiply: return chain2(a, b, a.v * b.v, b.v, a.v);
		case OpDivide: return chain2(a, b, a.v / b.v, 1.0f / b.v, -a.v / (b.v * b.v));
		case OpNegate: return chain1(a, -a.v, -1.0f);
		case OpSqrt: {
			const float f = sqrtf(a.v);
			return chain1(a, f, f > 0.0f ? 0.5f / f : 0.0f);
		}
		case OpAbs: return a.v < 0.0f ? chain1(a, -a.v, -1.0f) : a;
		case OpFloor: return dualConst(floorf(a.v));
		case OpSin: return chain1(a, sinf(a.v), cosf(a.v));
		case OpCos: return chain1(a, cosf(a.v), -sinf(a.v));
		case OpSign: return dualConst(a.v > 0.0f ? 1.0f : (a.v < 0.0f ? -1.0f : 0.0f));
		case OpAtan2: {
			const float r = b.v * b.v + a.v * a.v;
			return chain2(a, b, atan2f(a.v, b.v), b.v / r, -a.v / r);
		}
		case OpPow: {
			const float f = powf(a.v, b.v);
			return chain2(a, b, f, b.v * powf(a.v, b.v - 1.0f), f * (a.v > 0.0f ? logf(a.v) : 0.0f));
		}
		case OpMin: return a.v <= b.v ? a : b;
		case OpMax: return a.v >= b.v ? a : b;
		case OpSmin: {
			const float fa = fminf(fmaxf((c.v - (a.v - b.v)) / (2.0f * c.v), 0.0f), 1.0f);
			return chain2(a, b, smoothMinF(a.v, b.v, c.v), fa, 1.0f - fa);
		}
		case OpPosSq: return chain1(a, fmaxf(a.v, 0.0f) * fmaxf(a.v, 0.0f), 2.0f * fmaxf(a.v, 0.0f));
		case OpSelect: return a.v != 0.0f ? b : c;
		default: return dualConst(stepValue(op, a.v, b.v, c.v, value, p));
	}
}

__device__ __forceinline__ DualF evalDual(const GpuStep* __restrict__ code, uint32_t count, uint32_t resultSlot, DualF* slots, const float p[3]) {
	for (uint32_t i = 0; i < count; ++i) {
		const GpuStep s = code[i];
		slots[s.dst]    = dualStep(s.op, slots[s.a], slots[s.b], slots[s.c], s.value, p);
	}
	return slots[resultSlot];
}

__device__ __forceinline__ bool isJoin(uint8_t op) { return op == OpMin || op == OpSmin || op == OpMax || op == OpNegate || op == OpSelect; }

__device__ __forceinline__ uint32_t chosenOperand(uint8_t op, const SsaOps& o, const float* v) {
	const float a = v[o.a], b = v[o.b];
	switch (op) {
		case OpMin: case OpSmin: return a <= b ? o.a : o.b;
		case OpMax: return a >= b ? o.a : o.b;
		case OpSelect: return a != 0.0f ? o.b : o.c;
		default: return o.a;
	}
}

// Every step's value by step number, then the walk back through the joins
// (sdf/program.cpp:478 laneSourceOf): the leaf that decides the value, the
// leaf across the first smooth band and its share.
__device__ __forceinline__ void sourceOf(const GpuStep* __restrict__ code, const SsaOps* __restrict__ ssa, uint32_t count, uint32_t result, float* v, const float p[3], uint32_t& leaf, uint32_t& other, float& share) {
	for (uint32_t i = 0; i < count; ++i) {
		const GpuStep s = code[i];
		const SsaOps o  = ssa[i];
		v[i]            = stepValue(s.op, v[o.a], v[o.b], v[o.c], s.value, p);
	}
	other    = kNoLeaf;
	share    = 0.0f;
	uint32_t at = result;
	for (uint32_t guard = 0; guard < count && isJoin(code[at].op); ++guard) {
		const SsaOps o      = ssa[at];
		const uint8_t op    = code[at].op;
		const uint32_t next = chosenOperand(op, o, v);
		float s             = 0.0f;
		if (op == OpSmin) {
			const float radius = v[o.c];
			const float apart  = fabsf(v[o.a] - v[o.b]);
			s                  = radius > 0.0f && apart < radius ? 0.5f * (radius - apart) / radius : 0.0f;
		}
		if (s > 0.0f && other == kNoLeaf) {
			uint32_t side = next == o.a ? o.b : o.a;
			for (uint32_t g = 0; g < count && isJoin(code[side].op); ++g) side = chosenOperand(code[side].op, ssa[side], v);
			other = code[side].leaf;
			share = s;
		}
		at = next;
	}
	leaf = code[at].leaf;
}

} // namespace kdn
