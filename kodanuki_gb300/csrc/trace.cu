// The geometry kernels: sphere tracing through the cut octree.
//
// K-trace marches each ray (plugins/geometry/sphere_trace/sphere_trace.cpp:
// 203 sphereFromOutside, :188 sphereFromInside) by the field read from the
// kept programs of the octree leaf the point lies in: there the kept
// programs are exactly the objects that can be least (cut.cpp:442 deciding),
// so the step is the scene's field.  An empty leaf holds no surface, and
// the ray skips to where it leaves the cell.
// K-hit then evaluates the winning program once in duals for the normal and
// once by step number for its source leaf (sphere_trace.cpp:115 sphereField).
#include "kernels.h"
#include "locate.cuh"
#include "program.cuh"

#include <cuda_runtime.h>

namespace kdn {

namespace {

constexpr int kTraceBlock = 128;
// program steps a thread runs a turn of the step machine before the warp
// looks again for threads that need a new ray or a new cell (8 measured
// faster than 4 on config 2: fewer turns of overhead a program, whose march
// form is ~6 steps on average)
constexpr uint32_t kStepsPerTurn = 8;
// empty cells a thread passes a turn before the warp moves on
constexpr uint32_t kCellsPerTurn = 1;

__device__ __forceinline__ float slopeOf(float part) {
	const float tiny = 1e-12f;
	return 1.0f / (fabsf(part) < tiny ? copysignf(tiny, part) : part);
}

__device__ __forceinline__ float tolerance(const float p[3]) {
	const float big = fmaxf(fabsf(p[0]), fmaxf(fabsf(p[1]), fabsf(p[2])));
	return 2e-6f * fmaxf(1.0f, big * 0.25f);
}

__device__ __forceinline__ float nudge(float t) { return fmaxf(1e-5f, fabsf(t) * 2e-6f); }

__device__ __forceinline__ float cellExitBy(const float o[3], const float inv[3], const Located& l) {
	float up = 3.0e38f;
	for (int a = 0; a < 3; ++a) {
		const float x = (l.lo[a] - o[a]) * inv[a];
		const float y = (l.hi[a] - o[a]) * inv[a];
		up            = fminf(up, fmaxf(x, y));
	}
	return up;
}

__device__ __forceinline__ float cellExit(const float o[3], const float d[3], const Located& l) {
	float up = 3.0e38f;
	for (int a = 0; a < 3; ++a) {
		const float inv = slopeOf(d[a]);
		const float x   = (l.lo[a] - o[a]) * inv;
		const float y   = (l.hi[a] - o[a]) * inv;
		up              = fminf(up, fmaxf(x, y));
	}
	return up;
}

struct Field {
	float least;   // least program value
	float nearest; // least magnitude
	uint32_t index;  // which kept program is least
	uint32_t count;  // kept programs
	uint32_t first;  // first GpuProgram of the leaf
	bool empty;
	float exit;
};

// Whether a point is in a located cell: the half-open box the descent gives
// it (a coordinate equal to a midpoint goes to the upper half), so a point
// found here is the point the descent would find there.
__device__ __forceinline__ bool within(const Located& l, const float p[3]) {
	return l.leaf != kNoLeaf && p[0] >= l.lo[0] && p[0] < l.hi[0] && p[1] >= l.lo[1] && p[1] < l.hi[1] && p[2] >= l.lo[2] && p[2] < l.hi[2];
}

// The field at t from the kept programs of the cell the point lies in.  The
// cell of the previous step is kept in `cell`: a ray takes several steps in
// one cell, and only a point that has left it descends the octree again.
__device__ __forceinline__ Field fieldAt(const DeviceWorld& w, const float o[3], const float d[3], float t, float* slots, uint32_t stride, uint32_t& steps, Located& cell) {
	Field f;
	const float p[3] = { o[0] + d[0] * t, o[1] + d[1] * t, o[2] + d[2] * t };
	if (!within(cell, p)) cell = locate(w, p);
	const Located& l   = cell;
	const GpuLeaf leaf = w.leaves[l.leaf];
	f.first  = leaf.first;
	f.count  = leaf.count;
	f.empty  = leaf.occupancy == Empty || leaf.count == 0;
	f.least  = 3.0e38f;
	f.nearest = 3.0e38f;
	f.index  = 0;
	// A cell keeps only the objects whose surface may pass through it
	// (cut.cpp:442 deciding), so past its walls its field is no distance
	// bound: a step stops where the ray leaves the cell.
	f.exit   = cellExit(o, d, l);
	if (f.empty) return f;
	for (uint32_t k = 0; k < leaf.count; ++k) {
		const GpuProgram g = w.programs[leaf.first + k];
		const float v      = evalSlots(w.march + g.march, g.marchCount, g.marchSlot, slots, stride, p);
		steps += g.marchCount;
		if (v < f.least) {
			f.least = v;
			f.index = k;
		}
		f.nearest = fminf(f.nearest, fabsf(v));
	}
	return f;
}

// The least value at t, and the index of the kept program that is least a
// little further along among those tied with it (sphere_trace.cpp:96).
__device__ __forceinline__ uint32_t winnerAt(const DeviceWorld& w, const float o[3], const float d[3], float t, const Field& f, float* slots, uint32_t stride) {
	const float p[3] = { o[0] + d[0] * t, o[1] + d[1] * t, o[2] + d[2] * t };
	const float big  = fmaxf(fabsf(p[0]), fmaxf(fabsf(p[1]), fabsf(p[2])));
	const float band = 2e-6f * (1.0f + big);
	const float q[3] = { p[0] + d[0] * 2e-5f, p[1] + d[1] * 2e-5f, p[2] + d[2] * 2e-5f };
	uint32_t winner  = f.index;
	float onWinner   = 3.0e38f;
	bool tied        = false;
	float values[kMaxLeafProgs];
	for (uint32_t k = 0; k < f.count && k < kMaxLeafProgs; ++k) {
		const GpuProgram g = w.programs[f.first + k];
		values[k]          = evalSlots(w.march + g.march, g.marchCount, g.marchSlot, slots, stride, p);
		tied               = tied || (k != f.index && values[k] - f.least <= band);
	}
	if (!tied) return winner;
	for (uint32_t k = 0; k < f.count && k < kMaxLeafProgs; ++k) {
		if (!(values[k] - f.least <= band)) continue;
		const GpuProgram g = w.programs[f.first + k];
		const float on     = evalSlots(w.march + g.march, g.marchCount, g.marchSlot, slots, stride, q);
		if (on < onWinner) {
			onWinner = on;
			winner   = k;
		}
	}
	return winner;
}

// sphereFromInside at a point within the tolerance of the nearest surface:
// read the field a little past it.  kind 0: go on past (t += inset); 1: the
// ray leaves its solid here (winner among the cell's programs); 2: it meets
// a solid of another material (the program past the point).
struct InsideStop {
	uint32_t kind, first, index;
};

__device__ __forceinline__ InsideStop insideStop(const DeviceWorld& w, const uint32_t* objectMaterial, uint32_t medium, const float o[3], const float d[3], float t,
                                             float inset, const Field& f, const Located& cell, float* slots, uint32_t stride, uint32_t& steps) {
	Located beyond   = cell;
	const Field past = fieldAt(w, o, d, t + inset, slots, stride, steps, beyond);
	if (past.empty || past.least > 0.0f) return InsideStop { 1, f.first, winnerAt(w, o, d, t, f, slots, stride) };
	const GpuProgram g = w.programs[past.first + past.index];
	// a solid of another material than the one the ray is in: stop there
	if (objectMaterial != nullptr && objectMaterial[g.object] != medium) return InsideStop { 2, past.first, past.index };
	return InsideStop { 0, 0, 0 };
}

// The march as a step machine.  Each thread holds one ray at a time and
// every turn of the loop runs one program step for every thread that is
// evaluating, so threads whose cells hold programs of different lengths, or
// whose rays take different numbers of march steps, stay busy: a thread that
// finishes a program moves on to the next program of its cell, a thread that
// finishes a march step locates its next cell, and a thread whose ray ends
// takes the next ray of the launch (one atomic a warp).
enum LaneMode : uint32_t { Fetch = 0, Locating = 1, Evaluating = 2, Finished = 3 };

// Seven blocks an SM is what 72 registers a thread allow; saying so lets
// ptxas keep the step machine's state in registers (it spills 8 bytes with
// the hint, 44 without; 46.1 against 45.3 Msamples/s on config 2).
__global__ void __launch_bounds__(kTraceBlock, 7) traceKernel(TraceArgs args) {
	extern __shared__ float slotMemory[];
	const DeviceWorld& w  = args.world;
	const uint32_t stride = blockDim.x;
	float* slots          = slotMemory + threadIdx.x;
	setConstants(slots, stride);
	// capped rays in the low 16 bits, carried ones in the high: one register
	uint32_t marchSteps = 0, programSteps = 0, traced = 0, cappedCarried = 0, longest = 0;
	// the steps a ray may take in this launch: a launch's budget, or the cap
	const uint32_t allowance = args.budget > 0 ? args.budget : kMarchSteps;
	// the rays: [0, n1) and, after them in the fetch order, [second, second + n2)
	const uint32_t n1 = args.count ? *args.count : args.n;
	const uint32_t n  = n1 + (args.secondCount ? *args.secondCount : 0u);
	const unsigned lane = threadIdx.x & 31u;

	if (args.left != nullptr && args.counters != nullptr && blockIdx.x == 0 && threadIdx.x == 0) {
		const uint32_t left = *args.left;
		if (left) atomicAdd(&args.counters[6], (unsigned long long) left);
	}
	uint32_t mode = Fetch;
	uint32_t ray  = 0;
	float o[3], d[3], inv[3];
	float t = 0.0f, up = 0.0f;
	bool inside      = false;
	uint32_t medium  = kNoLeaf;
	uint32_t step    = 0;
	// where the ray's march stops in this launch: the cap, or sooner its budget
	uint32_t stepLimit = 0;
	Located cell;
	cell.leaf = kNoLeaf;
	float exitT = 0.0f;
	// the cell being evaluated: its run of kept programs and the one in hand
	uint32_t first = 0, count = 0, k = 0;
	const MarchStep* code = nullptr;
	MarchStep next {};
	uint32_t pc = 0, length = 0, resultSlot = 0;
	float p[3]  = { 0.0f, 0.0f, 0.0f };
	float least = 0.0f, second = 0.0f, nearest = 0.0f;
	uint32_t index = 0;
	// a ray ends: its state, the step counts, and the next ray
	auto done = [&](HitState h) {
		args.states[ray] = h;
		marchSteps += h.steps; // less the steps it had when taken (at the fetch)
		longest = max(longest, h.steps);
		cappedCarried += h.kind == kCarried ? 0x10000u : (h.steps >= args.maxSteps ? 1u : 0u);
		mode = Fetch;
	};

	for (;;) {
		// take new rays, one atomic a warp
		const bool want     = mode == Fetch;
		const unsigned mask = __ballot_sync(0xFFFFFFFFu, want);
		if (mask) {
			uint32_t base = 0;
			const int leader = __ffs(mask) - 1;
			if (int(lane) == leader) base = atomicAdd(args.fetch, uint32_t(__popc(mask)));
			base = __shfl_sync(0xFFFFFFFFu, base, leader);
			if (want) {
				ray = base + uint32_t(__popc(mask & ((1u << lane) - 1u)));
				if (ray >= n) {
					mode = Finished;
				} else {
					if (ray >= n1) ray = args.second + (ray - n1);
					const kdn_ray r = args.rays[ray];
					for (int a = 0; a < 3; ++a) {
						o[a]   = r.origin[a];
						d[a]   = r.direction[a];
						inv[a] = slopeOf(d[a]);
					}
					float lo = 0.0f;
					up       = r.far;
					for (int a = 0; a < 3; ++a) {
						const float x = (w.lower[a] - o[a]) * inv[a];
						const float y = (w.lower[a] + w.size[a] - o[a]) * inv[a];
						lo            = fmaxf(lo, fminf(x, y));
						up            = fminf(up, fmaxf(x, y));
					}
					t         = lo;
					inside    = r.inside != 0;
					medium    = r.within;
					step      = 0;
					// a carried ray goes on where its march stood
					if (args.carry != nullptr && (r.pad_[0] & kRayResumes)) {
						const uint2 c = args.carry[ray];
						t             = __uint_as_float(c.x);
						step          = c.y;
					} else {
						++traced; // a segment is counted once, in the launch that starts it
					}
					stepLimit = min(args.maxSteps, step + allowance);
					marchSteps -= step;
					cell.leaf = kNoLeaf;
					if (up < lo) {
						done(HitState { 0, t, kNoLeaf, 0, step });
					} else {
						mode = Locating;
					}
				}
			}
		}
		if (__all_sync(0xFFFFFFFFu, mode == Finished)) break;

		// find the cell of the point, skipping empty cells, and start its first program
		if (mode == Locating) {
			for (uint32_t skipped = 0;;) {
				// past the cap or the region: a miss, which keeps where its march
				// stopped (a held path resumes it); out of this launch's budget
				// before either: carried, the march's whole state being (t, step)
				if (!(step < stepLimit && t <= up)) {
					const bool carried = step < args.maxSteps && t <= up;
					done(HitState { carried ? kCarried : 0u, t, kNoLeaf, 0, step });
					break;
				}
				for (int a = 0; a < 3; ++a) p[a] = o[a] + d[a] * t;
				if (!within(cell, p)) cell = locate(w, p);
				const GpuLeaf leaf = w.leaves[cell.leaf];
				exitT              = cellExitBy(o, inv, cell);
				if (leaf.occupancy == Empty || leaf.count == 0) {
					t = fmaxf(exitT, t) + nudge(t);
					++step;
					if (++skipped < kCellsPerTurn) continue;
					break; // the next turn goes on locating
				}
				first   = leaf.first;
				count   = leaf.count;
				k       = 0;
				least   = 3.0e38f;
				second  = 3.0e38f;
				nearest = 3.0e38f;
				index   = 0;
				code       = w.march + leaf.march;
				length     = leaf.marchCount;
				resultSlot = leaf.marchSlot;
				pc         = 0;
				next       = code[0];
				mode       = Evaluating;
				setPoint(slots, stride, p);
				break;
			}
		}

		// a few program steps; each step's code is loaded a step ahead
		if (mode == Evaluating) {
			for (uint32_t u = 0; u < kStepsPerTurn; ++u) {
				const MarchStep s = next;
				if (pc + 1 < length) next = code[pc + 1];
				marchStep(s, slots, stride);
				if (++pc == length) break;
			}
			if (pc == length) {
				const float v = slots[resultSlot * stride];
				programSteps += length;
				if (v < least) {
					second = least;
					least  = v;
					index  = k;
				} else if (v < second) {
					second = v;
				}
				nearest = fminf(nearest, fabsf(v));
				if (++k < count) {
					const GpuProgram g = w.programs[first + k];
					code       = w.march + g.march;
					length     = g.marchCount;
					resultSlot = g.marchSlot;
					pc         = 0;
					next       = code[0];
				} else {
					// the march step: stop on the surface or go on by the field
					const float tol = tolerance(p);
					++step;
					mode = Locating;
					if (!inside) {
						if (least < tol) {
							Field f;
							f.least = least;
							f.index = index;
							f.count = count;
							f.first = first;
							const float big  = fmaxf(fabsf(p[0]), fmaxf(fabsf(p[1]), fabsf(p[2])));
							const bool tied  = second - least <= 2e-6f * (1.0f + big);
							const uint32_t winner = tied ? winnerAt(w, o, d, t, f, slots, stride) : index;
							done(HitState { 1, t, first, winner, step });
						} else {
							t = fminf(t + least, fmaxf(exitT, t) + nudge(t));
						}
					} else if (nearest < tol) {
						// sphereFromInside: stand on the nearest surface and read the field past it
						Field f;
						f.least = least;
						f.index = index;
						f.count = count;
						f.first = first;
						const float inset   = 2.0f * tol;
						const InsideStop at = insideStop(w, args.objectMaterial, medium, o, d, t, inset, f, cell, slots, stride, programSteps);
						if (at.kind == 0) t += inset;
						else done(HitState { at.kind, t, at.first, at.index, step });
					} else {
						t = fminf(t + nearest, fmaxf(exitT, t) + nudge(t));
					}
				}
			}
		}
	}
	if (args.counters) {
		// one add per warp
		for (int o = 16; o > 0; o >>= 1) {
			marchSteps += __shfl_down_sync(0xFFFFFFFFu, marchSteps, o);
			programSteps += __shfl_down_sync(0xFFFFFFFFu, programSteps, o);
			traced += __shfl_down_sync(0xFFFFFFFFu, traced, o);
			cappedCarried += __shfl_down_sync(0xFFFFFFFFu, cappedCarried, o);
			longest = max(longest, __shfl_down_sync(0xFFFFFFFFu, longest, o));
		}
		if ((threadIdx.x & 31) == 0) {
			atomicAdd(&args.counters[0], (unsigned long long) marchSteps);
			atomicAdd(&args.counters[1], (unsigned long long) programSteps);
			atomicMax(&args.counters[2], (unsigned long long) longest);
			atomicAdd(&args.counters[3], (unsigned long long) (cappedCarried & 0xFFFFu));
			atomicAdd(&args.counters[4], (unsigned long long) traced);
			if (cappedCarried >> 16) atomicAdd(&args.counters[5], (unsigned long long) (cappedCarried >> 16));
		}
	}
}

__global__ void __launch_bounds__(kTraceBlock) hitKernel(HitArgs args) {
	const DeviceWorld& w = args.world;
	const uint32_t n     = args.count ? *args.count : args.n;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const HitState h  = args.states[i];
		const kdn_ray ray = args.rays[i];
		kdn_hit out;
		out.kind = 0;
		out.pad0_[0] = out.pad0_[1] = out.pad0_[2] = 0;
		out.distance = 0.0f;
		for (int a = 0; a < 3; ++a) {
			out.point[a]  = 0.0f;
			out.normal[a] = 0.0f;
		}
		out.leaf      = kNoLeaf;
		out.other     = kNoLeaf;
		out.share     = 0.0f;
		out.loosened  = 0.0f;
		out.leaf_kind = 0;
		out.pad1_[0] = out.pad1_[1] = out.pad1_[2] = 0;
		out.cell      = kNoLeaf;
		if (h.kind == kCarried) {
			// the march goes on in a later launch: where it stands and its steps
			out.kind     = kHitCarried;
			out.distance = h.distance;
			out.cell     = h.steps;
		} else if (h.kind != 0) {
			const float d[3]  = { ray.direction[0], ray.direction[1], ray.direction[2] };
			const float t     = h.distance;
			const float p[3]  = { ray.origin[0] + d[0] * t, ray.origin[1] + d[1] * t, ray.origin[2] + d[2] * t };
			// For a crossing into another material the field is read past the point.
			const float inset = h.kind == 2 ? 2.0f * tolerance(p) : 0.0f;
			const float q[3]  = { p[0] + d[0] * inset, p[1] + d[1] * inset, p[2] + d[2] * inset };
			const GpuProgram g = w.programs[h.first + h.index];
			// every slot is written before a step reads it (the slots follow the SSA order)
			DualF dslots[kMaxSlots];
			const DualF v = evalDual(w.steps + g.code, g.count, g.slot, dslots, q);
			float values[kMaxSsa];
			uint32_t leaf, other;
			float share;
			sourceOf(w.steps + g.code, w.ssa + g.code, g.count, g.result, values, q, leaf, other, share);
			// sphereNormal (sphere_trace.cpp:140)
			float n[3];
			const float len = sqrtf(v.g0 * v.g0 + v.g1 * v.g1 + v.g2 * v.g2);
			if (!(len > 0.0f)) {
				for (int a = 0; a < 3; ++a) n[a] = -d[a];
			} else {
				n[0] = v.g0 / len;
				n[1] = v.g1 / len;
				n[2] = v.g2 / len;
				const float along = n[0] * d[0] + n[1] * d[1] + n[2] * d[2];
				if (ray.inside) {
					if (along < 0.0f) {
						for (int a = 0; a < 3; ++a) n[a] = -n[a];
					}
				} else if (along > 0.0f) {
					float gz[3];
					for (int a = 0; a < 3; ++a) gz[a] = n[a] - d[a] * (along + 0.02f);
					const float gl = sqrtf(gz[0] * gz[0] + gz[1] * gz[1] + gz[2] * gz[2]);
					for (int a = 0; a < 3; ++a) n[a] = gz[a] / gl;
				}
			}
			out.kind     = 1;
			out.distance = t;
			for (int a = 0; a < 3; ++a) {
				out.point[a]  = p[a];
				out.normal[a] = n[a];
			}
			out.leaf     = leaf;
			out.other    = other;
			out.share    = share;
			out.loosened = tolerance(p);
			out.cell     = g.object;
		}
		args.hits[i] = out;
	}
}

} // namespace

cudaError_t launchTrace(const TraceArgs& args, cudaStream_t stream, int smCount) {
	if (args.n == 0) return cudaSuccess;
	// a thread's register slots in shared memory, as many as the world's
	// largest march program uses: the rest of the SM's shared memory stays
	// L1 for the programs' code
	const size_t shared = size_t(std::max<uint32_t>(1, std::min(args.world.marchSlots, kMaxSlots))) * kTraceBlock * sizeof(float);
	// persistent blocks: as many as fit on the SMs at once, fewer for a small launch
	static thread_local size_t sizedFor = 0;
	static thread_local int resident    = 0;
	if (sizedFor != shared) {
		int perSm = 0;
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, traceKernel, kTraceBlock, shared) != cudaSuccess || perSm < 1) perSm = 1;
		resident = perSm;
		sizedFor = shared;
	}
	const uint64_t wanted = (uint64_t(args.n) + kTraceBlock - 1) / kTraceBlock;
	const uint32_t blocks = uint32_t(std::max<uint64_t>(1, std::min<uint64_t>(wanted, uint64_t(smCount) * uint64_t(resident))));
	cudaError_t e = cudaMemsetAsync(args.fetch, 0, sizeof(uint32_t), stream);
	if (e != cudaSuccess) return e;
	traceKernel<<<blocks, kTraceBlock, shared, stream>>>(args);
	return cudaGetLastError();
}

cudaError_t launchHits(const HitArgs& args, cudaStream_t stream, int smCount) {
	if (args.n == 0) return cudaSuccess;
	const uint32_t blocks = uint32_t(std::min<uint64_t>((uint64_t(args.n) + kTraceBlock - 1) / kTraceBlock, uint64_t(smCount) * 16));
	hitKernel<<<blocks, kTraceBlock, 0, stream>>>(args);
	return cudaGetLastError();
}

cudaError_t setTraceAttributes() {
	return cudaFuncSetAttribute(traceKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kMaxSlots * kTraceBlock * sizeof(float)));
}

} // namespace kdn
