// Device-resident world of the GB300 backend: the cut octree and the kept
// programs of its leaves, in the layout the trace kernel reads.
//
// The octree is a pointer-free array of 32-bit nodes, children of a node
// contiguous (breadth-first per parent).  A node holds the index of its first
// child, or ~leaf for a leaf.  A leaf names a run of kept programs; a program
// is a run of 16-byte GpuSteps whose operands are register slots (a linear
// scan over the straight-line program reuses a slot once its value is dead),
// so the march keeps a program's live values in a few shared-memory slots.
// The same steps keep their SSA operand numbers in a parallel array for the
// single evaluation at a hit that finds the source leaf (sdf/program.cpp:505).
#pragma once

#include <cstdint>

namespace kdn {

// sdf/program.h:20 Opcode values.
enum Op : uint8_t {
	OpConstant, OpArgument, OpPointX, OpPointY, OpPointZ, OpNormalX, OpNormalY, OpNormalZ,
	OpAdd, OpSubtract, OpMultiply, OpDivide, OpNegate, OpSqrt, OpAbs, OpFloor, OpSin, OpCos,
	OpSign, OpAtan2, OpPow, OpMin, OpMax, OpSmin, OpPosSq, OpLess, OpLessEq, OpEqual,
	OpNotEqual, OpAnd, OpOr, OpNot, OpSelect, OpCount
};

// The march form: a program lowered to steps r = post(fma(a, b, c), w).
// +, -, * and negation are one fused multiply-add each (x + y = fma(x, 1,
// y), x - y = fma(y, -1, x), x * y = fma(x, y, 0)); a product that feeds only
// a sum folds into it; sqrt, |x|, max(x, 0)^2, min, max and a smooth minimum
// of constant radius ride on the step that makes their operand where that
// step's result has no other use; double negations cancel.  Operands are
// slots of the thread's column: the first kMarchFirstSlot hold 0, 1, -1, the
// point and the step's immediate.  Every other reference operation is a
// rare step (kMarchRare + opcode) over slots a, b, c.
enum MarchPost : uint8_t { PostNone, PostSqrt, PostAbs, PostPosSq, PostMin, PostMax, PostSminK };
constexpr uint8_t kMarchRare = 64;
enum MarchSlot : uint8_t { SlotZero, SlotOne, SlotMinusOne, SlotX, SlotY, SlotZ, SlotImm, kMarchFirstSlot };

struct MarchStep {
	uint8_t op;  // MarchPost, or kMarchRare + reference opcode
	uint8_t dst; // slot of the result
	uint8_t a, b, c;
	uint8_t w;   // the post operation's second operand (min, max, smooth minimum)
	uint16_t pad;
	float value;   // the immediate (SlotImm); a smooth minimum's radius
	float quarter; // 0.25 / radius of a smooth minimum
};
static_assert(sizeof(MarchStep) == 16, "MarchStep is 16 bytes");

constexpr uint32_t kNoLeaf     = 0xFFFFFFFFu;
constexpr uint32_t kMaxSlots   = 48;   // register slots a leaf program may use
constexpr uint32_t kMaxSsa     = 1024; // steps a leaf program may hold
constexpr uint32_t kMaxLeafProgs = 64; // kept programs of one leaf
// The most steps a ray is marched (sphere_trace.h:37 sphereSteps): a ray that
// skims a surface for longer meets nothing.
constexpr uint32_t kMarchSteps = 1u << 16;

// A step of a program's full form, read once a hit: register slots a, b,
// c, the reference opcode and constant, and the leaf a step names.
struct GpuStep {
	uint8_t op;
	uint8_t dst;
	uint8_t a, b, c;
	uint8_t imm;
	uint16_t pad1;
	float value;
	uint32_t leaf;
};
static_assert(sizeof(GpuStep) == 16, "GpuStep is 16 bytes");

struct SsaOps {
	uint16_t a, b, c, pad;
};
static_assert(sizeof(SsaOps) == 8, "SsaOps is 8 bytes");

struct GpuProgram {
	uint32_t code;       // first GpuStep of the whole program (read at a hit)
	uint16_t count;      // its steps
	uint16_t result;     // SSA index of the result
	uint8_t slot;        // slot of the result
	uint8_t slots;       // slots used
	uint16_t marchCount; // steps of the march form
	uint32_t object;     // index into the scene's object programs
	uint32_t march;      // first MarchStep of the march form
	uint8_t marchSlot;   // slot of the result in the march form
	uint8_t marchSlots;
	uint16_t pad0;
	uint32_t pad1[2];
};
static_assert(sizeof(GpuProgram) == 32, "GpuProgram is 32 bytes");

enum Occupancy : uint8_t { Empty = 0, Filled = 1, Surface = 2 };

struct GpuLeaf {
	uint32_t first;     // first GpuProgram
	uint16_t count;     // kept programs
	uint8_t occupancy;
	uint8_t slots;      // most slots of its programs
	// the first program's march form, read with the leaf
	uint32_t march;
	uint16_t marchCount;
	uint8_t marchSlot;
	uint8_t pad;
};
static_assert(sizeof(GpuLeaf) == 16, "GpuLeaf is 16 bytes");

// The octree cut across at one level: for each cell of the uniform grid of
// that level, the node value there (first child, or ~leaf) and its level,
// less than the grid's where a leaf above it covers the cell.  A point is
// located by its grid cell (an estimate from its coordinates, set right
// against the grid's walls), one load, and the descent below it.  The walls
// are the descent's own midpoints, 0.5 * (lo + hi) level by level in FP32,
// so a point lands in the cell the descent from the root would give it.
struct GridCell {
	int32_t node;
	uint32_t level;
};
constexpr uint32_t kGridLevel = 6;

// Everything the trace kernel reads, as device pointers.
struct DeviceWorld {
	const int32_t* nodes;
	const GpuLeaf* leaves;
	const GpuProgram* programs;
	const GpuStep* steps;
	const MarchStep* march;
	const SsaOps* ssa;
	const uint32_t* leaf_material;
	const GridCell* grid; // (2^gridLevel)^3 cells, x fastest; null: descend from the root
	const float* gridWalls; // per axis 2^gridLevel + 1 walls
	uint32_t gridLevel;
	float gridScale[3];   // 2^gridLevel / size
	float lower[3];
	float size[3];
	uint32_t leaf_count;
	uint32_t material_count;
	uint32_t marchSlots; // the most slots a march-form program uses: the trace kernel's shared memory a thread
};

} // namespace kdn
