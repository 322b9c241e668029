// Host build of the cut octree (the world the trace kernel walks).
//
// Each cell is cut from its parent's kept programs by interval arithmetic
// over the cell's box: the reference's cutCell (plugins/geometry/tree/
// cut.cpp:463) with its rewrite of every step (cut.cpp:80-300 shortcut,
// resolvedStep, unsquared, positiveSquared) and its pruning
// (sdf/program.cpp:357-420 liveSteps, compactedProgram).  Intervals follow
// sdf/numbers.cpp:200-432 without directed rounding, as the reference's do,
// so a cell keeps exactly the programs and steps the reference's cut keeps.
//
// The levels are built breadth-first; the cells of one level are cut in
// parallel on host threads and numbered in a fixed order, so the world is the
// same for any thread count.
#include "octree.h"

#include <algorithm>
#include <atomic>
#include <unordered_map>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>

namespace kdn {

namespace {

constexpr double kPi        = 3.14159265358979323846;
constexpr uint32_t kNoOperand = 0xFFFFFFFFu;

struct Iv {
	double lo, hi;
};

int operandCount(uint8_t op) {
	switch (op) {
		case OpConstant: case OpArgument: case OpPointX: case OpPointY: case OpPointZ:
		case OpNormalX: case OpNormalY: case OpNormalZ: return 0;
		case OpNegate: case OpSqrt: case OpAbs: case OpFloor: case OpSin: case OpCos: case OpSign: case OpNot: return 1;
		case OpSelect: case OpSmin: return 3;
		default: return 2;
	}
}

inline double lesser(double a, double b) { return b < a ? b : a; }
inline double greater(double a, double b) { return a < b ? b : a; }

double smoothMin(double a, double b, double r) {
	const double blend = greater(r - std::fabs(a - b), 0.0) / r;
	return lesser(a, b) - blend * blend * r * 0.25;
}

double positiveSquare(double a) {
	const double p = greater(a, 0.0);
	return p * p;
}

double signOf(double a) { return a > 0 ? 1.0 : (a < 0 ? -1.0 : 0.0); }

Iv hull(double a, double b, double c, double d) {
	double lo = a, hi = a;
	if (b < lo) lo = b;
	if (c < lo) lo = c;
	if (d < lo) lo = d;
	if (hi < b) hi = b;
	if (hi < c) hi = c;
	if (hi < d) hi = d;
	return { lo, hi };
}

Iv mul(Iv a, Iv b) { return hull(a.lo * b.lo, a.lo * b.hi, a.hi * b.lo, a.hi * b.hi); }
bool hasZero(Iv a) { return a.lo <= 0 && a.hi >= 0; }
Iv divide(Iv a, Iv b) {
	if (hasZero(b)) return { -std::numeric_limits<double>::infinity(), std::numeric_limits<double>::infinity() };
	return mul(a, { 1 / b.hi, 1 / b.lo });
}
Iv neg(Iv a) { return { -a.hi, -a.lo }; }
Iv absolute(Iv a) {
	if (a.lo >= 0) return a;
	if (a.hi <= 0) return neg(a);
	return { 0, greater(-a.lo, a.hi) };
}
bool reaches(Iv a, double offset) {
	const double k = std::ceil((a.lo - offset) / (2 * kPi));
	return offset + 2 * kPi * k <= a.hi;
}
Iv sine(Iv a) {
	if (a.hi - a.lo >= 2 * kPi) return { -1, 1 };
	const double s0 = std::sin(a.lo), s1 = std::sin(a.hi);
	Iv out = { lesser(s0, s1), greater(s0, s1) };
	if (reaches(a, kPi / 2)) out.hi = 1;
	if (reaches(a, -kPi / 2)) out.lo = -1;
	return out;
}
Iv arcTangent(Iv y, Iv x) {
	if ((hasZero(x) && hasZero(y)) || (x.lo < 0 && hasZero(y))) return { -kPi, kPi };
	return hull(std::atan2(y.lo, x.lo), std::atan2(y.lo, x.hi), std::atan2(y.hi, x.lo), std::atan2(y.hi, x.hi));
}
Iv wholePower(Iv a, double n) {
	if (n >= 0 && std::fmod(n, 2.0) == 0) {
		const Iv m = absolute(a);
		return { std::pow(m.lo, n), std::pow(m.hi, n) };
	}
	if (n > 0) return { std::pow(a.lo, n), std::pow(a.hi, n) };
	return divide({ 1, 1 }, wholePower(a, -n));
}
Iv power(Iv a, Iv b) {
	if (b.lo == b.hi && b.lo == std::floor(b.lo)) return wholePower(a, b.lo);
	if (a.lo <= 0) return { -std::numeric_limits<double>::infinity(), std::numeric_limits<double>::infinity() };
	return hull(std::pow(a.lo, b.lo), std::pow(a.lo, b.hi), std::pow(a.hi, b.lo), std::pow(a.hi, b.hi));
}
Iv decided(bool yes, bool no) { return { yes ? 1.0 : 0.0, no ? 0.0 : 1.0 }; }
bool excludesZero(Iv a) { return a.lo > 0 || a.hi < 0; }
bool isZero(Iv a) { return a.lo == 0 && a.hi == 0; }
Iv comparison(uint8_t op, Iv a, Iv b) {
	const bool apart = a.hi < b.lo || b.hi < a.lo;
	const bool same  = a.lo == a.hi && b.lo == b.hi && a.lo == b.lo;
	switch (op) {
		case OpLess: return decided(a.hi < b.lo, a.lo >= b.hi);
		case OpLessEq: return decided(a.hi <= b.lo, a.lo > b.hi);
		case OpEqual: return decided(same, apart);
		case OpNotEqual: return decided(apart, same);
		case OpAnd: return decided(excludesZero(a) && excludesZero(b), isZero(a) || isZero(b));
		case OpOr: return decided(excludesZero(a) || excludesZero(b), isZero(a) && isZero(b));
		default: return decided(a.lo == a.hi && a.lo == 0, a.hi < 0 || 0 < a.lo);
	}
}
Iv smoothMinimum(Iv a, Iv b, Iv r) {
	const double lo = smoothMin(a.lo, b.lo, r.lo);
	const double hi = smoothMin(a.hi, b.hi, r.lo);
	return { std::isnan(lo) ? lesser(a.lo, b.lo) - r.lo / 4 : lo, std::isnan(hi) ? lesser(a.hi, b.hi) : hi };
}

Iv stepInterval(const kdn_step& s, const Iv* r, const Iv box[3]) {
	const Iv a = r[s.a], b = r[s.b];
	switch (s.opcode) {
		case OpConstant: return { s.value, s.value };
		case OpArgument: return { 0, 0 };
		case OpPointX: return box[0];
		case OpPointY: return box[1];
		case OpPointZ: return box[2];
		case OpNormalX: case OpNormalY: case OpNormalZ: return { 0, 0 };
		case OpAdd: return { a.lo + b.lo, a.hi + b.hi };
		case OpSubtract: return { a.lo - b.hi, a.hi - b.lo };
		case OpMultiply: return mul(a, b);
		case OpDivide: return divide(a, b);
		case OpNegate: return neg(a);
		case OpSqrt: return { std::sqrt(greater(a.lo, 0.0)), std::sqrt(greater(a.hi, 0.0)) };
		case OpAbs: return absolute(a);
		case OpFloor: return { std::floor(a.lo), std::floor(a.hi) };
		case OpSin: return sine(a);
		case OpCos: return sine({ a.lo + kPi / 2, a.hi + kPi / 2 });
		case OpSign: return { signOf(a.lo), signOf(a.hi) };
		case OpAtan2: return arcTangent(a, b);
		case OpPow: return power(a, b);
		case OpMin: return { lesser(a.lo, b.lo), lesser(a.hi, b.hi) };
		case OpMax: return { greater(a.lo, b.lo), greater(a.hi, b.hi) };
		case OpSmin: return smoothMinimum(a, b, r[s.c]);
		case OpPosSq: return { positiveSquare(a.lo), positiveSquare(a.hi) };
		case OpSelect: {
			const Iv c = r[s.c];
			if (excludesZero(a)) return b;
			if (isZero(a)) return c;
			return { lesser(b.lo, c.lo), greater(b.hi, c.hi) };
		}
		default: return comparison(s.opcode, a, b);
	}
}

// ---- the rewrite of one program over a cell (cut.cpp) ----
bool isPoint(Iv a) { return a.lo == a.hi; }
bool isLiteral(uint8_t op) { return op == OpConstant || op == OpArgument; }
bool isValue(Iv a, double v) { return a.lo == v && a.hi == v; }

uint32_t shortcut(const kdn_step& s, const Iv* r) {
	switch (s.opcode) {
		case OpAdd: case OpSubtract: case OpMultiply: case OpDivide: {
			const double neutral = (s.opcode == OpAdd || s.opcode == OpSubtract) ? 0.0 : 1.0;
			const bool commutes  = s.opcode == OpAdd || s.opcode == OpMultiply;
			if (isValue(r[s.b], neutral)) return s.a;
			if (commutes && isValue(r[s.a], neutral)) return s.b;
			return kNoOperand;
		}
		case OpMin: case OpMax: {
			const bool lowerWins = s.opcode == OpMin;
			if (r[s.a].hi <= r[s.b].lo) return lowerWins ? s.a : s.b;
			if (r[s.b].hi <= r[s.a].lo) return lowerWins ? s.b : s.a;
			return kNoOperand;
		}
		case OpSmin: {
			const double radius = r[s.c].lo;
			const Iv d          = { r[s.a].lo - r[s.b].hi, r[s.a].hi - r[s.b].lo };
			if (d.hi <= -radius) return s.a;
			if (d.lo >= radius) return s.b;
			return kNoOperand;
		}
		case OpAbs: return r[s.a].lo >= 0 ? s.a : kNoOperand;
		case OpSelect: {
			const Iv c = r[s.a];
			if (c.lo > 0 || c.hi < 0) return s.b;
			if (c.lo == 0 && c.hi == 0) return s.c;
			return kNoOperand;
		}
		default: return kNoOperand;
	}
}

kdn_step resolved(kdn_step s, const Iv* r, uint32_t index) {
	if (isPoint(r[index]) && !isLiteral(s.opcode)) {
		kdn_step c = {};
		c.opcode   = OpConstant;
		c.value    = r[index].lo;
		c.leaf     = s.leaf;
		return c;
	}
	if (s.opcode == OpPosSq && r[s.a].lo >= 0) {
		s.opcode = OpMultiply;
		s.b      = s.a;
		return s;
	}
	uint32_t negated = kNoOperand;
	if (s.opcode == OpAbs && r[s.a].hi <= 0) negated = s.a;
	else if (s.opcode == OpSubtract && isValue(r[s.a], 0)) negated = s.b;
	else if (s.opcode == OpMultiply && isValue(r[s.a], -1)) negated = s.b;
	else if (s.opcode == OpMultiply && isValue(r[s.b], -1)) negated = s.a;
	if (negated != kNoOperand) {
		s.opcode = OpNegate;
		s.a      = negated;
		s.b      = 0;
		s.c      = 0;
	}
	return s;
}

kdn_step unsquared(const kdn_step* steps, kdn_step s) {
	if (s.opcode != OpSqrt) return s;
	const kdn_step& inner = steps[s.a];
	if (inner.opcode == OpPosSq) {
		kdn_step positive = inner;
		positive.opcode   = OpMax;
		return positive;
	}
	if (inner.opcode != OpMultiply || inner.a != inner.b) return s;
	s.opcode = OpAbs;
	s.a      = inner.a;
	return s;
}

bool zeroStep(const kdn_step* steps, uint32_t i) { return steps[i].opcode == OpConstant && steps[i].value == 0; }

kdn_step positiveSquared(const kdn_step* steps, kdn_step s) {
	if (s.opcode != OpMultiply || s.a != s.b) return s;
	const kdn_step& inner = steps[s.a];
	if (inner.opcode != OpMax || !(zeroStep(steps, inner.a) || zeroStep(steps, inner.b))) return s;
	const bool zeroFirst = zeroStep(steps, inner.a);
	s.opcode             = OpPosSq;
	s.a                  = zeroFirst ? inner.b : inner.a;
	s.b                  = zeroFirst ? inner.a : inner.b;
	return s;
}

bool sameStep(const kdn_step& a, const kdn_step& b) {
	return a.opcode == b.opcode && a.a == b.a && a.b == b.b && a.c == b.c && std::memcmp(&a.value, &b.value, sizeof(double)) == 0 && a.leaf == b.leaf;
}

struct Scratch {
	std::vector<Iv> iv;
	std::vector<uint32_t> alias, live;
	std::vector<kdn_step> out;
};

// The cut of one program: its range over the box and, where not empty, the
// rewritten and pruned program (null where it is the program itself).
struct ObjectCut {
	Iv range;
	ProgPtr program;
};

ObjectCut cutProgram(const ProgPtr& program, const Iv box[3], Scratch& w) {
	const Prog& p        = *program;
	const uint32_t count = uint32_t(p.steps.size());
	w.iv.resize(count);
	for (uint32_t i = 0; i < count; ++i) w.iv[i] = stepInterval(p.steps[i], w.iv.data(), box);
	const Iv range = w.iv[p.result];
	if (range.lo > 0) return { range, nullptr };
	w.alias.resize(count);
	w.live.resize(count);
	w.out.resize(count);
	for (uint32_t i = 0; i < count; ++i) {
		const kdn_step& orig = p.steps[i];
		if (isLiteral(orig.opcode)) {
			w.alias[i]  = i;
			kdn_step lit = orig;
			lit.b       = 0;
			lit.c       = 0;
			w.out[i]    = lit;
			continue;
		}
		kdn_step s  = orig;
		const int n = operandCount(s.opcode);
		s.a         = n > 0 ? w.alias[orig.a] : orig.a;
		s.b         = n > 1 ? w.alias[orig.b] : 0;
		s.c         = n > 2 ? w.alias[orig.c] : 0;
		s           = positiveSquared(w.out.data(), unsquared(w.out.data(), s));
		const uint32_t other = isPoint(w.iv[i]) ? kNoOperand : shortcut(s, w.iv.data());
		w.alias[i]  = other != kNoOperand ? other : i;
		w.out[i]    = resolved(s, w.iv.data(), i);
	}
	const uint32_t result = w.alias[p.result];
	std::fill(w.live.begin(), w.live.end(), 0u);
	w.live[result] = 1;
	for (uint32_t i = count; i-- > 0;) {
		if (!w.live[i]) continue;
		const kdn_step& s   = w.out[i];
		const int n         = operandCount(s.opcode);
		const uint32_t op[3] = { s.a, s.b, s.c };
		for (int k = 0; k < n; ++k) w.live[op[k]] = 1;
	}
	auto made    = std::make_shared<Prog>();
	made->object = p.object;
	bool all     = true;
	for (uint32_t i = 0; i < count; ++i) all = all && w.live[i] != 0;
	if (all) {
		made->steps.assign(w.out.begin(), w.out.begin() + count);
		made->result = result;
	} else {
		uint32_t kept = 0;
		made->steps.reserve(count);
		for (uint32_t i = 0; i < count; ++i) {
			if (!w.live[i]) continue;
			w.live[i]   = kept++;
			kdn_step m  = w.out[i];
			const int n = operandCount(m.opcode);
			m.a         = n > 0 ? w.live[m.a] : m.a;
			m.b         = n > 1 ? w.live[m.b] : 0;
			m.c         = n > 2 ? w.live[m.c] : 0;
			made->steps.push_back(m);
		}
		made->result = w.live[result];
	}
	bool same = made->result == p.result && made->steps.size() == p.steps.size();
	for (size_t i = 0; same && i < made->steps.size(); ++i) same = sameStep(made->steps[i], p.steps[i]);
	return { range, same ? program : ProgPtr(made) };
}

// cutCell (cut.cpp:463) of the parent's kept programs over one box.
void cutCell(const std::vector<ProgPtr>& parent, const Iv box[3], Cell& cell, Scratch& w) {
	std::vector<ObjectCut> cuts;
	cuts.reserve(parent.size());
	for (const ProgPtr& p : parent) {
		cuts.push_back(cutProgram(p, box, w));
		if (cuts.back().range.hi < 0) {
			cell.occupancy = Filled;
			cell.programs  = { cuts.back().program };
			return;
		}
	}
	double lowest = std::numeric_limits<double>::infinity();
	for (const ObjectCut& c : cuts) lowest = lesser(lowest, c.range.hi);
	cell.programs.clear();
	for (const ObjectCut& c : cuts) {
		const bool surface = !(c.range.lo > 0) && !(c.range.hi < 0);
		if (surface && !(c.range.lo > lowest)) cell.programs.push_back(c.program);
	}
	cell.occupancy = cell.programs.empty() ? Empty : Surface;
}

Iv halfSpan(Iv s, int side) {
	const double middle = (s.lo + s.hi) / 2;
	return { side == 0 ? s.lo : middle, side == 0 ? middle : s.hi };
}

uint32_t stepsOf(const Cell& c) {
	uint32_t s = 0;
	for (const ProgPtr& p : c.programs) s += uint32_t(p->steps.size());
	return s;
}

struct Pending {
	uint32_t cell;
	Iv box[3];
};

template <typename F>
void parallelFor(size_t n, int threads, const F& body) {
	if (threads <= 1 || n < 64) {
		Scratch w;
		for (size_t i = 0; i < n; ++i) body(i, w);
		return;
	}
	std::vector<std::thread> pool;
	std::atomic<size_t> next(0);
	for (int t = 0; t < threads; ++t) {
		pool.emplace_back([&]() {
			Scratch w;
			for (;;) {
				const size_t i = next.fetch_add(16);
				if (i >= n) break;
				for (size_t k = i; k < std::min(n, i + 16); ++k) body(k, w);
			}
		});
	}
	for (std::thread& t : pool) t.join();
}

} // namespace

std::string buildOctree(const std::vector<ProgPtr>& objects, const double lower[3], const double size[3], const BuildOptions& options, Octree& tree) {
	tree = Octree();
	for (int a = 0; a < 3; ++a) {
		tree.lower[a] = lower[a];
		tree.size[a]  = size[a];
	}
	const int threads = std::max(1, std::min(32, int(std::thread::hardware_concurrency())));
	tree.cells.emplace_back();
	tree.cells[0].level = 0;
	Pending root        = { 0, {} };
	for (int a = 0; a < 3; ++a) root.box[a] = { lower[a], lower[a] + size[a] };
	{
		Scratch w;
		cutCell(objects, root.box, tree.cells[0], w);
	}
	std::vector<Pending> level = { root };
	while (!level.empty()) {
		std::vector<Pending> next;
		std::vector<uint32_t> parents;
		for (const Pending& p : level) {
			const Cell& parent = tree.cells[p.cell];
			const bool split   = parent.occupancy == Surface && (int(parent.level) < options.min_depth || (int(parent.level) < options.max_depth && stepsOf(parent) > options.split_steps));
			if (!split) continue;
			// copy what the children need: push_back below may move the cells
			Cell c;
			c.level    = parent.level;
			c.place[0] = parent.place[0];
			c.place[1] = parent.place[1];
			c.place[2] = parent.place[2];
			const uint32_t first = uint32_t(tree.cells.size());
			tree.cells[p.cell].firstChild = int64_t(first);
			for (int o = 0; o < 8; ++o) {
				Cell child;
				child.level    = c.level + 1;
				child.place[0] = c.place[0] * 2 + uint32_t(o & 1);
				child.place[1] = c.place[1] * 2 + uint32_t((o >> 1) & 1);
				child.place[2] = c.place[2] * 2 + uint32_t((o >> 2) & 1);
				tree.cells.push_back(child);
				Pending q = { first + uint32_t(o), { halfSpan(p.box[0], o & 1), halfSpan(p.box[1], (o >> 1) & 1), halfSpan(p.box[2], (o >> 2) & 1) } };
				next.push_back(q);
				parents.push_back(p.cell);
			}
		}
		if (tree.cells.size() > options.max_cells) {
			return "the cut octree passed its cell limit";
		}
		parallelFor(next.size(), threads, [&](size_t i, Scratch& w) {
			cutCell(tree.cells[parents[i]].programs, next[i].box, tree.cells[next[i].cell], w);
		});
		level.swap(next);
	}
	return "";
}

namespace {

// Assign register slots to a straight-line program: a slot is reused once
// the last step that reads its value has run.
std::string slotted(const Prog& p, std::vector<GpuStep>& steps, std::vector<SsaOps>& ssa, GpuProgram& out) {
	const uint32_t n = uint32_t(p.steps.size());
	if (n > kMaxSsa) return "a leaf program holds more than " + std::to_string(kMaxSsa) + " steps";
	std::vector<uint32_t> lastUse(n);
	for (uint32_t i = 0; i < n; ++i) lastUse[i] = i;
	for (uint32_t i = 0; i < n; ++i) {
		const kdn_step& s   = p.steps[i];
		const int k         = operandCount(s.opcode);
		const uint32_t op[3] = { s.a, s.b, s.c };
		for (int j = 0; j < k; ++j) lastUse[op[j]] = std::max(lastUse[op[j]], i);
	}
	lastUse[p.result] = n;
	std::vector<uint8_t> slot(n, 0);
	std::vector<uint8_t> freeSlots;
	uint32_t used = 0;
	out.code      = uint32_t(steps.size());
	for (uint32_t i = 0; i < n; ++i) {
		const kdn_step& s   = p.steps[i];
		const int k         = operandCount(s.opcode);
		const uint32_t op[3] = { s.a, s.b, s.c };
		GpuStep g           = {};
		g.op                = s.opcode;
		g.a                 = k > 0 ? slot[op[0]] : 0;
		g.b                 = k > 1 ? slot[op[1]] : 0;
		g.c                 = k > 2 ? slot[op[2]] : 0;
		g.value             = float(s.value);
		g.leaf              = s.leaf;
		if (s.opcode == OpArgument) g.value = 0.0f;
		for (int j = 0; j < k; ++j) {
			bool first = true;
			for (int m = 0; m < j; ++m) first = first && op[m] != op[j];
			if (first && lastUse[op[j]] == i) freeSlots.push_back(slot[op[j]]);
		}
		if (!freeSlots.empty()) {
			slot[i] = freeSlots.back();
			freeSlots.pop_back();
		} else {
			if (used >= kMaxSlots) return "a leaf program needs more than " + std::to_string(kMaxSlots) + " register slots";
			slot[i] = uint8_t(used++);
		}
		if (lastUse[i] == i) freeSlots.push_back(slot[i]);
		g.dst = slot[i];
		steps.push_back(g);
		SsaOps o = { uint16_t(k > 0 ? op[0] : 0), uint16_t(k > 1 ? op[1] : 0), uint16_t(k > 2 ? op[2] : 0), 0 };
		ssa.push_back(o);
	}
	out.count  = uint16_t(n);
	out.result = uint16_t(p.result);
	out.slot   = slot[p.result];
	out.slots  = uint8_t(std::max(used, 1u));
	out.object = p.object;
	return "";
}

// world.h MarchOp of a reference opcode.
uint8_t marchOpOf(uint8_t op) {
	switch (op) {
		case OpConstant: return MarchConstant;
		case OpPointX: return MarchPointX;
		case OpPointY: return MarchPointY;
		case OpPointZ: return MarchPointZ;
		case OpAdd: return MarchAdd;
		case OpSubtract: return MarchSubtract;
		case OpMultiply: return MarchMultiply;
		case OpSqrt: return MarchSqrt;
		case OpAbs: return MarchAbs;
		case OpMin: return MarchMin;
		case OpMax: return MarchMax;
		case OpPosSq: return MarchPosSq;
		default: return uint8_t(kMarchRare + op);
	}
}

// The march form of a program (world.h MarchOp):
//  - every constant a step reads becomes that step's immediate (one a step,
//    the last constant operand); constants no step reads from a slot any
//    more are left out;
//  - a common operation takes its immediate as b (the operands of +, *, min
//    and max are swapped, const - x is x subtracted from b), a smooth minimum
//    of constant radius carries the radius and 0.25 / radius;
//  - an operand that is the result of the step just before is read from a
//    register (kFromPrevious*), and a result read only that way is not
//    stored (kNoStore) and takes no slot;
//  - the slots are allocated again over what remains.
std::string marchCode(const Prog& p, std::vector<GpuStep>& steps, GpuProgram& out) {
	const uint32_t n = uint32_t(p.steps.size());
	constexpr uint32_t kNone = 0xFFFFFFFFu;
	std::vector<uint8_t> imm(n, 0), needed(n, 0);
	needed[p.result] = 1;
	for (uint32_t i = 0; i < n; ++i) {
		const kdn_step& s    = p.steps[i];
		const int k          = operandCount(s.opcode);
		const uint32_t op[3] = { s.a, s.b, s.c };
		if (s.opcode != OpConstant && s.opcode != OpArgument) {
			for (int j = k - 1; j >= 0; --j) {
				if (p.steps[op[j]].opcode == OpConstant) {
					imm[i] = uint8_t(j + 1);
					break;
				}
			}
		}
		for (int j = 0; j < k; ++j) {
			if (imm[i] != j + 1) needed[op[j]] = 1;
		}
	}
	// the kept steps, and each one's form: op, operand sources (SSA index or kNone), immediate
	struct Form {
		uint8_t op;
		uint8_t imm;
		uint32_t src[3];
		float value;
		uint32_t leaf;
		bool rare;
	};
	std::vector<Form> form(n);
	std::vector<uint32_t> order;
	for (uint32_t i = 0; i < n; ++i) {
		const kdn_step& s = p.steps[i];
		if (s.opcode == OpConstant && !needed[i]) continue;
		order.push_back(i);
		const int k          = operandCount(s.opcode);
		const uint32_t op[3] = { s.a, s.b, s.c };
		Form f;
		f.op    = marchOpOf(s.opcode);
		f.imm   = imm[i];
		f.value = imm[i] ? float(p.steps[op[imm[i] - 1]].value) : (s.opcode == OpArgument ? 0.0f : float(s.value));
		f.leaf  = s.leaf;
		f.rare  = f.op >= kMarchRare;
		for (int j = 0; j < 3; ++j) f.src[j] = j < k && imm[i] != j + 1 ? op[j] : kNone;
		const bool commutes = s.opcode == OpAdd || s.opcode == OpMultiply || s.opcode == OpMin || s.opcode == OpMax;
		if (s.opcode == OpNegate) {
			if (imm[i] == 1) { // a negated constant is a constant
				f.op    = MarchConstant;
				f.imm   = 0;
				f.value = -f.value;
				f.src[0] = kNone;
			} else { // -x as 0 - x
				f.op  = MarchSubtractFrom;
				f.imm = 2;
				f.value = 0.0f;
			}
			f.rare = false;
		} else if (s.opcode == OpSubtract && imm[i] == 1) {
			f.op     = MarchSubtractFrom;
			f.imm    = 2;
			f.src[0] = op[1];
			f.src[1] = kNone;
		} else if (commutes && imm[i] == 1) {
			f.imm    = 2;
			f.src[0] = op[1];
			f.src[1] = kNone;
		} else if (s.opcode == OpSmin && imm[i] == 3 && f.value != 0.0f) {
			const float quarter = 0.25f / f.value;
			f.op                = MarchSminK;
			std::memcpy(&f.leaf, &quarter, sizeof quarter);
		} else if (!f.rare && imm[i] == 1) {
			// a common unary operation of a constant: the general form
			f.op   = uint8_t(kMarchRare + s.opcode);
			f.rare = true;
		}
		if (s.opcode == OpSmin && f.op != MarchSminK) {
			f.op   = uint8_t(kMarchRare + OpSmin);
			f.rare = true;
		}
		form[i] = f;
	}
	// forwarding: an a or b operand that is the step just before
	std::vector<uint16_t> flags(n, 0);
	std::vector<uint8_t> stored(n, 0);
	std::vector<uint32_t> lastRead(n, 0);
	for (size_t e = 0; e < order.size(); ++e) {
		const uint32_t i    = order[e];
		const uint32_t prev = e > 0 ? order[e - 1] : kNone;
		for (int j = 0; j < 3; ++j) {
			const uint32_t src = form[i].src[j];
			if (src == kNone) continue;
			if (j < 2 && src == prev) {
				flags[i] |= uint16_t(j == 0 ? kFromPreviousA : kFromPreviousB);
			} else {
				stored[src]   = 1;
				lastRead[src] = std::max(lastRead[src], i);
			}
		}
	}
	stored[p.result]   = 1;
	lastRead[p.result] = n;
	std::vector<uint8_t> slot(n, 0);
	std::vector<uint8_t> freeSlots;
	uint32_t used = 0;
	out.march     = uint32_t(steps.size());
	for (const uint32_t i : order) {
		const Form& f = form[i];
		GpuStep g     = {};
		g.op          = f.op;
		g.imm         = f.imm;
		g.value       = f.value;
		g.leaf        = f.leaf;
		g.flags       = flags[i];
		g.a           = f.src[0] != kNone && !(flags[i] & kFromPreviousA) ? slot[f.src[0]] : 0;
		g.b           = f.src[1] != kNone && !(flags[i] & kFromPreviousB) ? slot[f.src[1]] : 0;
		g.c           = f.src[2] != kNone ? slot[f.src[2]] : 0;
		// free the slots whose last read is this step (each value once)
		for (int j = 0; j < 3; ++j) {
			const uint32_t src = f.src[j];
			if (src == kNone || (j == 0 && (flags[i] & kFromPreviousA)) || (j == 1 && (flags[i] & kFromPreviousB))) continue;
			bool first = true;
			for (int m = 0; m < j; ++m) {
				const bool viaSlot = !((m == 0 && (flags[i] & kFromPreviousA)) || (m == 1 && (flags[i] & kFromPreviousB)));
				first              = first && !(viaSlot && f.src[m] == src);
			}
			if (first && stored[src] && lastRead[src] == i) freeSlots.push_back(slot[src]);
		}
		if (stored[i]) {
			if (!freeSlots.empty()) {
				slot[i] = freeSlots.back();
				freeSlots.pop_back();
			} else {
				if (used >= kMaxSlots) return "a leaf program needs more than " + std::to_string(kMaxSlots) + " register slots";
				slot[i] = uint8_t(used++);
			}
			g.dst = slot[i];
		} else {
			g.flags |= kNoStore;
		}
		steps.push_back(g);
	}
	out.marchCount = uint16_t(order.size());
	out.marchSlot  = slot[p.result];
	out.marchSlots = uint8_t(std::max(used, 1u));
	return "";
}

} // namespace

std::string flattenOctree(const Octree& tree, FlatWorld& flat) {
	flat = FlatWorld();
	flat.nodes.resize(tree.cells.size());
	std::unordered_map<const Prog*, uint32_t> made;
	for (size_t i = 0; i < tree.cells.size(); ++i) {
		const Cell& c = tree.cells[i];
		if (c.firstChild >= 0) {
			flat.nodes[i] = int32_t(c.firstChild);
			continue;
		}
		if (c.programs.size() > kMaxLeafProgs) return "a leaf keeps more than " + std::to_string(kMaxLeafProgs) + " programs";
		GpuLeaf leaf   = {};
		leaf.occupancy = c.occupancy;
		leaf.count     = uint16_t(c.programs.size());
		leaf.first     = uint32_t(flat.leafPrograms.size());
		uint32_t slots = 1;
		for (const ProgPtr& p : c.programs) {
			auto found = made.find(p.get());
			uint32_t index;
			if (found == made.end()) {
				GpuProgram g     = {};
				std::string error = slotted(*p, flat.steps, flat.ssa, g);
				if (!error.empty()) return error;
				error = marchCode(*p, flat.march, g);
				if (!error.empty()) return error;
				index = uint32_t(flat.programs.size());
				flat.programs.push_back(g);
				made.emplace(p.get(), index);
			} else {
				index = found->second;
			}
			slots = std::max<uint32_t>(slots, flat.programs[index].slots);
			flat.leafPrograms.push_back(index);
		}
		leaf.slots    = uint8_t(slots);
		flat.nodes[i] = ~int32_t(flat.leaves.size());
		flat.leaves.push_back(leaf);
	}
	// Each leaf names its programs through an indirection; the kernel reads
	// them as one run, so lay the GpuPrograms out per leaf.
	std::vector<GpuProgram> runs;
	runs.reserve(flat.leafPrograms.size());
	for (uint32_t k : flat.leafPrograms) runs.push_back(flat.programs[k]);
	flat.programs.swap(runs);
	return "";
}

std::vector<GridCell> gridOf(const FlatWorld& flat, uint32_t level) {
	const uint32_t side = 1u << level;
	std::vector<GridCell> grid(size_t(side) * side * side);
	for (uint32_t z = 0; z < side; ++z) {
		for (uint32_t y = 0; y < side; ++y) {
			for (uint32_t x = 0; x < side; ++x) {
				int32_t node = flat.nodes[0];
				uint32_t at  = 0;
				for (; at < level && node >= 0; ++at) {
					// the child of the cell holding (x, y, z): its bit at this level per axis
					const uint32_t shift = level - 1 - at;
					const uint32_t o     = ((x >> shift) & 1u) | (((y >> shift) & 1u) << 1) | (((z >> shift) & 1u) << 2);
					node                 = flat.nodes[size_t(node) + o];
				}
				grid[(size_t(z) * side + y) * side + x] = GridCell { node, at };
			}
		}
	}
	return grid;
}

} // namespace kdn
