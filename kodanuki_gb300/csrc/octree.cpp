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

// The march form of a program (world.h MarchStep).
namespace march {

// Where a lowered value lives: the result of lowered step `node`, an
// immediate (kept in double until it is written), or a reserved slot (0, 1,
// -1, the point's coordinates).  `from` is the reference step whose value
// it is; `shared` marks a value read around a negation, which another step
// may still read.
struct Operand {
	enum Kind : uint8_t { Node, Immediate, Reserved } kind = Reserved;
	uint32_t node = 0;
	double value  = 0.0;
	uint8_t slot  = SlotZero;
	uint32_t from = 0xFFFFFFFFu;
	bool shared   = false;
};

Operand immediate(double v) {
	Operand o;
	o.kind  = Operand::Immediate;
	o.value = v;
	return o;
}
Operand reserved(uint8_t slot) {
	Operand o;
	o.kind = Operand::Reserved;
	o.slot = slot;
	return o;
}

// r = post(fma(a, b, c), w), or a rare reference operation over a, b, c.
struct Node {
	bool rare     = false;
	uint8_t refOp = 0;
	Operand a, b, c, w;
	uint8_t post  = PostNone;
	double radius = 0.0;
	bool negation = false; // fma(x, -1, 0): -x
	bool product  = false; // fma(x, y, 0) from a multiplication
};

// sdf/program.cpp:57 runStep in double, for steps of constants alone.
double folded(uint8_t op, double a, double b, double c) {
	switch (op) {
		case OpAdd: return a + b;
		case OpSubtract: return a - b;
		case OpMultiply: return a * b;
		case OpDivide: return a / b;
		case OpNegate: return -a;
		case OpSqrt: return std::sqrt(a);
		case OpAbs: return std::fabs(a);
		case OpFloor: return std::floor(a);
		case OpSin: return std::sin(a);
		case OpCos: return std::cos(a);
		case OpSign: return signOf(a);
		case OpAtan2: return std::atan2(a, b);
		case OpPow: return std::pow(a, b);
		case OpMin: return lesser(a, b);
		case OpMax: return greater(a, b);
		case OpSmin: return smoothMin(a, b, c);
		case OpPosSq: return positiveSquare(a);
		case OpLess: return a < b ? 1.0 : 0.0;
		case OpLessEq: return a <= b ? 1.0 : 0.0;
		case OpEqual: return a == b ? 1.0 : 0.0;
		case OpNotEqual: return a != b ? 1.0 : 0.0;
		case OpAnd: return a != 0.0 && b != 0.0 ? 1.0 : 0.0;
		case OpOr: return a != 0.0 || b != 0.0 ? 1.0 : 0.0;
		case OpNot: return a == 0.0 ? 1.0 : 0.0;
		case OpSelect: return a != 0.0 ? b : c;
		default: return 0.0;
	}
}

struct Lowering {
	std::vector<Node> nodes;
	std::vector<uint32_t> refUses; // consumers of each reference step (the result counts one)

	Operand make(const Node& n, uint32_t from) {
		nodes.push_back(n);
		Operand o;
		o.kind = Operand::Node;
		o.node = uint32_t(nodes.size() - 1);
		o.from = from;
		return o;
	}
	static int immediates(const Node& n) {
		return (n.a.kind == Operand::Immediate) + (n.b.kind == Operand::Immediate) + (n.c.kind == Operand::Immediate) +
		       (n.w.kind == Operand::Immediate) + (n.post == PostSminK ? 1 : 0);
	}
	// a step that may take on more: its value has one reader, this one
	bool open(const Operand& o) const {
		return o.kind == Operand::Node && !o.shared && o.from != 0xFFFFFFFFu && refUses[o.from] == 1 && !nodes[o.node].rare &&
		       nodes[o.node].post == PostNone;
	}
	// an immediate as a step of its own, where a step has room for one
	Operand alone(const Operand& o, uint32_t from) {
		if (o.kind != Operand::Immediate) return o;
		Node n;
		n.a = o;
		n.b = reserved(SlotOne);
		n.c = reserved(SlotZero);
		Operand r = make(n, from);
		r.shared  = true;
		return r;
	}
};

} // namespace march

// Lower a program to the march form (world.h MarchStep): constants become
// immediates (a step of constants alone is folded in double), the point is
// read from reserved slots, +, -, * and negation become fused multiply-adds,
// a product read only by a sum folds into it, double negations cancel, and
// sqrt, |x|, max(x, 0)^2, min, max and a smooth minimum of constant radius
// ride on the step that makes their operand where nothing else reads it.
// Slots are then allocated over the steps the result needs.
std::string marchCode(const Prog& p, std::vector<MarchStep>& steps, GpuProgram& out) {
	using namespace march;
	const uint32_t n = uint32_t(p.steps.size());
	Lowering L;
	L.refUses.assign(n, 0);
	for (uint32_t i = 0; i < n; ++i) {
		const kdn_step& s    = p.steps[i];
		const uint32_t op[3] = { s.a, s.b, s.c };
		for (int j = 0; j < operandCount(s.opcode); ++j) L.refUses[op[j]] += 1;
	}
	L.refUses[p.result] += 1;
	const Operand zero = reserved(SlotZero), one = reserved(SlotOne), minusOne = reserved(SlotMinusOne);
	const auto fma3 = [](const Operand& a, const Operand& b, const Operand& c) {
		Node f;
		f.a = a;
		f.b = b;
		f.c = c;
		return f;
	};
	std::vector<Operand> val(n);
	for (uint32_t i = 0; i < n; ++i) {
		const kdn_step& s = p.steps[i];
		const int k       = operandCount(s.opcode);
		const Operand A = k > 0 ? val[s.a] : zero, B = k > 1 ? val[s.b] : zero, C = k > 2 ? val[s.c] : zero;
		switch (s.opcode) {
			case OpConstant: val[i] = immediate(s.value); continue;
			case OpArgument: case OpNormalX: case OpNormalY: case OpNormalZ: val[i] = immediate(0.0); continue;
			case OpPointX: val[i] = reserved(SlotX); continue;
			case OpPointY: val[i] = reserved(SlotY); continue;
			case OpPointZ: val[i] = reserved(SlotZ); continue;
			default: break;
		}
		if (k > 0 && A.kind == Operand::Immediate && (k < 2 || B.kind == Operand::Immediate) && (k < 3 || C.kind == Operand::Immediate)) {
			val[i] = immediate(folded(s.opcode, A.value, B.value, C.value));
			continue;
		}
		const auto isNeg = [&](const Operand& o) { return o.kind == Operand::Node && L.nodes[o.node].negation; };
		const auto inner = [&](const Operand& o) {
			Operand x = L.nodes[o.node].a;
			x.shared  = true;
			return x;
		};
		switch (s.opcode) {
			case OpNegate: {
				if (isNeg(A)) {
					val[i] = inner(A); // -(-x) = x
				} else {
					Node f     = fma3(A, minusOne, zero);
					f.negation = true;
					val[i]     = L.make(f, i);
				}
				continue;
			}
			case OpAdd: case OpSubtract: {
				// x + y or x - y; x + (-y) = x - y, x - (-y) = x + y, (-x) + y = y - x
				Operand x = A, y = B;
				bool minus = s.opcode == OpSubtract;
				if (isNeg(y)) {
					y     = inner(y);
					minus = !minus;
				} else if (!minus && isNeg(x)) {
					const Operand t = inner(x);
					x               = y;
					y               = t;
					minus           = true;
				}
				if (!minus) {
					// a product read only here: fma(p, q, other)
					const Operand* pr[2] = { &x, &y };
					bool done            = false;
					for (int j = 0; j < 2 && !done; ++j) {
						const Operand& m = *pr[j];
						if (!L.open(m) || !L.nodes[m.node].product) continue;
						const Node f = fma3(L.nodes[m.node].a, L.nodes[m.node].b, *pr[1 - j]);
						if (Lowering::immediates(f) > 1) continue;
						val[i] = L.make(f, i);
						done   = true;
					}
					if (done) continue;
					val[i] = L.make(fma3(x, one, y), i);
				} else {
					val[i] = L.make(fma3(y, minusOne, x), i);
				}
				continue;
			}
			case OpMultiply: {
				Operand x = A, y = B;
				if (isNeg(x) && isNeg(y)) {
					x = inner(x);
					y = inner(y);
				}
				Node f    = fma3(x, y, zero);
				f.product = true;
				if (Lowering::immediates(f) > 1) f.a = L.alone(f.a, i);
				val[i] = L.make(f, i);
				continue;
			}
			case OpSqrt: case OpAbs: case OpPosSq: {
				const uint8_t post = s.opcode == OpSqrt ? PostSqrt : (s.opcode == OpAbs ? PostAbs : PostPosSq);
				if (L.open(A)) {
					Node& f    = L.nodes[A.node];
					f.post     = post;
					f.product  = false;
					f.negation = false;
					val[i]     = A;
					val[i].from = i;
				} else {
					Node f = fma3(A, one, zero);
					f.post = post;
					val[i] = L.make(f, i);
				}
				continue;
			}
			case OpMin: case OpMax: case OpSmin: {
				const bool smooth = s.opcode == OpSmin;
				if (smooth && !(C.kind == Operand::Immediate && C.value != 0.0)) break; // a rare step
				const uint8_t post = smooth ? PostSminK : (s.opcode == OpMin ? PostMin : PostMax);
				Operand x = A, y = B;
				if (smooth) { // the radius takes the step's immediate
					x = L.alone(x, i);
					y = L.alone(y, i);
				}
				// ride on the step making one operand (the operations are symmetric); the other is w
				Operand host = x, other = y;
				bool ride    = L.open(x);
				if (!ride && L.open(y)) {
					host  = y;
					other = x;
					ride  = true;
				}
				Operand wOp = other;
				Node f      = ride ? L.nodes[host.node] : fma3(host, one, zero);
				f.post      = post;
				f.w         = wOp;
				f.radius    = smooth ? C.value : 0.0;
				f.product   = false;
				f.negation  = false;
				if (Lowering::immediates(f) > 1 && wOp.kind == Operand::Immediate) {
					// w an immediate beside the step's own: w as a step of its own
					wOp = L.alone(other, i);
					f.w = wOp;
				}
				if (Lowering::immediates(f) > 1) {
					// the riding step's immediate beside the radius: a step of its own
					ride     = false;
					f        = fma3(host, one, zero);
					f.post   = post;
					f.w      = wOp;
					f.radius = smooth ? C.value : 0.0;
				}
				// the riding step is made again after its new operand w (the old one
				// has no reader left), so every step still follows what it reads
				val[i] = L.make(f, i);
				continue;
			}
			default: break;
		}
		// a rare step: the reference operation over slots, one immediate at most
		Node r;
		r.rare  = true;
		r.refOp = s.opcode;
		r.a     = A;
		r.b     = k > 1 ? B : zero;
		r.c     = k > 2 ? C : zero;
		bool seen = false;
		for (Operand* o : { &r.a, &r.b, &r.c }) {
			if (o->kind != Operand::Immediate) continue;
			if (seen) *o = L.alone(*o, i);
			seen = true;
		}
		val[i] = L.make(r, i);
	}
	// the result as a step
	Operand result = val[p.result];
	if (result.kind != Operand::Node) result = L.make(fma3(result, one, zero), p.result);
	// the steps the result needs, and each one's last reader
	const uint32_t m = uint32_t(L.nodes.size());
	std::vector<uint8_t> live(m, 0);
	live[result.node] = 1;
	for (uint32_t j = m; j-- > 0;) {
		if (!live[j]) continue;
		const Node& x = L.nodes[j];
		for (const Operand* o : { &x.a, &x.b, &x.c, &x.w }) {
			if (o->kind == Operand::Node) live[o->node] = 1;
		}
	}
	std::vector<uint32_t> lastRead(m, 0);
	for (uint32_t j = 0; j < m; ++j) {
		if (!live[j]) continue;
		const Node& x   = L.nodes[j];
		const bool usesW = x.post == PostMin || x.post == PostMax || x.post == PostSminK;
		for (const Operand* o : { &x.a, &x.b, &x.c, &x.w }) {
			if (o == &x.w && !usesW) continue;
			if (o->kind == Operand::Node) lastRead[o->node] = std::max(lastRead[o->node], j);
		}
	}
	lastRead[result.node] = m;
	std::vector<uint8_t> slot(m, 0);
	std::vector<uint8_t> freeSlots;
	uint32_t used = kMarchFirstSlot;
	uint32_t kept = 0;
	out.march     = uint32_t(steps.size());
	for (uint32_t j = 0; j < m; ++j) {
		if (!live[j]) continue;
		const Node& x    = L.nodes[j];
		const bool usesW = x.post == PostMin || x.post == PostMax || x.post == PostSminK;
		MarchStep g      = {};
		g.op             = x.rare ? uint8_t(kMarchRare + x.refOp) : x.post;
		double immValue  = 0.0;
		const auto slotOf = [&](const Operand& o) -> uint8_t {
			if (o.kind == Operand::Node) return slot[o.node];
			if (o.kind == Operand::Immediate) {
				immValue = o.value;
				return SlotImm;
			}
			return o.slot;
		};
		g.a       = slotOf(x.a);
		g.b       = slotOf(x.b);
		g.c       = slotOf(x.c);
		g.w       = usesW ? slotOf(x.w) : uint8_t(SlotZero);
		g.value   = float(x.post == PostSminK ? x.radius : immValue);
		g.quarter = x.post == PostSminK ? float(0.25 / x.radius) : 0.0f;
		// free the slots read here for the last time (each value once)
		const Operand* reads[4] = { &x.a, &x.b, &x.c, &x.w };
		for (int r = 0; r < 4; ++r) {
			const Operand* o = reads[r];
			if (r == 3 && !usesW) continue;
			if (o->kind != Operand::Node || lastRead[o->node] != j) continue;
			bool first = true;
			for (int q = 0; q < r; ++q) first = first && !(reads[q]->kind == Operand::Node && reads[q]->node == o->node);
			if (first) freeSlots.push_back(slot[o->node]);
		}
		if (!freeSlots.empty()) {
			slot[j] = freeSlots.back();
			freeSlots.pop_back();
		} else {
			if (used >= kMaxSlots) return "a leaf program needs more than " + std::to_string(kMaxSlots) + " register slots";
			slot[j] = uint8_t(used++);
		}
		if (lastRead[j] == j) freeSlots.push_back(slot[j]);
		g.dst = slot[j];
		steps.push_back(g);
		++kept;
	}
	out.marchCount = uint16_t(kept);
	out.marchSlot  = slot[result.node];
	out.marchSlots = uint8_t(used);
	return "";
}

} // namespace

std::string flattenOctree(const Octree& tree, FlatWorld& flat) {
	flat = FlatWorld();
	flat.nodes.resize(tree.cells.size());
	// the distinct programs, in the order the leaves first name them
	std::unordered_map<const Prog*, uint32_t> made;
	std::vector<const Prog*> order;
	std::vector<uint32_t> named; // each leaf's programs, in leaf order
	for (size_t i = 0; i < tree.cells.size(); ++i) {
		const Cell& c = tree.cells[i];
		if (c.firstChild >= 0) continue;
		if (c.programs.size() > kMaxLeafProgs) return "a leaf keeps more than " + std::to_string(kMaxLeafProgs) + " programs";
		for (const ProgPtr& p : c.programs) {
			auto found = made.find(p.get());
			if (found == made.end()) {
				found = made.emplace(p.get(), uint32_t(order.size())).first;
				order.push_back(p.get());
			}
			named.push_back(found->second);
		}
	}
	// Compile them on every core: contiguous runs of the order, each into
	// its own buffers (offsets from the run's start), then laid end to end
	// in order, so the layout is the one a single thread would make.
	struct Run {
		size_t first, end;
		std::vector<GpuProgram> programs;
		std::vector<GpuStep> steps;
		std::vector<SsaOps> ssa;
		std::vector<MarchStep> march;
		std::string error;
		size_t failed = SIZE_MAX;
	};
	const int threads = std::max(1, std::min(32, int(std::thread::hardware_concurrency())));
	const size_t runCount = std::max<size_t>(1, std::min<size_t>(order.size() / 256 + 1, size_t(threads) * 8));
	std::vector<Run> runs(runCount);
	for (size_t r = 0; r < runCount; ++r) {
		runs[r].first = order.size() * r / runCount;
		runs[r].end   = order.size() * (r + 1) / runCount;
	}
	parallelFor(runCount, runCount < 64 ? 1 : threads, [&](size_t r, Scratch&) {
		Run& run = runs[r];
		run.programs.reserve(run.end - run.first);
		for (size_t k = run.first; k < run.end; ++k) {
			GpuProgram g = {};
			std::string error = slotted(*order[k], run.steps, run.ssa, g);
			if (error.empty()) error = marchCode(*order[k], run.march, g);
			if (!error.empty()) {
				run.error  = error;
				run.failed = k;
				return;
			}
			run.programs.push_back(g);
		}
	});
	for (const Run& run : runs) {
		if (!run.error.empty()) return run.error;
	}
	std::vector<size_t> stepBase(runCount), marchBase(runCount);
	size_t stepTotal = 0, marchTotal = 0;
	for (size_t r = 0; r < runCount; ++r) {
		stepBase[r]  = stepTotal;
		marchBase[r] = marchTotal;
		stepTotal += runs[r].steps.size();
		marchTotal += runs[r].march.size();
	}
	std::vector<GpuProgram> programs(order.size());
	flat.steps.resize(stepTotal);
	flat.ssa.resize(stepTotal);
	flat.march.resize(marchTotal);
	parallelFor(runCount, runCount < 64 ? 1 : threads, [&](size_t r, Scratch&) {
		const Run& run = runs[r];
		std::copy(run.steps.begin(), run.steps.end(), flat.steps.begin() + std::ptrdiff_t(stepBase[r]));
		std::copy(run.ssa.begin(), run.ssa.end(), flat.ssa.begin() + std::ptrdiff_t(stepBase[r]));
		std::copy(run.march.begin(), run.march.end(), flat.march.begin() + std::ptrdiff_t(marchBase[r]));
		for (size_t k = 0; k < run.programs.size(); ++k) {
			GpuProgram g = run.programs[k];
			g.code += uint32_t(stepBase[r]);
			g.march += uint32_t(marchBase[r]);
			programs[run.first + k] = g;
		}
	});
	// the leaves; each names its programs through an indirection, and the
	// kernel reads them as one run, so the GpuPrograms are laid out per leaf
	flat.programs.reserve(named.size());
	size_t at = 0;
	for (size_t i = 0; i < tree.cells.size(); ++i) {
		const Cell& c = tree.cells[i];
		if (c.firstChild >= 0) {
			flat.nodes[i] = int32_t(c.firstChild);
			continue;
		}
		GpuLeaf leaf   = {};
		leaf.occupancy = c.occupancy;
		leaf.count     = uint16_t(c.programs.size());
		leaf.first     = uint32_t(flat.programs.size());
		uint32_t slots = 1;
		for (size_t k = 0; k < c.programs.size(); ++k) {
			const GpuProgram& g = programs[named[at++]];
			slots               = std::max<uint32_t>(slots, g.slots);
			flat.programs.push_back(g);
		}
		leaf.slots = uint8_t(slots);
		if (leaf.count > 0) {
			const GpuProgram& g = flat.programs[leaf.first];
			leaf.march          = g.march;
			leaf.marchCount     = g.marchCount;
			leaf.marchSlot      = g.marchSlot;
		}
		flat.nodes[i] = ~int32_t(flat.leaves.size());
		flat.leaves.push_back(leaf);
	}
	return "";
}

std::vector<float> gridWallsOf(const float lower[3], const float size[3], uint32_t level) {
	const uint32_t n = 1u << level;
	std::vector<float> walls(3 * size_t(n + 1));
	for (int a = 0; a < 3; ++a) {
		float* w = walls.data() + size_t(a) * (n + 1);
		w[0]     = lower[a];
		w[n]     = lower[a] + size[a];
		for (uint32_t stride = n; stride > 1; stride /= 2) {
			for (uint32_t i = 0; i < n; i += stride) {
				const volatile float sum = w[i] + w[i + stride]; // as the descent: the sum, then the half
				w[i + stride / 2]        = 0.5f * sum;
			}
		}
	}
	return walls;
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
