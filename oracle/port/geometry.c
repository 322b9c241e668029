/*
 * Oracle geometry: SDF programs over double, intervals and duals; the
 * interval cut of programs to a cell; the cut octree; sphere tracing.
 * Test infrastructure only (see kdn_port.h).
 */
#include "kdn_port.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define KP_PI 3.14159265358979323846
#define NO_OPERAND 0xFFFFFFFFu
#define NO_LEAF 0xFFFFFFFFu

/* sdf/program.cpp:15 operandCount */
static int operand_count(int op) {
	switch (op) {
		case KP_CONSTANT: case KP_ARGUMENT: case KP_POINTX: case KP_POINTY: case KP_POINTZ:
		case KP_NORMALX: case KP_NORMALY: case KP_NORMALZ: return 0;
		case KP_NEGATE: case KP_SQRT: case KP_ABS: case KP_FLOOR: case KP_SIN: case KP_COS: case KP_SIGN: case KP_NOT: return 1;
		case KP_SELECT: case KP_SMIN: return 3;
		default: return 2;
	}
}

/* ---------------- double (sdf/numbers.cpp:107-190) ---------------- */
static double truth(int b) { return b ? 1.0 : 0.0; }
static double dmin(double a, double b) { return b < a ? b : a; } /* std::min */
static double dmax(double a, double b) { return a < b ? b : a; } /* std::max */

static double smooth_min(double a, double b, double r) {
	const double blend = dmax(r - fabs(a - b), 0.0) / r;
	return dmin(a, b) - blend * blend * r * 0.25;
}

static double pos_sq(double a) {
	const double p = dmax(a, 0.0);
	return p * p;
}

static double compare_d(int op, double a, double b) {
	switch (op) {
		case KP_LESS: return truth(a < b);
		case KP_LESSEQ: return truth(a <= b);
		case KP_EQUAL: return truth(a == b);
		case KP_NOTEQUAL: return truth(a != b);
		case KP_AND: return truth(a != 0 && b != 0);
		case KP_OR: return truth(a != 0 || b != 0);
		default: return truth(a == 0); /* Not: compare(Equal, a, 0) */
	}
}

static double step_d(const kp_step* s, const double* r, const double pt[3], const double* n, const double* arguments) {
	const double a = r[s->a], b = r[s->b];
	switch (s->opcode) {
		case KP_CONSTANT: return s->value;
		case KP_ARGUMENT: return arguments ? arguments[s->a] : 0.0;
		case KP_POINTX: return pt[0];
		case KP_POINTY: return pt[1];
		case KP_POINTZ: return pt[2];
		case KP_NORMALX: return n ? n[0] : 0.0;
		case KP_NORMALY: return n ? n[1] : 0.0;
		case KP_NORMALZ: return n ? n[2] : 0.0;
		case KP_ADD: return a + b;
		case KP_SUBTRACT: return a - b;
		case KP_MULTIPLY: return a * b;
		case KP_DIVIDE: return a / b;
		case KP_NEGATE: return -a;
		case KP_SQRT: return sqrt(a);
		case KP_ABS: return fabs(a);
		case KP_FLOOR: return floor(a);
		case KP_SIN: return sin(a);
		case KP_COS: return cos(a);
		case KP_SIGN: return a > 0 ? 1.0 : (a < 0 ? -1.0 : 0.0);
		case KP_ATAN2: return atan2(a, b);
		case KP_POW: return pow(a, b);
		case KP_MIN: return dmin(a, b);
		case KP_MAX: return dmax(a, b);
		case KP_SMIN: return smooth_min(a, b, r[s->c]);
		case KP_POSSQ: return pos_sq(a);
		case KP_SELECT: return a != 0 ? b : r[s->c];
		default: return compare_d(s->opcode, a, b);
	}
}

double kp_eval(const kp_program* p, const double pt[3], double* regs) {
	for (uint32_t i = 0; i < p->count; ++i) {
		regs[i] = step_d(&p->steps[i], regs, pt, NULL, NULL);
	}
	return regs[p->result];
}

double kp_eval_inputs(const kp_program* p, const double pt[3], const double n[3], const double* arguments, double* regs) {
	for (uint32_t i = 0; i < p->count; ++i) {
		regs[i] = step_d(&p->steps[i], regs, pt, n, arguments);
	}
	return regs[p->result];
}

/* ---------------- intervals (sdf/numbers.cpp:200-432) ---------------- */
static kp_interval iv(double l, double u) {
	kp_interval r = { l, u };
	return r;
}

static kp_interval hull4(double a, double b, double c, double d) {
	/* std::min / std::max over an initializer list keep the first extreme */
	double lo = a, hi = a;
	if (b < lo) lo = b;
	if (c < lo) lo = c;
	if (d < lo) lo = d;
	if (hi < b) hi = b;
	if (hi < c) hi = c;
	if (hi < d) hi = d;
	return iv(lo, hi);
}

static kp_interval i_mul(kp_interval a, kp_interval b) {
	return hull4(a.lower * b.lower, a.lower * b.upper, a.upper * b.lower, a.upper * b.upper);
}

static int contains_zero(kp_interval a) { return a.lower <= 0 && a.upper >= 0; }

static kp_interval i_div(kp_interval a, kp_interval b) {
	if (contains_zero(b)) return iv(-INFINITY, INFINITY);
	return i_mul(a, iv(1 / b.upper, 1 / b.lower));
}

static kp_interval i_neg(kp_interval a) { return iv(-a.upper, -a.lower); }

static kp_interval i_abs(kp_interval a) {
	if (a.lower >= 0) return a;
	if (a.upper <= 0) return i_neg(a);
	return iv(0, dmax(-a.lower, a.upper));
}

static int reaches(kp_interval a, double offset) {
	const double k = ceil((a.lower - offset) / (2 * KP_PI));
	return offset + 2 * KP_PI * k <= a.upper;
}

static kp_interval i_sin(kp_interval a) {
	if (a.upper - a.lower >= 2 * KP_PI) return iv(-1, 1);
	const double s0 = sin(a.lower), s1 = sin(a.upper);
	kp_interval out = iv(dmin(s0, s1), dmax(s0, s1));
	if (reaches(a, KP_PI / 2)) out.upper = 1;
	if (reaches(a, -KP_PI / 2)) out.lower = -1;
	return out;
}

static double sign_d(double a) { return a > 0 ? 1.0 : (a < 0 ? -1.0 : 0.0); }

static kp_interval i_atan2(kp_interval y, kp_interval x) {
	const int near_origin = contains_zero(x) && contains_zero(y);
	const int across_cut = x.lower < 0 && contains_zero(y);
	if (near_origin || across_cut) return iv(-KP_PI, KP_PI);
	return hull4(atan2(y.lower, x.lower), atan2(y.lower, x.upper), atan2(y.upper, x.lower), atan2(y.upper, x.upper));
}

static kp_interval whole_power(kp_interval a, double n) {
	if (n >= 0 && fmod(n, 2.0) == 0) {
		const kp_interval m = i_abs(a);
		return iv(pow(m.lower, n), pow(m.upper, n));
	}
	if (n > 0) return iv(pow(a.lower, n), pow(a.upper, n));
	return i_div(iv(1, 1), whole_power(a, -n));
}

static kp_interval i_pow(kp_interval a, kp_interval b) {
	if (b.lower == b.upper && b.lower == floor(b.lower)) return whole_power(a, b.lower);
	if (a.lower <= 0) return iv(-INFINITY, INFINITY);
	return hull4(pow(a.lower, b.lower), pow(a.lower, b.upper), pow(a.upper, b.lower), pow(a.upper, b.upper));
}

static kp_interval decided(int yes, int no) { return iv(yes ? 1.0 : 0.0, no ? 0.0 : 1.0); }
static int excludes_zero(kp_interval a) { return a.lower > 0 || a.upper < 0; }
static int is_zero(kp_interval a) { return a.lower == 0 && a.upper == 0; }

static kp_interval i_compare(int op, kp_interval a, kp_interval b) {
	const int apart = a.upper < b.lower || b.upper < a.lower;
	const int same = a.lower == a.upper && b.lower == b.upper && a.lower == b.lower;
	switch (op) {
		case KP_LESS: return decided(a.upper < b.lower, a.lower >= b.upper);
		case KP_LESSEQ: return decided(a.upper <= b.lower, a.lower > b.upper);
		case KP_EQUAL: return decided(same, apart);
		case KP_NOTEQUAL: return decided(apart, same);
		case KP_AND: return decided(excludes_zero(a) && excludes_zero(b), is_zero(a) || is_zero(b));
		case KP_OR: return decided(excludes_zero(a) || excludes_zero(b), is_zero(a) && is_zero(b));
		default: {
			/* Not = compare(Equal, a, constant 0) */
			const kp_interval z = iv(0, 0);
			const int ap = a.upper < z.lower || z.upper < a.lower;
			const int sm = a.lower == a.upper && a.lower == 0;
			return decided(sm, ap);
		}
	}
}

static kp_interval i_smin(kp_interval a, kp_interval b, kp_interval r) {
	const double lower = smooth_min(a.lower, b.lower, r.lower);
	const double upper = smooth_min(a.upper, b.upper, r.lower);
	return iv(isnan(lower) ? dmin(a.lower, b.lower) - r.lower / 4 : lower, isnan(upper) ? dmin(a.upper, b.upper) : upper);
}

static kp_interval step_i(const kp_step* s, const kp_interval* r, const kp_interval box[3]) {
	const kp_interval a = r[s->a], b = r[s->b];
	switch (s->opcode) {
		case KP_CONSTANT: return iv(s->value, s->value);
		case KP_ARGUMENT: return iv(0, 0);
		case KP_POINTX: return box[0];
		case KP_POINTY: return box[1];
		case KP_POINTZ: return box[2];
		case KP_NORMALX: case KP_NORMALY: case KP_NORMALZ: return iv(0, 0);
		case KP_ADD: return iv(a.lower + b.lower, a.upper + b.upper);
		case KP_SUBTRACT: return iv(a.lower - b.upper, a.upper - b.lower);
		case KP_MULTIPLY: return i_mul(a, b);
		case KP_DIVIDE: return i_div(a, b);
		case KP_NEGATE: return i_neg(a);
		case KP_SQRT: return iv(sqrt(dmax(a.lower, 0.0)), sqrt(dmax(a.upper, 0.0)));
		case KP_ABS: return i_abs(a);
		case KP_FLOOR: return iv(floor(a.lower), floor(a.upper));
		case KP_SIN: return i_sin(a);
		case KP_COS: return i_sin(iv(a.lower + KP_PI / 2, a.upper + KP_PI / 2));
		case KP_SIGN: return iv(sign_d(a.lower), sign_d(a.upper));
		case KP_ATAN2: return i_atan2(a, b);
		case KP_POW: return i_pow(a, b);
		case KP_MIN: return iv(dmin(a.lower, b.lower), dmin(a.upper, b.upper));
		case KP_MAX: return iv(dmax(a.lower, b.lower), dmax(a.upper, b.upper));
		case KP_SMIN: return i_smin(a, b, r[s->c]);
		case KP_POSSQ: return iv(pos_sq(a.lower), pos_sq(a.upper));
		case KP_SELECT: {
			const kp_interval c = r[s->c];
			if (excludes_zero(a)) return b;
			if (is_zero(a)) return c;
			return iv(dmin(b.lower, c.lower), dmax(b.upper, c.upper));
		}
		default: return i_compare(s->opcode, a, b);
	}
}

kp_interval kp_eval_interval(const kp_program* p, const kp_interval box[3], kp_interval* regs) {
	for (uint32_t i = 0; i < p->count; ++i) {
		regs[i] = step_i(&p->steps[i], regs, box);
	}
	return regs[p->result];
}

/* ---------------- duals (sdf/numbers.cpp:440-590) ---------------- */
static kp_dual dconst(double v) {
	kp_dual d = { v, { 0, 0, 0 } };
	return d;
}

static kp_dual chain1(kp_dual a, double f, double d1) {
	kp_dual o = dconst(f);
	for (int i = 0; i < 3; ++i) o.g[i] = d1 * a.g[i];
	return o;
}

static kp_dual chain2(kp_dual a, kp_dual b, double f, double fa, double fb) {
	kp_dual o = dconst(f);
	for (int i = 0; i < 3; ++i) o.g[i] = fa * a.g[i] + fb * b.g[i];
	return o;
}

static double clampd(double x, double lo, double hi) { return x < lo ? lo : (hi < x ? hi : x); }

static kp_dual step_dual(const kp_step* s, const kp_dual* r, const double pt[3]) {
	const kp_dual a = r[s->a], b = r[s->b];
	switch (s->opcode) {
		case KP_CONSTANT: return dconst(s->value);
		case KP_ARGUMENT: return dconst(0);
		case KP_POINTX: case KP_POINTY: case KP_POINTZ: {
			kp_dual d = dconst(pt[s->opcode - KP_POINTX]);
			d.g[s->opcode - KP_POINTX] = 1;
			return d;
		}
		case KP_NORMALX: case KP_NORMALY: case KP_NORMALZ: return dconst(0);
		case KP_ADD: return chain2(a, b, a.v + b.v, 1, 1);
		case KP_SUBTRACT: return chain2(a, b, a.v - b.v, 1, -1);
		case KP_MULTIPLY: return chain2(a, b, a.v * b.v, b.v, a.v);
		case KP_DIVIDE: return chain2(a, b, a.v / b.v, 1 / b.v, -a.v / (b.v * b.v));
		case KP_NEGATE: return chain1(a, -a.v, -1);
		case KP_SQRT: {
			const double f = sqrt(a.v);
			return chain1(a, f, f > 0 ? 0.5 / f : 0);
		}
		case KP_ABS: return a.v < 0 ? chain1(a, -a.v, -1) : a;
		case KP_FLOOR: return dconst(floor(a.v));
		case KP_SIN: return chain1(a, sin(a.v), cos(a.v));
		case KP_COS: return chain1(a, cos(a.v), -sin(a.v));
		case KP_SIGN: return dconst(sign_d(a.v));
		case KP_ATAN2: {
			const double rr = b.v * b.v + a.v * a.v;
			return chain2(a, b, atan2(a.v, b.v), b.v / rr, -a.v / rr);
		}
		case KP_POW: {
			const double f = pow(a.v, b.v);
			return chain2(a, b, f, b.v * pow(a.v, b.v - 1), f * (a.v > 0 ? log(a.v) : 0));
		}
		case KP_MIN: return a.v <= b.v ? a : b;
		case KP_MAX: return a.v >= b.v ? a : b;
		case KP_SMIN: {
			const kp_dual rr = r[s->c];
			const double fa = clampd((rr.v - (a.v - b.v)) / (2 * rr.v), 0.0, 1.0);
			return chain2(a, b, smooth_min(a.v, b.v, rr.v), fa, 1 - fa);
		}
		case KP_POSSQ: return chain1(a, pos_sq(a.v), 2 * dmax(a.v, 0.0));
		case KP_SELECT: return a.v != 0 ? b : r[s->c];
		default: return dconst(compare_d(s->opcode, a.v, b.v));
	}
}

kp_dual kp_eval_dual(const kp_program* p, const double pt[3], kp_dual* regs) {
	for (uint32_t i = 0; i < p->count; ++i) {
		regs[i] = step_dual(&p->steps[i], regs, pt);
	}
	return regs[p->result];
}

/* ---------------- source of a value (sdf/program.cpp:440-524) ---------------- */
static int is_join(int op) { return op == KP_MIN || op == KP_SMIN || op == KP_MAX || op == KP_NEGATE || op == KP_SELECT; }

static uint32_t chosen_operand(const kp_step* s, const double* v) {
	const double a = v[s->a], b = v[s->b];
	switch (s->opcode) {
		case KP_MIN: case KP_SMIN: return a <= b ? s->a : s->b;
		case KP_MAX: return a >= b ? s->a : s->b;
		case KP_SELECT: return a != 0 ? s->b : s->c;
		default: return s->a;
	}
}

static uint32_t leaf_from(const kp_program* p, const double* v, uint32_t at) {
	while (is_join(p->steps[at].opcode)) at = chosen_operand(&p->steps[at], v);
	return p->steps[at].leaf;
}

kp_source kp_source_of(const kp_program* p, const double* v) {
	kp_source src = { NO_LEAF, NO_LEAF, 0 };
	uint32_t at = p->result;
	while (is_join(p->steps[at].opcode)) {
		const kp_step* s = &p->steps[at];
		const uint32_t next = chosen_operand(s, v);
		double share = 0;
		if (s->opcode == KP_SMIN) {
			const double radius = v[s->c];
			const double apart = fabs(v[s->a] - v[s->b]);
			share = radius > 0 && apart < radius ? 0.5 * (radius - apart) / radius : 0;
		}
		if (share > 0 && src.other == NO_LEAF) {
			src.other = leaf_from(p, v, next == s->a ? s->b : s->a);
			src.share = share;
		}
		at = next;
	}
	src.leaf = p->steps[at].leaf;
	return src;
}

/* ---------------- the cut (plugins/geometry/tree/cut.cpp:80-400) ---------------- */
static int is_point(kp_interval a) { return a.lower == a.upper; }
static int is_literal(int op) { return op == KP_CONSTANT || op == KP_ARGUMENT; }
static int is_value(kp_interval a, double v) { return a.lower == v && a.upper == v; }

static uint32_t separated(const kp_step* s, const kp_interval* r, int lower_wins) {
	const kp_interval a = r[s->a], b = r[s->b];
	if (a.upper <= b.lower) return lower_wins ? s->a : s->b;
	if (b.upper <= a.lower) return lower_wins ? s->b : s->a;
	return NO_OPERAND;
}

static uint32_t outside_blend(const kp_step* s, const kp_interval* r) {
	const double radius = r[s->c].lower;
	const kp_interval d = iv(r[s->a].lower - r[s->b].upper, r[s->a].upper - r[s->b].lower);
	if (d.upper <= -radius) return s->a;
	if (d.lower >= radius) return s->b;
	return NO_OPERAND;
}

static uint32_t neutral_operand(const kp_step* s, const kp_interval* r, double neutral) {
	const int commutes = s->opcode == KP_ADD || s->opcode == KP_MULTIPLY;
	if (is_value(r[s->b], neutral)) return s->a;
	if (commutes && is_value(r[s->a], neutral)) return s->b;
	return NO_OPERAND;
}

static uint32_t shortcut(const kp_step* s, const kp_interval* r) {
	switch (s->opcode) {
		case KP_ADD: case KP_SUBTRACT: return neutral_operand(s, r, 0);
		case KP_MULTIPLY: case KP_DIVIDE: return neutral_operand(s, r, 1);
		case KP_MIN: return separated(s, r, 1);
		case KP_MAX: return separated(s, r, 0);
		case KP_SMIN: return outside_blend(s, r);
		case KP_ABS: return r[s->a].lower >= 0 ? s->a : NO_OPERAND;
		case KP_SELECT: {
			const kp_interval c = r[s->a];
			if (c.lower > 0 || c.upper < 0) return s->b;
			if (c.lower == 0 && c.upper == 0) return s->c;
			return NO_OPERAND;
		}
		default: return NO_OPERAND;
	}
}

static uint32_t negated_operand(const kp_step* s, const kp_interval* r) {
	const int product = s->opcode == KP_MULTIPLY;
	if (s->opcode == KP_ABS && r[s->a].upper <= 0) return s->a;
	if (s->opcode == KP_SUBTRACT && is_value(r[s->a], 0)) return s->b;
	if (product && is_value(r[s->a], -1)) return s->b;
	if (product && is_value(r[s->b], -1)) return s->a;
	return NO_OPERAND;
}

static kp_step resolved_step(kp_step s, const kp_interval* r, uint32_t index) {
	if (is_point(r[index]) && !is_literal(s.opcode)) {
		kp_step c = { KP_CONSTANT, 0, 0, 0, r[index].lower, s.leaf };
		return c;
	}
	if (s.opcode == KP_POSSQ && r[s.a].lower >= 0) {
		s.opcode = KP_MULTIPLY;
		s.b = s.a;
		return s;
	}
	const uint32_t neg = negated_operand(&s, r);
	if (neg != NO_OPERAND) {
		s.opcode = KP_NEGATE;
		s.a = neg;
		s.b = 0;
		s.c = 0;
	}
	return s;
}

static kp_step unsquared(const kp_step* steps, kp_step s) {
	if (s.opcode != KP_SQRT) return s;
	const kp_step inner = steps[s.a];
	if (inner.opcode == KP_POSSQ) {
		kp_step positive = inner;
		positive.opcode = KP_MAX;
		return positive;
	}
	if (inner.opcode != KP_MULTIPLY || inner.a != inner.b) return s;
	s.opcode = KP_ABS;
	s.a = inner.a;
	return s;
}

static int is_zero_step(const kp_step* steps, uint32_t i) { return steps[i].opcode == KP_CONSTANT && steps[i].value == 0; }

static kp_step positive_squared(const kp_step* steps, kp_step s) {
	if (s.opcode != KP_MULTIPLY || s.a != s.b) return s;
	const kp_step inner = steps[s.a];
	if (inner.opcode != KP_MAX || !(is_zero_step(steps, inner.a) || is_zero_step(steps, inner.b))) return s;
	const int zero_first = is_zero_step(steps, inner.a);
	s.opcode = KP_POSSQ;
	s.a = zero_first ? inner.b : inner.a;
	s.b = zero_first ? inner.a : inner.b;
	return s;
}

static kp_step aliased_operands(kp_step s, const uint32_t* alias) {
	const int n = operand_count(s.opcode);
	s.a = n > 0 ? alias[s.a] : s.a;
	s.b = n > 1 ? alias[s.b] : 0;
	s.c = n > 2 ? alias[s.c] : 0;
	return s;
}

/*
 * cutWith (cut.cpp:306): rewrite every step, then prunedCompact
 * (sdf/program.cpp:414).  out must hold p->count steps; returns the new count
 * and writes the new result.  *unchanged is set where the compacted program
 * is step for step the input (cut.cpp:438 sameProgram).
 */
static uint32_t cut_program(const kp_program* p, const kp_interval* r, kp_step* out, uint32_t* result, uint32_t* alias, uint32_t* live) {
	for (uint32_t i = 0; i < p->count; ++i) {
		const kp_step orig = p->steps[i];
		if (is_literal(orig.opcode)) {
			alias[i] = i;
			kp_step lit = orig;
			lit.b = 0;
			lit.c = 0;
			out[i] = lit;
			continue;
		}
		const kp_step s = positive_squared(out, unsquared(out, aliased_operands(orig, alias)));
		const uint32_t other = is_point(r[i]) ? NO_OPERAND : shortcut(&s, r);
		alias[i] = other != NO_OPERAND ? other : i;
		out[i] = resolved_step(s, r, i);
	}
	const uint32_t res = alias[p->result];
	/* liveSteps (program.cpp:357) */
	memset(live, 0, sizeof(uint32_t) * p->count);
	live[res] = 1;
	for (uint32_t i = p->count; i-- > 0;) {
		if (!live[i]) continue;
		const kp_step s = out[i];
		const int n = operand_count(s.opcode);
		const uint32_t ops[3] = { s.a, s.b, s.c };
		for (int k = 0; k < n; ++k) live[ops[k]] = 1;
	}
	uint32_t all = 1;
	for (uint32_t i = 0; i < p->count; ++i) all &= live[i] != 0;
	if (all) {
		*result = res;
		return p->count;
	}
	/* compactedProgram (program.cpp:379) */
	uint32_t kept = 0;
	for (uint32_t i = 0; i < p->count; ++i) {
		if (live[i]) {
			live[i] = kept;
			kp_step m = out[i];
			const int n = operand_count(m.opcode);
			m.a = n > 0 ? live[m.a] : m.a;
			m.b = n > 1 ? live[m.b] : 0;
			m.c = n > 2 ? live[m.c] : 0;
			out[kept++] = m;
		}
	}
	*result = live[res];
	return kept;
}

static int same_step(const kp_step* a, const kp_step* b) {
	return a->opcode == b->opcode && a->a == b->a && a->b == b->b && a->c == b->c && memcmp(&a->value, &b->value, sizeof(double)) == 0 && a->leaf == b->leaf;
}

/* ---------------- the cut octree ---------------- */
typedef struct cell_prog {
	uint32_t object;
	uint32_t result;
	uint32_t count;
	kp_step* steps; /* owned by the tree's arena list */
} cell_prog;

typedef struct cell_rec {
	uint32_t level, place[3], occupancy, nprog;
	cell_prog* progs;
} cell_rec;

struct kp_octree {
	double lower[3], size[3];
	int min_depth, max_depth;
	uint32_t split_steps;
	cell_rec* cells;
	uint64_t ncells, cap;
	/* every allocation, freed at the end */
	void** blocks;
	uint64_t nblocks, capblocks;
	/* scratch */
	kp_interval* ir;
	uint32_t* alias;
	uint32_t* live;
	kp_step* tmp;
	uint32_t scratch;
	/* leaf index: the cell index of each node's first child, for descent */
	int64_t* first_child;
};

static void* arena(kp_octree* t, size_t bytes) {
	if (t->nblocks == t->capblocks) {
		t->capblocks = t->capblocks ? t->capblocks * 2 : 1024;
		t->blocks = (void**) realloc(t->blocks, t->capblocks * sizeof(void*));
	}
	void* p = malloc(bytes ? bytes : 1);
	t->blocks[t->nblocks++] = p;
	return p;
}

static void ensure_scratch(kp_octree* t, uint32_t n) {
	if (n <= t->scratch) return;
	t->scratch = n;
	t->ir = (kp_interval*) realloc(t->ir, n * sizeof(kp_interval));
	t->alias = (uint32_t*) realloc(t->alias, n * sizeof(uint32_t));
	t->live = (uint32_t*) realloc(t->live, n * sizeof(uint32_t));
	t->tmp = (kp_step*) realloc(t->tmp, n * sizeof(kp_step));
}

static uint64_t push_cell(kp_octree* t) {
	if (t->ncells == t->cap) {
		t->cap = t->cap ? t->cap * 2 : 4096;
		t->cells = (cell_rec*) realloc(t->cells, t->cap * sizeof(cell_rec));
		t->first_child = (int64_t*) realloc(t->first_child, t->cap * sizeof(int64_t));
	}
	t->first_child[t->ncells] = -1;
	return t->ncells++;
}

/* cutCell (cut.cpp:463) of the parent's programs over one box. */
static void cut_cell(kp_octree* t, uint64_t ci, const cell_prog* parent, uint32_t n, const kp_interval box[3]) {
	cell_prog* kept = (cell_prog*) arena(t, sizeof(cell_prog) * (n ? n : 1));
	double* lower = (double*) malloc(sizeof(double) * (n ? n : 1));
	double* upper = (double*) malloc(sizeof(double) * (n ? n : 1));
	int* occ = (int*) malloc(sizeof(int) * (n ? n : 1));
	cell_prog* cand = (cell_prog*) malloc(sizeof(cell_prog) * (n ? n : 1));
	for (uint32_t i = 0; i < n; ++i) {
		const kp_program p = { parent[i].steps, parent[i].count, parent[i].result };
		ensure_scratch(t, p.count + 1);
		const kp_interval range = kp_eval_interval(&p, box, t->ir);
		lower[i] = range.lower;
		upper[i] = range.upper;
		occ[i] = range.lower > 0 ? KP_EMPTY : (range.upper < 0 ? KP_FILLED : KP_SURFACE);
		cand[i] = parent[i];
		if (occ[i] != KP_EMPTY) {
			uint32_t res = 0;
			const uint32_t count = cut_program(&p, t->ir, t->tmp, &res, t->alias, t->live);
			int same = count == p.count && res == p.result;
			for (uint32_t k = 0; same && k < count; ++k) same = same_step(&t->tmp[k], &p.steps[k]);
			if (!same) {
				kp_step* st = (kp_step*) arena(t, sizeof(kp_step) * count);
				memcpy(st, t->tmp, sizeof(kp_step) * count);
				cand[i].steps = st;
				cand[i].count = count;
				cand[i].result = res;
			}
		}
		if (occ[i] == KP_FILLED) {
			kept[0] = cand[i];
			t->cells[ci].occupancy = KP_FILLED;
			t->cells[ci].nprog = 1;
			t->cells[ci].progs = kept;
			free(lower);
			free(upper);
			free(occ);
			free(cand);
			return;
		}
	}
	double lowest = INFINITY;
	for (uint32_t i = 0; i < n; ++i) lowest = dmin(lowest, upper[i]);
	uint32_t m = 0;
	for (uint32_t i = 0; i < n; ++i) {
		if (occ[i] == KP_SURFACE && !(lower[i] > lowest)) kept[m++] = cand[i];
	}
	t->cells[ci].occupancy = m ? KP_SURFACE : KP_EMPTY;
	t->cells[ci].nprog = m;
	t->cells[ci].progs = kept;
	free(lower);
	free(upper);
	free(occ);
	free(cand);
}

static uint32_t cell_steps(const cell_rec* c) {
	uint32_t s = 0;
	for (uint32_t i = 0; i < c->nprog; ++i) s += c->progs[i].count;
	return s;
}

/* cut.cpp:512 halfSpan */
static kp_interval half_span(kp_interval s, int side) {
	const double middle = (s.lower + s.upper) / 2;
	return iv(side == 0 ? s.lower : middle, side == 0 ? middle : s.upper);
}

static void grow(kp_octree* t, uint64_t ci, const kp_interval box[3]) {
	cell_rec c = t->cells[ci];
	const int split = c.occupancy == KP_SURFACE && ((int) c.level < t->min_depth || ((int) c.level < t->max_depth && cell_steps(&c) > t->split_steps));
	if (!split) return;
	const uint64_t first = t->ncells;
	for (int o = 0; o < 8; ++o) push_cell(t);
	t->first_child[ci] = (int64_t) first;
	for (int o = 0; o < 8; ++o) {
		const uint64_t k = first + (uint64_t) o;
		t->cells[k].level = c.level + 1;
		t->cells[k].place[0] = c.place[0] * 2 + (uint32_t) (o & 1);
		t->cells[k].place[1] = c.place[1] * 2 + (uint32_t) ((o >> 1) & 1);
		t->cells[k].place[2] = c.place[2] * 2 + (uint32_t) ((o >> 2) & 1);
		kp_interval child[3] = { half_span(box[0], o & 1), half_span(box[1], (o >> 1) & 1), half_span(box[2], (o >> 2) & 1) };
		cut_cell(t, k, t->cells[ci].progs, t->cells[ci].nprog, child);
	}
	for (int o = 0; o < 8; ++o) {
		kp_interval child[3] = { half_span(box[0], o & 1), half_span(box[1], (o >> 1) & 1), half_span(box[2], (o >> 2) & 1) };
		grow(t, first + (uint64_t) o, child);
	}
}

kp_octree* kp_octree_build(const kp_program* programs, uint32_t count, const double lower[3], const double size[3], int min_depth, int max_depth, uint32_t split_steps) {
	kp_octree* t = (kp_octree*) calloc(1, sizeof(kp_octree));
	for (int a = 0; a < 3; ++a) {
		t->lower[a] = lower[a];
		t->size[a] = size[a];
	}
	t->min_depth = min_depth;
	t->max_depth = max_depth;
	t->split_steps = split_steps;
	cell_prog* root = (cell_prog*) arena(t, sizeof(cell_prog) * (count ? count : 1));
	for (uint32_t i = 0; i < count; ++i) {
		root[i].object = i;
		root[i].steps = (kp_step*) programs[i].steps;
		root[i].count = programs[i].count;
		root[i].result = programs[i].result;
	}
	/* the cells keep the object index of each program they were cut from */
	const uint64_t r = push_cell(t);
	t->cells[r].level = 0;
	t->cells[r].place[0] = t->cells[r].place[1] = t->cells[r].place[2] = 0;
	kp_interval box[3];
	for (int a = 0; a < 3; ++a) box[a] = iv(lower[a], lower[a] + size[a]);
	cut_cell(t, r, root, count, box);
	grow(t, r, box);
	return t;
}

void kp_octree_free(kp_octree* t) {
	if (!t) return;
	for (uint64_t i = 0; i < t->nblocks; ++i) free(t->blocks[i]);
	free(t->blocks);
	free(t->cells);
	free(t->first_child);
	free(t->ir);
	free(t->alias);
	free(t->live);
	free(t->tmp);
	free(t);
}

uint64_t kp_octree_cells(const kp_octree* t) { return t->ncells; }

/* The pre-order of the reference's recursive dump is the depth-first order;
 * the build above stores children breadth-first per parent, so the index
 * here is a depth-first walk computed on demand. */
static uint64_t dfs_index(const kp_octree* t, uint64_t node, uint64_t* counter, uint64_t want, int* found) {
	if (*counter == want) {
		*found = 1;
		return node;
	}
	*counter += 1;
	if (t->first_child[node] < 0) return 0;
	for (int o = 0; o < 8; ++o) {
		const uint64_t r = dfs_index(t, (uint64_t) t->first_child[node] + (uint64_t) o, counter, want, found);
		if (*found) return r;
	}
	return 0;
}

static const cell_rec* cell_at(const kp_octree* t, uint64_t i) {
	uint64_t counter = 0;
	int found = 0;
	const uint64_t n = dfs_index(t, 0, &counter, i, &found);
	return found ? &t->cells[n] : NULL;
}

uint32_t kp_octree_cell(const kp_octree* t, uint64_t i, uint32_t head[5]) {
	const cell_rec* c = cell_at(t, i);
	if (!c) return 0;
	head[0] = c->level;
	head[1] = c->place[0];
	head[2] = c->place[1];
	head[3] = c->place[2];
	head[4] = c->occupancy;
	return c->nprog;
}

void kp_octree_cell_program(const kp_octree* t, uint64_t i, uint32_t k, uint32_t* object, kp_program* program) {
	const cell_rec* c = cell_at(t, i);
	*object = c->progs[k].object;
	program->steps = c->progs[k].steps;
	program->count = c->progs[k].count;
	program->result = c->progs[k].result;
}

/* ---------------- sphere tracing (sphere_trace.cpp:21-227) ---------------- */
#define SPHERE_TOL 1e-6
#define SPHERE_STEPS (1 << 16)
#define SPHERE_INSET (2 * SPHERE_TOL)
#define SPHERE_TIE 1e-12
#define SPHERE_GRAZE 0.02
#define SPHERE_MIN_PART 1e-12

typedef struct field_src {
	/* evaluate the field's candidate programs at a point */
	const kp_octree* tree;
	const kp_program* programs;
	uint32_t count;
	double* regs;
	uint32_t nregs;
	kp_dual* dregs;
} field_src;

typedef struct cand_list {
	const kp_program* progs[4096];
	uint32_t objects[4096];
	uint32_t n;
	int empty;         /* the point is in an empty cell */
	double exit_t;     /* where the ray leaves that cell */
} cand_list;

static double slope_of(double part) {
	return 1 / (fabs(part) < SPHERE_MIN_PART ? copysign(SPHERE_MIN_PART, part) : part);
}

static void point_at(const kp_ray* ray, double t, double p[3]) {
	for (int a = 0; a < 3; ++a) p[a] = (double) ray->origin[a] + (double) ray->direction[a] * t;
}

/* Where the ray leaves an axis-aligned box, from t onward. */
static double box_exit(const kp_ray* ray, const double lo[3], const double hi[3]) {
	double upper = INFINITY;
	for (int a = 0; a < 3; ++a) {
		const double s = slope_of((double) ray->direction[a]);
		const double x = (lo[a] - (double) ray->origin[a]) * s;
		const double y = (hi[a] - (double) ray->origin[a]) * s;
		upper = dmin(upper, dmax(x, y));
	}
	return upper;
}

/* The kept programs of the leaf cell that holds a point. */
static void candidates(const kp_octree* tree, const kp_program* programs, uint32_t count, const kp_ray* ray, const double p[3], cand_list* out, kp_program* storage) {
	out->n = 0;
	out->empty = 0;
	out->exit_t = INFINITY;
	if (!tree) {
		for (uint32_t i = 0; i < count && i < 4096; ++i) {
			out->progs[out->n] = &programs[i];
			out->objects[out->n++] = i;
		}
		return;
	}
	uint64_t node = 0;
	double lo[3], hi[3];
	for (int a = 0; a < 3; ++a) {
		lo[a] = tree->lower[a];
		hi[a] = tree->lower[a] + tree->size[a];
	}
	while (tree->first_child[node] >= 0) {
		int o = 0;
		for (int a = 0; a < 3; ++a) {
			const double mid = (lo[a] + hi[a]) / 2;
			if (p[a] >= mid) {
				o |= 1 << a;
				lo[a] = mid;
			} else {
				hi[a] = mid;
			}
		}
		node = (uint64_t) tree->first_child[node] + (uint64_t) o;
	}
	const cell_rec* c = &tree->cells[node];
	/* A cell keeps only the objects whose surface may pass through it
	 * (cut.cpp:442 deciding), so past its walls its field is no distance
	 * bound: a step stops where the ray leaves the cell. */
	out->exit_t = box_exit(ray, lo, hi);
	if (c->occupancy == KP_EMPTY) {
		out->empty = 1;
		return;
	}
	for (uint32_t i = 0; i < c->nprog && i < 4096; ++i) {
		storage[i].steps = c->progs[i].steps;
		storage[i].count = c->progs[i].count;
		storage[i].result = c->progs[i].result;
		out->progs[out->n] = &storage[i];
		out->objects[out->n++] = c->progs[i].object;
	}
}

static int inside_region(const double lower[3], const double size[3], const double p[3]) {
	for (int a = 0; a < 3; ++a) {
		if (!(p[a] >= lower[a] && p[a] <= lower[a] + size[a])) return 0;
	}
	return 1;
}

typedef struct march {
	const kp_octree* tree;
	const kp_program* programs;
	uint32_t count;
	const uint32_t* leaf_material;
	const kp_ray* ray;
	double* regs;
	kp_dual* dregs;
	kp_program* storage;
	cand_list* cand;
	cand_list* cand2;
	int rule; /* stopping rule: 0 the reference's (SPHERE_TOL), 1 the device's (tolerance_at) */
} march;

/* The stopping tolerance at t: the reference's 1e-6 (sphere_trace.h:14
 * sphereTolerance), or, as a sensitivity check of the reference's own
 * answer, the FP32 device march's 2e-6 max(1, |p|_inf / 4). */
static double tolerance_at(const march* m, double t) {
	if (m->rule == 0) return SPHERE_TOL;
	const double p0 = fabs((double) m->ray->origin[0] + (double) m->ray->direction[0] * t);
	const double p1 = fabs((double) m->ray->origin[1] + (double) m->ray->direction[1] * t);
	const double p2 = fabs((double) m->ray->origin[2] + (double) m->ray->direction[2] * t);
	const double big = p0 > p1 ? (p0 > p2 ? p0 : p2) : (p1 > p2 ? p1 : p2);
	return 2e-6 * (big * 0.25 > 1.0 ? big * 0.25 : 1.0);
}

static void values_at(march* m, double t, cand_list* c, double* values) {
	double p[3];
	point_at(m->ray, t, p);
	candidates(m->tree, m->programs, m->count, m->ray, p, c, m->storage + (c == m->cand ? 0 : 4096));
	for (uint32_t i = 0; i < c->n; ++i) values[i] = kp_eval(c->progs[i], p, m->regs);
}

static uint32_t least_of(const double* v, uint32_t n) {
	uint32_t least = 0;
	for (uint32_t k = 0; k < n; ++k) least = v[k] < v[least] ? k : least;
	return least;
}

static void field_hit(march* m, double t, const kp_program* prog, uint32_t object, kp_hit* hit) {
	double p[3];
	point_at(m->ray, t, p);
	const kp_dual d = kp_eval_dual(prog, p, m->dregs);
	for (uint32_t i = 0; i < prog->count; ++i) m->regs[i] = m->dregs[i].v;
	const kp_source src = kp_source_of(prog, m->regs);
	/* sphereNormal (sphere_trace.cpp:140) */
	double n[3];
	const double len = sqrt(d.g[0] * d.g[0] + d.g[1] * d.g[1] + d.g[2] * d.g[2]);
	const double dir[3] = { m->ray->direction[0], m->ray->direction[1], m->ray->direction[2] };
	if (!(len > 0)) {
		for (int a = 0; a < 3; ++a) n[a] = -dir[a];
	} else {
		for (int a = 0; a < 3; ++a) n[a] = d.g[a] / len;
		const double along = n[0] * dir[0] + n[1] * dir[1] + n[2] * dir[2];
		if (m->ray->inside) {
			if (along < 0) for (int a = 0; a < 3; ++a) n[a] = -n[a];
		} else if (along > 0) {
			double g[3];
			for (int a = 0; a < 3; ++a) g[a] = n[a] - dir[a] * (along + SPHERE_GRAZE);
			const double gl = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
			for (int a = 0; a < 3; ++a) n[a] = g[a] / gl;
		}
	}
	hit->kind = 1;
	hit->distance = (float) t;
	for (int a = 0; a < 3; ++a) {
		hit->point[a] = (float) p[a];
		hit->normal[a] = (float) n[a];
	}
	hit->leaf = src.leaf;
	hit->other = src.other;
	hit->share = (float) src.share;
	hit->object = object;
}

static void landed(march* m, const double* values, uint32_t n, double t, kp_hit* hit) {
	/* sphereWinner (sphere_trace.cpp:96): the tie goes to the least value a
	 * little further along. */
	double p[3];
	point_at(m->ray, t, p);
	const double big = dmax(fabs(p[0]), dmax(fabs(p[1]), fabs(p[2])));
	const double band = SPHERE_TIE * (1 + big);
	const uint32_t first = least_of(values, n);
	uint32_t winner = first;
	int tied = 0;
	for (uint32_t k = 0; k < n; ++k) tied |= k != first && values[k] - values[first] <= band;
	if (tied) {
		double q[3];
		point_at(m->ray, t + 2 * tolerance_at(m, t), q);
		double on[4096];
		for (uint32_t k = 0; k < n; ++k) on[k] = kp_eval(m->cand->progs[k], q, m->regs);
		for (uint32_t k = 0; k < n; ++k) winner = values[k] - values[first] <= band && on[k] < on[winner] ? k : winner;
	}
	field_hit(m, t, m->cand->progs[winner], m->cand->objects[winner], hit);
}

static void missed(kp_hit* hit) {
	memset(hit, 0, sizeof(*hit));
	hit->leaf = NO_LEAF;
	hit->other = NO_LEAF;
	hit->object = NO_LEAF;
}

static void trace_one(march* m, const double lower[3], const double size[3], kp_hit* hit) {
	const kp_ray* ray = m->ray;
	double lo = 0, up = (double) ray->far;
	for (int a = 0; a < 3; ++a) {
		const double s = slope_of((double) ray->direction[a]);
		const double x = (lower[a] - (double) ray->origin[a]) * s;
		const double y = (lower[a] + size[a] - (double) ray->origin[a]) * s;
		lo = dmax(lo, dmin(x, y));
		up = dmin(up, dmax(x, y));
	}
	missed(hit);
	if (up < lo) return;
	double values[4096];
	double t = lo;
	for (int step = 0; step < SPHERE_STEPS && t <= up; ++step) {
		values_at(m, t, m->cand, values);
		hit->steps = (uint32_t) step + 1;
		const double tol = tolerance_at(m, t), inset = 2 * tol;
		/* an empty cell, or from inside a body one it fills (no surface
		 * passes through it: the full field's steps would cross it whole) */
		if (m->cand->empty || (ray->inside && m->cand->n == 0)) {
			t = dmax(m->cand->exit_t, t) + SPHERE_TOL;
			continue;
		}
		if (m->cand->n == 0) return;
		if (!ray->inside) {
			const double least = values[least_of(values, m->cand->n)];
			if (least < tol) {
				landed(m, values, m->cand->n, t, hit);
				return;
			}
			t = dmin(t + least, dmax(m->cand->exit_t, t) + SPHERE_TOL);
			continue;
		}
		/* sphereFromInside (sphere_trace.cpp:188) */
		double nearest = fabs(values[0]);
		for (uint32_t k = 0; k < m->cand->n; ++k) nearest = dmin(nearest, fabs(values[k]));
		if (nearest < tol) {
			double past[4096];
			values_at(m, t + inset, m->cand2, past);
			const int past_empty = m->cand2->empty || m->cand2->n == 0;
			const uint32_t least = past_empty ? 0 : least_of(past, m->cand2->n);
			if (past_empty || past[least] > 0) {
				values_at(m, t, m->cand, values);
				landed(m, values, m->cand->n, t, hit);
				return;
			}
			kp_hit there;
			field_hit(m, t + inset, m->cand2->progs[least], m->cand2->objects[least], &there);
			if (there.leaf != NO_LEAF && m->leaf_material && m->leaf_material[there.leaf] != ray->within) {
				double p[3];
				point_at(ray, t, p);
				there.distance = (float) t;
				for (int a = 0; a < 3; ++a) there.point[a] = (float) p[a];
				there.steps = hit->steps;
				*hit = there;
				return;
			}
		}
		t = nearest < tol ? t + inset : dmin(t + nearest, dmax(m->cand->exit_t, t) + SPHERE_TOL);
	}
	missed(hit);
}

static void trace_all(const kp_octree* tree, const kp_program* programs, uint32_t count, const uint32_t* leaf_material, const double lower[3], const double size[3], const kp_ray* rays, uint32_t n, kp_hit* hits, int rule) {
	uint32_t longest = 1;
	if (tree) {
		for (uint64_t i = 0; i < tree->ncells; ++i)
			for (uint32_t k = 0; k < tree->cells[i].nprog; ++k) longest = tree->cells[i].progs[k].count > longest ? tree->cells[i].progs[k].count : longest;
	} else {
		for (uint32_t i = 0; i < count; ++i) longest = programs[i].count > longest ? programs[i].count : longest;
	}
	march m;
	m.tree = tree;
	m.programs = programs;
	m.count = count;
	m.leaf_material = leaf_material;
	m.regs = (double*) malloc(sizeof(double) * longest);
	m.dregs = (kp_dual*) malloc(sizeof(kp_dual) * longest);
	m.storage = (kp_program*) malloc(sizeof(kp_program) * 8192);
	m.cand = (cand_list*) malloc(sizeof(cand_list));
	m.cand2 = (cand_list*) malloc(sizeof(cand_list));
	m.rule = rule;
	for (uint32_t i = 0; i < n; ++i) {
		m.ray = &rays[i];
		trace_one(&m, lower, size, &hits[i]);
	}
	free(m.regs);
	free(m.dregs);
	free(m.storage);
	free(m.cand);
	free(m.cand2);
}

/* A reusable single-ray tracer over an octree, one per thread. */
struct kp_tracer {
	march m;
	const kp_octree* tree;
};

kp_tracer* kp_tracer_new(const kp_octree* tree, const uint32_t* leaf_material) {
	kp_tracer* t = (kp_tracer*) calloc(1, sizeof(kp_tracer));
	uint32_t longest = 1;
	for (uint64_t i = 0; i < tree->ncells; ++i)
		for (uint32_t k = 0; k < tree->cells[i].nprog; ++k) longest = tree->cells[i].progs[k].count > longest ? tree->cells[i].progs[k].count : longest;
	t->tree = tree;
	t->m.tree = tree;
	t->m.programs = NULL;
	t->m.count = 0;
	t->m.leaf_material = leaf_material;
	t->m.regs = (double*) malloc(sizeof(double) * longest);
	t->m.dregs = (kp_dual*) malloc(sizeof(kp_dual) * longest);
	t->m.storage = (kp_program*) malloc(sizeof(kp_program) * 8192);
	t->m.cand = (cand_list*) malloc(sizeof(cand_list));
	t->m.cand2 = (cand_list*) malloc(sizeof(cand_list));
	return t;
}

void kp_tracer_trace(kp_tracer* t, const kp_ray* ray, kp_hit* hit) {
	t->m.ray = ray;
	trace_one(&t->m, t->tree->lower, t->tree->size, hit);
}

void kp_tracer_free(kp_tracer* t) {
	if (!t) return;
	free(t->m.regs);
	free(t->m.dregs);
	free(t->m.storage);
	free(t->m.cand);
	free(t->m.cand2);
	free(t);
}

void kp_sphere_trace(const kp_program* programs, uint32_t count, const uint32_t* leaf_material, const double lower[3], const double size[3], const kp_ray* rays, uint32_t n, kp_hit* hits) {
	trace_all(NULL, programs, count, leaf_material, lower, size, rays, n, hits, 0);
}

void kp_sphere_trace_rule(const kp_program* programs, uint32_t count, const uint32_t* leaf_material, const double lower[3], const double size[3], const kp_ray* rays, uint32_t n, kp_hit* hits, int rule) {
	trace_all(NULL, programs, count, leaf_material, lower, size, rays, n, hits, rule);
}

void kp_normal_at(const kp_program* program, const kp_ray* ray, double t, double normal[3], double* gradient_length) {
	kp_dual* dregs = (kp_dual*) malloc(sizeof(kp_dual) * (program->count ? program->count : 1));
	double* regs   = (double*) malloc(sizeof(double) * (program->count ? program->count : 1));
	march m;
	memset(&m, 0, sizeof m);
	m.ray   = ray;
	m.regs  = regs;
	m.dregs = dregs;
	kp_hit hit;
	field_hit(&m, t, program, 0, &hit);
	double p[3];
	point_at(ray, t, p);
	const kp_dual d = kp_eval_dual(program, p, dregs);
	*gradient_length = sqrt(d.g[0] * d.g[0] + d.g[1] * d.g[1] + d.g[2] * d.g[2]);
	for (int a = 0; a < 3; ++a) normal[a] = hit.normal[a];
	free(dregs);
	free(regs);
}

void kp_octree_trace(const kp_octree* tree, const uint32_t* leaf_material, const kp_ray* rays, uint32_t n, kp_hit* hits) {
	trace_all(tree, NULL, 0, leaf_material, tree->lower, tree->size, rays, n, hits, 0);
}
