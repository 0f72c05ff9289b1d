/* Host harness around the library's VA13 state machine (va13.cuh): the same
 * extended-Rosenbrock trace as the oracle's orc_minfor_trace, for an exact
 * comparison of the two implementations, and traces of the machine's warp
 * form (provide_w, run here with the serial executor, which takes the
 * elements of each section in descending order) on several objectives. */
#include <cmath>
#include <cstddef>
#include "../../gpuattract_2.0_gb300/csrc/va13.cuh"
#include "va13_objectives.h"

namespace {

/* kinds 0, 1, 4, 5: va13_objectives.h (the same bits on the device); 2: log
 * wells under a sine of the coordinate sum (nonconvex); 3: a gradient that
 * is not the objective's, through sin and cos */
double objective(int kind, int n, const double* s, double* g) {
	if (va13_exact_kind(kind)) return va13_exact_objective(kind, n, s, g);
	double f = 0.0;
	for (int i = 0; i < n; ++i) g[i] = 0.0;
	if (kind == 2) {
		double sum = 0.0;
		for (int i = 0; i < n; ++i) sum = sum + s[i];
		for (int i = 0; i < n; ++i) {
			const double a = i + 1.0, e = s[i] - 0.5, den = 1.0 + a * e * e;
			f = f + std::log(den);
			g[i] = 2.0 * a * e / den + 0.3 * std::cos(sum);
		}
		f = f + 0.3 * std::sin(sum);
	} else {
		for (int i = 0; i < n; ++i) {
			f = f + s[i] * std::sin(3.0 * s[i]);
			g[i] = std::cos(2.0 * s[i]) + 0.1 * (i + 1);
		}
	}
	return f;
}

template <int NMAX, bool WARP>
int trace(int n, const double* x0, int ivmax, double* out, int cap, int nan_eval, int kind) {
	gba::VA13<NMAX> va;
	va.start(x0, n, ivmax);
	int k = 0;
	double g[NMAX];
	while (!va.done()) {
		const double* s = va.point();   /* 0-based */
		const double f = objective(kind, n, s, g);
		if (k == nan_eval) g[0] = std::nan("");
		if (k < cap) {
			for (int i = 0; i < n; ++i) out[(size_t)k * (n + 1) + i] = s[i];
			out[(size_t)k * (n + 1) + n] = f;
		}
		++k;
		if constexpr (WARP) va.provide_w(f, [&](int j) { return g[j - 1]; }, gba::VaSerial{});
		else va.provide(f, g);
	}
	return k < cap ? k : cap;
}

}  // namespace

extern "C" int va13_trace_nan(int n, const double* x0, int ivmax, double* trace, int cap, int nan_eval);

extern "C" int va13_trace(int n, const double* x0, int ivmax, double* trace, int cap) {
	return va13_trace_nan(n, x0, ivmax, trace, cap, -1);
}

/* evaluation nan_eval (0-based; -1: none) hands the machine a NaN gradient
 * component, as an overflowing energy does */
extern "C" int va13_trace_nan(int n, const double* x0, int ivmax, double* out, int cap, int nan_eval) {
	if (n < 1 || n > 32) return -1;
	return trace<32, false>(n, x0, ivmax, out, cap, nan_eval, 0);
}

/* either form on objective `kind` (warp != 0: provide_w) */
extern "C" int va13_trace_form(int n, const double* x0, int ivmax, double* out, int cap, int nan_eval, int kind,
		int warp) {
	if (n < 1 || n > 31 || kind < 0 || kind > 5) return -1;
	return warp ? trace<31, true>(n, x0, ivmax, out, cap, nan_eval, kind)
	            : trace<31, false>(n, x0, ivmax, out, cap, nan_eval, kind);
}

/* mc11a and mc11e against their warp forms on arbitrary inputs (every path
 * of mc11a, including those minfor never takes): out_* receive the packed
 * factors (n (n + 1) / 2 entries), z and w (n each) and ir.  alias != 0
 * passes z as w, as minfor's second update does; solve != 0 runs mc11e on
 * the factors instead of mc11a. */
extern "C" int va13_update_forms(int n, const double* a0, const double* z0, const double* w0, double sig, int ir0,
		int mk, double eps, int alias, int solve, double* out_seq, double* out_warp) {
	if (n < 1 || n > 31) return -1;
	const int na = n * (n + 1) / 2;
	for (int form = 0; form < 2; ++form) {
		double a[31 * 32 / 2 + 1], z[32], w[32], q[32], t[32];
		for (int k = 0; k < na; ++k) a[k + 1] = a0[k];
		for (int k = 0; k < n; ++k) {
			z[k + 1] = z0[k];
			w[k + 1] = w0[k];
		}
		double* wp = alias ? z : w;
		int ir = ir0;
		if (solve) {
			if (form == 0) gba::mc11e(a, n, z, wp, ir);
			else gba::mc11e_w(a, n, z, wp, ir, q, t, gba::VaSerial{});
		} else {
			if (form == 0) gba::mc11a(a, n, z, sig, wp, ir, mk, eps);
			else gba::mc11a_w(a, n, z, sig, wp, ir, mk, eps, q, t, gba::VaSerial{});
		}
		double* out = form == 0 ? out_seq : out_warp;
		for (int k = 0; k < na; ++k) out[k] = a[k + 1];
		for (int k = 0; k < n; ++k) {
			out[na + k] = z[k + 1];
			out[na + n + k] = wp[k + 1];
		}
		out[na + 2 * n] = ir;
	}
	return 0;
}
