/* Host harness around the library's VA13 state machine (va13.cuh): the same
 * extended-Rosenbrock trace as the oracle's orc_minfor_trace, for an exact
 * comparison of the two implementations. */
#include <cmath>
#include <cstddef>
#include "../../gpuattract_2.0_gb300/csrc/va13.cuh"

extern "C" int va13_trace_nan(int n, const double* x0, int ivmax, double* trace, int cap, int nan_eval);

extern "C" int va13_trace(int n, const double* x0, int ivmax, double* trace, int cap) {
	return va13_trace_nan(n, x0, ivmax, trace, cap, -1);
}

/* evaluation nan_eval (0-based; -1: none) hands the machine a NaN gradient
 * component, as an overflowing energy does */
extern "C" int va13_trace_nan(int n, const double* x0, int ivmax, double* trace, int cap, int nan_eval) {
	if (n < 1 || n > 32) return -1;
	gba::VA13<32> va;
	va.start(x0, n, ivmax);
	int k = 0;
	double g[32];
	while (!va.done()) {
		const double* s = va.point();   /* 0-based */
		double f = 0.0;
		for (int i = 0; i < n; ++i) g[i] = 0.0;
		for (int i = 0; i < n - 1; ++i) {
			const double a = s[i + 1] - s[i] * s[i], b = 1.0 - s[i];
			f = f + 100.0 * a * a + b * b;
			g[i] = g[i] - 400.0 * s[i] * a - 2.0 * b;
			g[i + 1] = g[i + 1] + 200.0 * a;
		}
		if (k == nan_eval) g[0] = std::nan("");
		if (k < cap) {
			for (int i = 0; i < n; ++i) trace[(size_t)k * (n + 1) + i] = s[i];
			trace[(size_t)k * (n + 1) + n] = f;
		}
		++k;
		va.provide(f, g);
	}
	return k < cap ? k : cap;
}
