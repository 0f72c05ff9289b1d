/* Test objectives for the VA13 machine that evaluate to the same bits on the
 * host and on the device: every product through gba::vm (never contracted
 * into a fused multiply-add), sums in a fixed order, IEEE divisions, no
 * transcendental functions.  s: the point (0-based, n entries); g receives
 * the gradient; returns f.
 *   kind 0: extended Rosenbrock (the oracle's orc_minfor_trace objective)
 *   kind 1: coupled double wells
 *   kind 4: rational wells with a weak chain coupling (nonconvex)
 *   kind 5: a gradient that is not the objective's (drives the machine's
 *           failure branches) */
#ifndef GBA_TEST_VA13_OBJECTIVES_H_
#define GBA_TEST_VA13_OBJECTIVES_H_

#include "../../gpuattract_2.0_gb300/csrc/va13.cuh"

GBA_HD bool va13_exact_kind(int kind) { return kind == 0 || kind == 1 || kind == 4 || kind == 5; }

GBA_HD double va13_exact_objective(int kind, int n, const double* s, double* g) {
	using gba::vm;
	double f = 0.0;
	for (int i = 0; i < n; ++i) g[i] = 0.0;
	if (kind == 0) {
		for (int i = 0; i < n - 1; ++i) {
			const double a = s[i + 1] - vm(s[i], s[i]), b = 1.0 - s[i];
			f = f + vm(vm(100.0, a), a) + vm(b, b);
			g[i] = g[i] - vm(vm(400.0, s[i]), a) - vm(2.0, b);
			g[i + 1] = g[i + 1] + vm(200.0, a);
		}
	} else if (kind == 1) {
		for (int i = 0; i < n; ++i) {
			const double a = i + 1.0, u = vm(s[i], s[i]) - 1.0, nx = s[(i + 1) % n];
			f = f + vm(vm(a, u), u) + vm(s[i], nx);
			g[i] = g[i] + vm(vm(vm(4.0, a), s[i]), u) + nx;
			g[(i + 1) % n] = g[(i + 1) % n] + s[i];
		}
	} else if (kind == 4) {
		for (int i = 0; i < n; ++i) {
			const double a = i + 1.0, e = s[i] - 0.5, den = 1.0 + vm(e, e);
			f = f + vm(a, vm(e, e)) / den;
			g[i] = g[i] + vm(vm(2.0, a), e) / vm(den, den);
			if (i + 1 < n) {
				f = f - vm(0.05, vm(s[i], s[i + 1]));
				g[i] = g[i] - vm(0.05, s[i + 1]);
				g[i + 1] = g[i + 1] - vm(0.05, s[i]);
			}
		}
	} else {
		for (int i = 0; i < n; ++i) {
			f = f + vm(vm(s[i], s[i]), s[i]) - s[i];
			g[i] = 1.0 - vm(2.0, vm(s[i], s[i])) + vm(0.1, i + 1.0);
		}
	}
	return f;
}

#endif
