/*
 * va13.cuh -- the VA13 variable-metric minimizer as a resumable state machine.
 *
 * Follows the Harwell routine the reference runs for every pose
 * (src/apps/em/minfor.f:1-182 with mc11a/mc11e, src/apps/em/mc11a.f:1-143),
 * in FP64 like the Fortran's real*8, generalised from its fixed 6 DOF to n DOF.
 * Instead of calling the energy function, the machine stops whenever minfor
 * would call it: `point()` is the DOF vector to evaluate, `provide(f, g)` hands
 * back the objective and gradient and runs to the next evaluation (or to the
 * end).  The same code runs on the host (plain per-step driver) and inside the
 * persistent device kernel.  Arrays are 1-based, mirroring the Fortran.
 */
#ifndef GBA_VA13_CUH_
#define GBA_VA13_CUH_

#include <cmath>

#ifdef __CUDACC__
#define GBA_HD __host__ __device__ __forceinline__
#else
#define GBA_HD inline
#endif

/* Device loops of the machine stay rolled: lane 0 runs it between two
 * evaluations of the whole warp, and unrolled copies of its loops evicted the
 * evaluation's code from the instruction cache (measured: instruction-fetch
 * stalls; the minimizers ran 7-9 % slower unrolled). */
#ifdef __CUDA_ARCH__
#define GBA_VA_LOOP _Pragma("unroll 1")
#else
#define GBA_VA_LOOP
#endif

namespace gba {

/* max, min and abs with the C++ library's semantics (std::max(a, b) =
 * a < b ? b : a, std::min(a, b) = b < a ? b : a, fabs clears the sign bit),
 * which decide what a NaN or a signed zero does: a pose whose energy
 * overflows hands the machine NaN gradients, and every form of the
 * minimizer must take the same branch on them. */
GBA_HD double va_max(double a, double b) { return a < b ? b : a; }
GBA_HD double va_min(double a, double b) { return b < a ? b : a; }
GBA_HD double va_abs(double a) { return fabs(a); }

/* Products are never contracted with a following add: the host build runs
 * with -ffp-contract=off and the device uses round-to-nearest multiplies, so
 * both sides take bit-identical steps (nvcc would otherwise form FMAs). */
GBA_HD double vm(double a, double b) {
#ifdef __CUDA_ARCH__
	return __dmul_rn(a, b);
#else
	return a * b;
#endif
}

/* mc11a: rank-one update of the packed LDL^T factors (mc11a.f:1-112). */
GBA_HD void mc11a(double* a, int n, double* z, double sig, double* w, int& ir, int mk, double eps) {
	double ti = 0, v, tim, b, r, y, gm, al;
	int np, ij = 1, ip, mm, j;
	if (n > 1) goto L1;
	a[1] = a[1] + vm(vm(sig, z[1]), z[1]);
	ir = 1;
	if (a[1] > 0.0) return;
	a[1] = 0.0;
	ir = 0;
	return;
L1:
	np = n + 1;
	if (sig > 0.0) goto L40;
	if (sig == 0.0 || ir == 0) return;
	ti = 1.0 / sig;
	ij = 1;
	if (mk == 0) goto L10;
	GBA_VA_LOOP
	for (int i = 1; i <= n; ++i) {
		if (a[ij] != 0.0) ti = ti + vm(w[i], w[i]) / a[ij];
		ij = ij + np - i;
	}
	goto L20;
L10:
	GBA_VA_LOOP
	for (int i = 1; i <= n; ++i) w[i] = z[i];
	GBA_VA_LOOP
	for (int i = 1; i <= n; ++i) {
		ip = i + 1;
		v = w[i];
		if (a[ij] > 0.0) {
			ti = ti + vm(v, v) / a[ij];
			if (i != n)
				for (j = ip; j <= n; ++j) {
					ij = ij + 1;
					w[j] = w[j] - vm(v, a[ij]);
				}
			ij = ij + 1;
		} else {
			w[i] = 0.0;
			ij = ij + np - i;
		}
	}
L20:
	if (ir <= 0) {
		ti = 0.;
		ir = -ir - 1;
		goto L23;
	}
	if (ti > 0.0) {
		ti = eps / sig;
		if (eps == 0.0) ir = ir - 1;
		goto L23;
	}
	if (mk - 1 <= 0) goto L40;
L23:
	mm = 1;
	tim = ti;
	GBA_VA_LOOP
	for (int i = 1; i <= n; ++i) {
		j = np - i;
		ij = ij - i;
		if (a[ij] != 0.0) tim = ti - vm(w[j], w[j]) / a[ij];
		w[j] = ti;
		ti = tim;
	}
	goto L41;
L40:
	mm = 0;
	tim = 1.0 / sig;
L41:
	ij = 1;
	GBA_VA_LOOP
	for (int i = 1; i <= n; ++i) {
		ip = i + 1;
		v = z[i];
		if (!(a[ij] > 0.0)) {
			if (ir > 0 || sig < 0.0 || v == 0.0) {
				ti = tim;
				ij = ij + np - i;
				continue;
			}
			ir = 1 - ir;
			a[ij] = vm(v, v) / tim;
			if (i == n) return;
			GBA_VA_LOOP
			for (j = ip; j <= n; ++j) {
				ij = ij + 1;
				a[ij] = z[j] / v;
			}
			return;
		}
		al = v / a[ij];
		if (mm <= 0) ti = tim + vm(v, al);
		else ti = w[i];
		r = ti / tim;
		a[ij] = vm(a[ij], r);
		if (r == 0.0) break;
		if (i == n) break;
		b = al / ti;
		if (r > 4.0) {
			gm = tim / ti;
			GBA_VA_LOOP
			for (j = ip; j <= n; ++j) {
				ij = ij + 1;
				y = a[ij];
				a[ij] = vm(b, z[j]) + vm(y, gm);
				z[j] = z[j] - vm(v, y);
			}
		} else {
			GBA_VA_LOOP
			for (j = ip; j <= n; ++j) {
				ij = ij + 1;
				z[j] = z[j] - vm(v, a[ij]);
				a[ij] = a[ij] + vm(b, z[j]);
			}
		}
		tim = ti;
		ij = ij + 1;
	}
	if (ir < 0) ir = -ir;
}

/* mc11e: solves with the packed factors (entry mc11e, mc11a.f:114-142). */
GBA_HD void mc11e(const double* a, int n, double* z, double* w, int ir) {
	if (ir < n) return;
	w[1] = z[1];
	if (n <= 1) {
		z[1] = z[1] / a[1];
		return;
	}
	int ij = 0;
	GBA_VA_LOOP
	for (int i = 2; i <= n; ++i) {
		ij = i;
		double v = z[i];
		GBA_VA_LOOP
		for (int j = 1; j <= i - 1; ++j) {
			v = v - vm(a[ij], z[j]);
			ij = ij + n - j;
		}
		w[i] = v;
		z[i] = v;
	}
	z[n] = z[n] / a[ij];
	const int np = n + 1;
	GBA_VA_LOOP
	for (int nip = 2; nip <= n; ++nip) {
		const int i = np - nip;
		int ii = ij - nip;
		double v = z[i] / a[ii];
		ij = ii;
		GBA_VA_LOOP
		for (int j = i + 1; j <= n; ++j) {
			ii = ii + 1;
			v = v - vm(a[ii], z[j]);
		}
		z[i] = v;
	}
}

/* minfor (minfor.f:1-182) as a machine stopped at each energy call. */
template <int NMAX>
struct VA13 {
	enum Phase { kInit = 0, kAfterFirst = 1, kAfterLine = 2, kDone = 3 };
	int phase, jn, ivmax, nfun, itr, isfv, ir;
	double gesa, c, acc, dff, dgb, fa, fb, fmin, gmin, dga;
	double step, stepbd, steplb, stmin;
	double h[NMAX * (NMAX + 1) / 2 + 1];
	double x[NMAX + 1], g[NMAX + 1], ga[NMAX + 1], gb[NMAX + 1], w[NMAX + 1];
	double xaa[NMAX + 1], xbb[NMAX + 1], d[NMAX + 1];

	/* minfor.f:31-61 up to the first energy call */
	GBA_HD void start(const double* x0, int n, int max_eval) {
		jn = n;
		ivmax = max_eval;
		const double xnull = 0.0;
		dga = xnull;
		GBA_VA_LOOP
		for (int i = 1; i <= jn; ++i) {
			x[i] = x0[i - 1];
			ga[i] = xnull;
			d[i] = xnull;
			xaa[i] = x[i];
		}
		nfun = 0;
		itr = 0;
		const int np = jn + 1;
		acc = 0.000000001;
		c = 1.0;
		int k = (jn * np) / 2;
		GBA_VA_LOOP
		for (int i = 1; i <= k; ++i) h[i] = xnull;
		k = 1;
		GBA_VA_LOOP
		for (int i = 1; i <= jn; ++i) {
			h[k] = vm(0.01, c);
			k = k + np - i;
		}
		dff = xnull;
		phase = kAfterFirst;
	}

	GBA_HD bool done() const { return phase == kDone; }

	/* The DOF vector (0-based view) minfor evaluates next. */
	GBA_HD const double* point() const { return phase == kAfterFirst ? xaa + 1 : xbb + 1; }

	/* Hands back f and grad (0-based) at point(); runs to the next call. */
	GBA_HD void provide(double f, const double* grad) {
		const double xnull = 0.0;
		int i;
		if (phase == kAfterFirst) {
			gesa = f;
			GBA_VA_LOOP
			for (i = 1; i <= jn; ++i) g[i] = grad[i - 1];
			goto L110;
		}
		if (phase != kAfterLine) return;
		fb = f;
		GBA_VA_LOOP
		for (i = 1; i <= jn; ++i) gb[i] = grad[i - 1];
		/* minfor.f:114-144 */
		isfv = isfv < 2 ? isfv : 2;
		if (fb > gesa) goto L220;
		if (fb < gesa) goto L200;
		{
			double gl1 = xnull, gl2 = xnull;
			GBA_VA_LOOP
			for (i = 1; i <= jn; ++i) {
				gl1 = gl1 + vm(g[i], g[i]);
				gl2 = gl2 + vm(gb[i], gb[i]);
			}
			if (gl2 >= gl1) goto L220;
		}
	L200:
		isfv = 3;
		gesa = fb;
		GBA_VA_LOOP
		for (i = 1; i <= jn; ++i) {
			x[i] = xbb[i];
			g[i] = gb[i];
		}
	L220:
		dgb = xnull;
		GBA_VA_LOOP
		for (i = 1; i <= jn; ++i) dgb = dgb + vm(gb[i], d[i]);
		if (fb - fa <= vm(vm(0.1, c), dga)) goto L280;
		if (step > steplb) goto L270;
	L240:
		if (isfv >= 2) goto L110;
		phase = kDone;
		return;
	L270:
		stepbd = step;
		c = gmin + dgb - vm(3.0, fb - fmin) / step;
		c = gmin / (c + gmin - sqrt(vm(c, c) - vm(gmin, dgb)));
		step = vm(step, va_max(0.1, c));
		goto L170;
	L280:
		stepbd = stepbd - step;
		stmin = c;
		fmin = fb;
		gmin = dgb;
		step = vm(9.0, stmin);
		if (stepbd > xnull) step = vm(0.5, stepbd);
		c = dga + vm(3.0, dgb) - vm(4.0, fb - fa) / stmin;
		if (c > xnull) step = va_min(step, vm(stmin, va_max(1.0, -dgb / c)));
		if (dgb < vm(0.7, dga)) goto L170;
		isfv = 4 - isfv;
		if (stmin + step <= steplb) goto L240;
		ir = -jn;
		GBA_VA_LOOP
		for (i = 1; i <= jn; ++i) {
			xaa[i] = xbb[i];
			xbb[i] = ga[i];
			d[i] = gb[i] - ga[i];
			ga[i] = gb[i];
		}
		mc11a(h, jn, xbb, 1.0 / dga, w, ir, 1, xnull);
		ir = -ir;
		mc11a(h, jn, d, 1.0 / vm(stmin, dgb - dga), d, ir, 0, xnull);
		if (ir < jn) {
			phase = kDone;
			return;
		}
		dff = fa - fb;
		fa = fb;
		goto L135;
	L110:
		fa = gesa;
		isfv = 1;
		GBA_VA_LOOP
		for (i = 1; i <= jn; ++i) ga[i] = g[i];
	L135:
		itr = itr + 1;
		GBA_VA_LOOP
		for (i = 1; i <= jn; ++i) d[i] = -ga[i];
		mc11e(h, jn, d, w, jn);
		c = xnull;
		dga = xnull;
		GBA_VA_LOOP
		for (i = 1; i <= jn; ++i) {
			c = va_max(c, va_abs(d[i]));
			dga = dga + vm(ga[i], d[i]);
		}
		if (dga >= xnull) goto L240;
		stmin = xnull;
		stepbd = xnull;
		steplb = acc / c;
		fmin = fa;
		gmin = dga;
		step = 1.0;
		if (dff <= xnull) step = va_min(step, 1.0 / c);
		if (dff > xnull) step = va_min(step, (dff + dff) / (-dga));
	L170:
		c = stmin + step;
		if (nfun >= ivmax) {
			phase = kDone;
			return;
		}
		nfun = nfun + 1;
		GBA_VA_LOOP
		for (i = 1; i <= jn; ++i) xbb[i] = xaa[i] + vm(c, d[i]);
		phase = kAfterLine;
	}
};

}  // namespace gba

#endif
