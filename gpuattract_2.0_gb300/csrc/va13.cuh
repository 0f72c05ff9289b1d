/*
 * va13.cuh -- the VA13 variable-metric minimizer as a resumable state machine.
 *
 * Follows the Harwell routine the reference runs for every pose
 * (src/apps/em/minfor.f:1-182 with mc11a/mc11e, src/apps/em/mc11a.f:1-143),
 * in FP64 like the Fortran's real*8, generalised from its fixed 6 DOF to n DOF.
 * Instead of calling the energy function, the machine stops whenever minfor
 * would call it: `point()` is the DOF vector to evaluate, `provide(f, g)` hands
 * back the objective and gradient and runs to the next evaluation (or to the
 * end).  The host (plain per-step driver) runs `provide`; the device kernels
 * run `provide_w`, the same arithmetic spread over a warp's lanes (the warp
 * form, below), which takes the same trajectory bit for bit.  Arrays are
 * 1-based, mirroring the Fortran.
 */
#ifndef GBA_VA13_CUH_
#define GBA_VA13_CUH_

#include <cmath>

#ifdef __CUDACC__
#define GBA_HD __host__ __device__ __forceinline__
#else
#define GBA_HD inline
#endif

/* Device loops of the machine stay rolled: it runs between two evaluations
 * of the whole warp, and unrolled copies of its loops evicted the
 * evaluation's code from the instruction cache (measured with one lane
 * stepping it: instruction-fetch stalls; the minimizers ran 7-9 % slower
 * unrolled). */
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

/* ---- the warp form ----------------------------------------------------
 * On GB300 every FP64 instruction a warp issues occupies the narrow FP64
 * pipe for the whole warp, whether one lane or 32 take part, so the machine
 * run by one lane costs what its ~650 FP64 instructions per step cost.  The
 * warp form runs the same arithmetic with every lane of the warp:
 * - scalar work is done redundantly by all lanes (same operands, same
 *   results), so it costs no more than on one lane;
 * - element-wise updates (element j on lane j) take one instruction for all
 *   elements instead of one per element;
 * - divisions that do not depend on each other are issued together on
 *   separate lanes.
 * Each element sees the same operations in the same order as in mc11a,
 * mc11e and minfor, so the trajectory is the same bit for bit.
 *
 * Executors.  `each(lo, hi, f)` runs f(j) for the elements j in [lo, hi]:
 * on the device on lanes lo..hi between two __syncwarp()s; on the host (the
 * tests) in DESCENDING order, so that an element that depended on another
 * element of the same section would change the trajectory.  Shared state is
 * written only inside `each` (so no lane can read a location in scalar code
 * while another lane writes it); scalar code between sections only reads. */
struct VaSerial {
	GBA_HD void sync() const {}
	template <class F>
	GBA_HD void each(int lo, int hi, F f) const {
		for (int j = hi; j >= lo; --j) f(j);
	}
};

struct VaWarp {
	int lane;
	GBA_HD void sync() const {
#ifdef __CUDA_ARCH__
		__syncwarp();
#endif
	}
	template <class F>
	GBA_HD void each(int lo, int hi, F f) const {
#ifdef __CUDA_ARCH__
		__syncwarp();
		if (lane >= lo && lane <= hi) f(lane);
		__syncwarp();
#else
		for (int j = hi; j >= lo; --j) f(j);
#endif
	}
};

/* index of diagonal entry i in the packed upper triangle (row-major, rows of
 * n, n-1, ... entries; 1-based) */
GBA_HD int va_diag(int i, int n) { return (i - 1) * (2 * n - i + 2) / 2 + 1; }

/* mc11a in the warp form (every lane calls it; ir in and out on every lane;
 * q, t: scratch of n + 1 doubles).  Beyond the element-wise updates:
 * - the first loop (mk != 0) only feeds ti, which ir <= 0 discards at L20
 *   (minfor's first call always has ir = -n): it runs only for ir > 0, its
 *   divisions together;
 * - the divisions of the L23 recurrence, w_j^2 / a_jj, depend only on the
 *   entry values: all at once;
 * - in the L41 loop, r = ti/tim, b = al/ti, gm = tim/ti and the next row's
 *   al = (z_{i+1} - v a_{i,i+1}) / a_{i+1,i+1} -- z_{i+1} after this row's
 *   update, which both branches compute as z - v * (old a) -- in one
 *   division on four lanes. */
template <class X>
GBA_HD void mc11a_w(double* a, int n, double* z, double sig, double* w, int& ir, int mk, double eps, double* q,
		double* t, const X& ex) {
	if (n <= 1) {
		const double a1 = a[1] + vm(vm(sig, z[1]), z[1]);
		ex.each(1, 1, [&](int) { a[1] = a1 > 0.0 ? a1 : 0.0; });
		ir = a1 > 0.0 ? 1 : 0;
		return;
	}
	const int np = n + 1;
	double ti = 0.0, tim = 0.0;
	int mm = 0;
	if (sig > 0.0) goto L40;
	if (sig == 0.0 || ir == 0) return;
	ti = 1.0 / sig;
	if (mk == 0) goto L10;
	if (ir > 0) {
		ex.each(1, n, [&](int j) {
			const double dj = a[va_diag(j, n)];
			q[j] = dj != 0.0 ? vm(w[j], w[j]) / dj : 0.0;
		});
		for (int i = 1; i <= n; ++i)
			if (a[va_diag(i, n)] != 0.0) ti = ti + q[i];
	}
	goto L20;
L10:
	ex.each(1, n, [&](int j) { w[j] = z[j]; });
	for (int i = 1; i <= n; ++i) {
		const int ij = va_diag(i, n);
		const double v = w[i];
		if (a[ij] > 0.0) {
			ti = ti + vm(v, v) / a[ij];
			if (i != n) ex.each(i + 1, n, [&](int j) { w[j] = w[j] - vm(v, a[ij + j - i]); });
		} else {
			ex.each(i, i, [&](int) { w[i] = 0.0; });
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
	ex.each(1, n, [&](int j) {
		const double dj = a[va_diag(j, n)];
		q[j] = dj != 0.0 ? vm(w[j], w[j]) / dj : 0.0;
	});
	tim = ti;
	for (int i = 1; i <= n; ++i) {
		const int j = np - i;
		if (a[va_diag(j, n)] != 0.0) tim = ti - q[j];
		ex.each(0, 0, [&](int) { t[j] = ti; });
		ti = tim;
	}
	ex.each(1, n, [&](int j) { w[j] = t[j]; });
	goto L41;
L40:
	mm = 0;
	tim = 1.0 / sig;
L41: {
	bool have_al = false;
	double al = 0.0;
	for (int i = 1; i <= n; ++i) {
		const int ij = va_diag(i, n);
		const double v = z[i];
		const double aii = a[ij];
		if (!(aii > 0.0)) {
			if (ir > 0 || sig < 0.0 || v == 0.0) {
				ti = tim;
				have_al = false;
				continue;
			}
			ir = 1 - ir;
			ex.each(i, n, [&](int j) {
				if (j == i) a[ij] = vm(v, v) / tim;
				else a[ij + j - i] = z[j] / v;
			});
			return;
		}
		if (!have_al) al = v / aii;
		if (mm <= 0) ti = tim + vm(v, al);
		else ti = w[i];
		ex.each(0, 3, [&](int k) {
			double nu = ti, de = tim;                     /* r */
			if (k == 1) { nu = al; de = ti; }             /* b */
			else if (k == 2) { nu = tim; de = ti; }       /* gm */
			else if (k == 3) {                            /* the next row's al */
				nu = 0.0;
				de = 1.0;
				if (i < n) {
					nu = z[i + 1] - vm(v, a[ij + 1]);
					de = a[va_diag(i + 1, n)];
				}
			}
			q[k] = nu / de;
		});
		const double r = q[0], b = q[1], gm = q[2];
		al = q[3];
		have_al = true;
		if (r == 0.0 || i == n) {
			ex.each(i, i, [&](int) { a[ij] = vm(aii, r); });
			break;
		}
		if (r > 4.0) {
			ex.each(i, n, [&](int j) {
				if (j == i) {
					a[ij] = vm(aii, r);
					return;
				}
				const int k = ij + j - i;
				const double y = a[k];
				a[k] = vm(b, z[j]) + vm(y, gm);
				z[j] = z[j] - vm(v, y);
			});
		} else {
			ex.each(i, n, [&](int j) {
				if (j == i) {
					a[ij] = vm(aii, r);
					return;
				}
				const int k = ij + j - i;
				z[j] = z[j] - vm(v, a[k]);
				a[k] = a[k] + vm(b, z[j]);
			});
		}
		tim = ti;
	}
}
	if (ir < 0) ir = -ir;
}

/* mc11e in the warp form (q, t: scratch of n + 1 doubles).  The forward
 * substitution by columns: after z_j is final, lanes i > j subtract
 * a(j,i) z_j, so each z_i meets a(1,i) z_1, a(2,i) z_2, ... in the row
 * form's order.  The back substitution's divisions z_i / a_ii use the
 * forward values and go together; each row's products go together, its
 * differences stay a chain in the row form's order. */
template <class X>
GBA_HD void mc11e_w(const double* a, int n, double* z, double* w, int ir, double* q, double* t, const X& ex) {
	if (ir < n) return;
	if (n <= 1) {
		ex.each(1, 1, [&](int) {
			w[1] = z[1];
			z[1] = z[1] / a[1];
		});
		return;
	}
	for (int j = 1; j < n; ++j) {
		const double zj = z[j];
		const int dj = va_diag(j, n);
		ex.each(j + 1, n, [&](int i) {
			z[i] = z[i] - vm(a[dj + i - j], zj);
			if (i == j + 1) w[i] = z[i];
		});
	}
	/* the divisions; z_n's is its result; the products of row n - 1 */
	const int dm = va_diag(n - 1, n);
	ex.each(1, n, [&](int i) {
		if (i == 1) w[1] = z[1];
		q[i] = z[i] / a[va_diag(i, n)];
		if (i == n) {
			z[n] = q[n];
			t[n] = vm(a[dm + 1], q[n]);
		}
	});
	for (int i = n - 1; i >= 1; --i) {
		double v = q[i];
		for (int j = i + 1; j <= n; ++j) v = v - t[j];
		/* z_i final; the products of row i - 1 (z_i's from v) */
		const int dp = i > 1 ? va_diag(i - 1, n) : 0;
		ex.each(i, n, [&](int j) {
			if (j == i) z[i] = v;
			if (i > 1) t[j] = vm(a[dp + j - (i - 1)], j == i ? v : z[j]);
		});
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
	double q[NMAX + 1], t[NMAX + 1];   /* scratch of the warp form */

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

	/* provide() in the warp form (see VaWarp): every lane of the warp calls
	 * it, the state in memory all lanes read (shared memory).  grad(j) is
	 * gradient element j (1-based), called on the lane that owns element j.
	 * The scalars live in registers, identical on every lane, and go back to
	 * the state at the end. */
	template <class X, class Grad>
	GBA_HD void provide_w(double f, Grad grad, const X& ex) {
		static_assert(NMAX >= 3 && NMAX <= 31, "one lane per element; four division lanes");
		ex.sync();   /* start() or the last step wrote the state */
		int phase = this->phase;
		if (phase != kAfterFirst && phase != kAfterLine) return;
		const int jn = this->jn, ivmax = this->ivmax;
		const double acc = this->acc;
		int nfun = this->nfun, itr = this->itr, isfv = this->isfv, ir = this->ir;
		double gesa = this->gesa, c = this->c, dff = this->dff, dgb = this->dgb, fa = this->fa, fb = this->fb;
		double fmin = this->fmin, gmin = this->gmin, dga = this->dga;
		double step = this->step, stepbd = this->stepbd, steplb = this->steplb, stmin = this->stmin;
		const double xnull = 0.0;
		int i;
		if (phase == kAfterFirst) {
			gesa = f;
			ex.each(1, jn, [&](int j) { g[j] = grad(j); });
			goto L110;
		}
		fb = f;
		ex.each(1, jn, [&](int j) { gb[j] = grad(j); });
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
		ex.each(1, jn, [&](int j) {
			x[j] = xbb[j];
			g[j] = gb[j];
		});
	L220:
		dgb = xnull;
		GBA_VA_LOOP
		for (i = 1; i <= jn; ++i) dgb = dgb + vm(gb[i], d[i]);
		if (fb - fa <= vm(vm(0.1, c), dga)) goto L280;
		if (step > steplb) goto L270;
	L240:
		if (isfv >= 2) goto L110;
		phase = kDone;
		goto Lsave;
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
		ex.each(1, jn, [&](int j) {
			xaa[j] = xbb[j];
			xbb[j] = ga[j];
			d[j] = gb[j] - ga[j];
			ga[j] = gb[j];
		});
		mc11a_w(h, jn, xbb, 1.0 / dga, w, ir, 1, xnull, q, t, ex);
		ir = -ir;
		mc11a_w(h, jn, d, 1.0 / vm(stmin, dgb - dga), d, ir, 0, xnull, q, t, ex);
		if (ir < jn) {
			phase = kDone;
			goto Lsave;
		}
		dff = fa - fb;
		fa = fb;
		goto L135;
	L110:
		fa = gesa;
		isfv = 1;
		ex.each(1, jn, [&](int j) { ga[j] = g[j]; });
	L135:
		itr = itr + 1;
		ex.each(1, jn, [&](int j) { d[j] = -ga[j]; });
		mc11e_w(h, jn, d, w, jn, q, t, ex);
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
			goto Lsave;
		}
		nfun = nfun + 1;
		ex.each(1, jn, [&](int j) { xbb[j] = xaa[j] + vm(c, d[j]); });
		phase = kAfterLine;
	Lsave:
		ex.each(0, 0, [&](int) {
			this->phase = phase;
			this->nfun = nfun;
			this->itr = itr;
			this->isfv = isfv;
			this->ir = ir;
			this->gesa = gesa;
			this->c = c;
			this->dff = dff;
			this->dgb = dgb;
			this->fa = fa;
			this->fb = fb;
			this->fmin = fmin;
			this->gmin = gmin;
			this->dga = dga;
			this->step = step;
			this->stepbd = stepbd;
			this->steplb = steplb;
			this->stmin = stmin;
		});
	}
};

}  // namespace gba

#endif
