/*
 * energy_modes.cu -- fused normal-mode (flexible) docking energy + gradients.
 *
 * CPU semantics followed: CPUEnergyService6DModes::createItemProcessor
 * (src/service/CPUEnergyService6DModes.tpp:121-327).  One warp owns one pose:
 *   receptor pass  deform by the receptor amplitudes (rotate_translate_deform,
 *                  src/model/transform_modes.h:54-93), move into the ligand
 *                  frame with the "inverted" DOF (invertDOF, :27-41: angles
 *                  negated, t' = R^T (-t)), interpolate in the LIGAND grid,
 *                  rotate the force back by R (rotate_forces, :146-166) and
 *                  project it on the receptor modes (reduceModeForce, no
 *                  rotation, src/model/reduction_modes.h:68-90);
 *   ligand pass    deform + transform the ligand, interpolate in the receptor
 *                  grid, add the NL pair term against the DEFORMED receptor
 *                  (neighborlist_modes.h:21-206) whose reaction forces are
 *                  projected on the receptor modes pair by pair; reduce force,
 *                  energy, torque (undeformed ligand coordinates, reduceTorque)
 *                  and the ligand mode projection of R^T f (reduceModeForce
 *                  with rotation, reduction_modes.h:29-57);
 *   epilogue       warp sums, correctModeForce (delta += 4 k delta^4,
 *                  reduction_modes.h:101-115), ForceLim, TorqueMat.
 * The energy holds only the ligand-side terms, as in the reference.
 * Neighbour receptor positions are re-deformed per pair with the same unfused
 * operation sequence as the receptor pass, so no per-pose scratch is needed.
 * The reference's own GPU modes kernels are not followed: they mis-index the
 * deformed receptor and mode buffers (src/model/neighborlist_modes.cu:81-83,
 * src/model/transform_modes.cu:154, src/model/reduction_modes.cu:68-69).
 */
#include "energy_dev.cuh"
#include "va13.cuh"

namespace gba {

namespace {

/* Deformed receptor bead j (receptor frame): x_j + sum_m a_m v_jm, unfused in
 * mode order as rotate_translate_deform does. */
struct DeformedRecPos {
	const float4* __restrict__ xyzq;
	const float* __restrict__ modes;   /* [i][m][axis], stride ms floats */
	uint32_t M, ms;
	const float* amp;                  /* M amplitudes (registers of the caller) */
	__device__ __forceinline__ void operator()(uint32_t j, float& x, float& y, float& z, float& q) const {
		const float4 r = __ldg(&xyzq[j]);
		x = r.x; y = r.y; z = r.z; q = r.w;
		const float* v = modes + (size_t)j * ms;
#pragma unroll
		for (int m = 0; m < GBA_MODES_MAX; ++m) {
			if (m < (int)M) {
				x = fadd(x, fmul(amp[m], __ldg(v + 3 * m)));
				y = fadd(y, fmul(amp[m], __ldg(v + 3 * m + 1)));
				z = fadd(z, fmul(amp[m], __ldg(v + 3 * m + 2)));
			}
		}
	}
};

/* Projects each NL pair force on the receptor modes: the reaction force on
 * receptor bead j is -f, and the receptor mode gradient is -sum (force . v). */
struct RecModeHook {
	const float* __restrict__ modes;
	uint32_t M, ms;
	float* acc;                         /* M accumulators */
	__device__ __forceinline__ void operator()(uint32_t j, float fx, float fy, float fz) const {
		const float* v = modes + (size_t)j * ms;
#pragma unroll
		for (int m = 0; m < GBA_MODES_MAX; ++m)
			if (m < (int)M)
				acc[m] += fx * __ldg(v + 3 * m) + fy * __ldg(v + 3 * m + 1) + fz * __ldg(v + 3 * m + 2);
	}
};

}  // namespace

/* One pose of the modes energy.  Lane k (k < 26) brings the k-th float of the
 * DOF_6D_Modes record; returns on lane k (k < 27) the k-th float of the
 * Result_6D_Modes record.  Only the model fields of L are read. */
__device__ __forceinline__ float eval_pose_modes(const ModesLaunch& L, const float dv, const int lane) {
	const uint32_t Mr = L.rec.n_modes, Ml = L.lig.n_modes;
	{
		const float tx = __shfl_sync(GBA_FULL_MASK, dv, 0);
		const float ty = __shfl_sync(GBA_FULL_MASK, dv, 1);
		const float tz = __shfl_sync(GBA_FULL_MASK, dv, 2);
		const float a0 = __shfl_sync(GBA_FULL_MASK, dv, 3);
		const float a1 = __shfl_sync(GBA_FULL_MASK, dv, 4);
		const float a2 = __shfl_sync(GBA_FULL_MASK, dv, 5);
		float ampR[GBA_MODES_MAX], ampL[GBA_MODES_MAX];
#pragma unroll
		for (int m = 0; m < GBA_MODES_MAX; ++m) {
			ampR[m] = __shfl_sync(GBA_FULL_MASK, dv, 6 + m);
			ampL[m] = __shfl_sync(GBA_FULL_MASK, dv, 16 + m);
		}
		const PoseRot R = pose_rotation(a0, a1, a2, lane);
		/* R(-ang): same sin/cos with the sines negated (exact sign flips) */
		PoseRot Ri = R;
		{
			const float cphi = R.cphi, sphi = -R.sphi, cssi = R.cssi, sssi = -R.sssi;
			const float crot = R.crot, srot = -R.srot;
			const float cSSI_cPHI = fmul(cssi, cphi), cSSI_sPHI = fmul(cssi, sphi);
			const float sSSI_cPHI = fmul(sssi, cphi), sSSI_sPHI = fmul(sssi, sphi);
			Ri.m[0] = fadd(fmul(crot, cSSI_cPHI), fmul(srot, sphi));
			Ri.m[1] = fsub(fmul(srot, cSSI_cPHI), fmul(crot, sphi));
			Ri.m[2] = sSSI_cPHI;
			Ri.m[3] = fsub(fmul(crot, cSSI_sPHI), fmul(srot, cphi));
			Ri.m[4] = fadd(fmul(srot, cSSI_sPHI), fmul(crot, cphi));
			Ri.m[5] = sSSI_sPHI;
			Ri.m[6] = fmul(-crot, sssi);
			Ri.m[7] = fmul(-srot, sssi);
			Ri.m[8] = cssi;
		}
		/* t' = R^T * (-t), RotMat * Vec3 on the transposed matrix */
		const float ipx = fadd(fadd(fmul(R.m[0], -tx), fmul(R.m[3], -ty)), fmul(R.m[6], -tz));
		const float ipy = fadd(fadd(fmul(R.m[1], -tx), fmul(R.m[4], -ty)), fmul(R.m[7], -tz));
		const float ipz = fadd(fadd(fmul(R.m[2], -tx), fmul(R.m[5], -ty)), fmul(R.m[8], -tz));

		float gR[GBA_MODES_MAX], gL[GBA_MODES_MAX];
#pragma unroll
		for (int m = 0; m < GBA_MODES_MAX; ++m) { gR[m] = 0.f; gL[m] = 0.f; }

		/* ---- receptor beads in the ligand grid ---- */
		for (uint32_t j = lane; j < L.rec.n; j += 32) {
			const uint32_t mapped = __ldg(&L.rec.tm[j]) >> 16;
			if (mapped == 0) continue;
			float x, y, z, q;
			DeformedRecPos{L.rec.xyzq, L.rec_modes, Mr, L.rec_ms, ampR}(j, x, y, z, q);
			float px, py, pz;
			rot_apply(Ri.m, x, y, z, px, py, pz);
			px = fadd(px, ipx); py = fadd(py, ipy); pz = fadd(pz, ipz);
			float4 pot;
			bool charged;
			if (!bead_grid_term(L.grid_lig, px, py, pz, mapped, q, pot, charged)) continue;
			const float fx = R.m[0] * pot.x + R.m[1] * pot.y + R.m[2] * pot.z;
			const float fy = R.m[3] * pot.x + R.m[4] * pot.y + R.m[5] * pot.z;
			const float fz = R.m[6] * pot.x + R.m[7] * pot.y + R.m[8] * pot.z;
			const float* v = L.rec_modes + (size_t)j * L.rec_ms;
#pragma unroll
			for (int m = 0; m < GBA_MODES_MAX; ++m)
				if (m < (int)Mr)
					gR[m] -= fx * __ldg(v + 3 * m) + fy * __ldg(v + 3 * m + 1) + fz * __ldg(v + 3 * m + 2);
		}

		/* ---- ligand beads in the receptor grid + NL against the deformed receptor ---- */
		float sE = 0.f, sFx = 0.f, sFy = 0.f, sFz = 0.f;
		float T[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
		const DeformedRecPos recpos{L.rec.xyzq, L.rec_modes, Mr, L.rec_ms, ampR};
		const RecModeHook hook{L.rec_modes, Mr, L.rec_ms, gR};
		for (uint32_t i = lane; i < L.lig.n; i += 32) {
			const float4 b = __ldg(&L.lig.xyzq[i]);
			const uint32_t tm = __ldg(&L.lig.tm[i]);
			const uint32_t type = tm & 0xffffu, mapped = tm >> 16;
			const float* vl = L.lig_modes + (size_t)i * L.lig_ms;
			float x = b.x, y = b.y, z = b.z;
#pragma unroll
			for (int m = 0; m < GBA_MODES_MAX; ++m)
				if (m < (int)Ml) {
					x = fadd(x, fmul(ampL[m], __ldg(vl + 3 * m)));
					y = fadd(y, fmul(ampL[m], __ldg(vl + 3 * m + 1)));
					z = fadd(z, fmul(ampL[m], __ldg(vl + 3 * m + 2)));
				}
			float px, py, pz;
			rot_apply(R.m, x, y, z, px, py, pz);
			px = fadd(px, tx); py = fadd(py, ty); pz = fadd(pz, tz);
			float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
			float4 pot;
			bool charged;
			if (bead_grid_term(L.grid_rec, px, py, pz, mapped, b.w, pot, charged)) {
				fx = pot.x; fy = pot.y; fz = pot.z; e = pot.w;
			}
			if (type != 0) {
				uint32_t npairs = 0;
				bead_nl_term(L.grid_rec.nl, L.par, L.rec.tm, recpos, px, py, pz, type, b.w,
						fx, fy, fz, e, npairs, hook);
			}
			sE += e; sFx += fx; sFy += fy; sFz += fz;
			T[0] += b.x * fx; T[1] += b.y * fx; T[2] += b.z * fx;
			T[3] += b.x * fy; T[4] += b.y * fy; T[5] += b.z * fy;
			T[6] += b.x * fz; T[7] += b.y * fz; T[8] += b.z * fz;
			/* R^T f, projected on the ligand modes */
			const float rx = R.m[0] * fx + R.m[3] * fy + R.m[6] * fz;
			const float ry = R.m[1] * fx + R.m[4] * fy + R.m[7] * fz;
			const float rz = R.m[2] * fx + R.m[5] * fy + R.m[8] * fz;
#pragma unroll
			for (int m = 0; m < GBA_MODES_MAX; ++m)
				if (m < (int)Ml)
					gL[m] -= rx * __ldg(vl + 3 * m) + ry * __ldg(vl + 3 * m + 1) + rz * __ldg(vl + 3 * m + 2);
		}

		sE = warp_sum(sE); sFx = warp_sum(sFx); sFy = warp_sum(sFy); sFz = warp_sum(sFz);
#pragma unroll
		for (int k = 0; k < 9; ++k) T[k] = warp_sum(T[k]);
#pragma unroll
		for (int m = 0; m < GBA_MODES_MAX; ++m) {
			if (m < (int)Mr) gR[m] = warp_sum(gR[m]);
			if (m < (int)Ml) gL[m] = warp_sum(gL[m]);
		}
		force_lim(sFx, sFy, sFz);
		float ang[3];
		torque_reduce(R, T, ang);
		/* correctModeForce: delta += (float)(4 k * delta^4) */
#pragma unroll
		for (int m = 0; m < GBA_MODES_MAX; ++m) {
			if (m < (int)Mr) {
				const double dl = gR[m];
				gR[m] = gR[m] + (float)((double)(4.0f * L.rec.mode_force[m]) * (dl * dl) * (dl * dl));
			}
			if (m < (int)Ml) {
				const double dl = gL[m];
				gL[m] = gL[m] + (float)((double)(4.0f * L.lig.mode_force[m]) * (dl * dl) * (dl * dl));
			}
		}
		/* Result_6D_Modes: E, pos xyz, ang xyz, modesRec[10], modesLig[10] */
		float v = 0.f;
		if (lane == 0) v = sE;
		else if (lane == 1) v = sFx;
		else if (lane == 2) v = sFy;
		else if (lane == 3) v = sFz;
		else if (lane == 4) v = ang[0];
		else if (lane == 5) v = ang[1];
		else if (lane == 6) v = ang[2];
#pragma unroll
		for (int m = 0; m < GBA_MODES_MAX; ++m) {
			if (lane == 7 + m) v = m < (int)Mr ? gR[m] : 0.f;
			if (lane == 17 + m) v = m < (int)Ml ? gL[m] : 0.f;
		}
		return v;
	}
}

__global__ void __launch_bounds__(256) modes_energy_kernel(const ModesLaunch L) {
	const int lane = threadIdx.x & 31;
	const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
	for (size_t p = warp; p < L.n; p += nwarps) {
		const float* d = reinterpret_cast<const float*>(L.dofs + p);
		const float dv = lane < 26 ? __ldg(d + lane) : 0.f;
		const float v = eval_pose_modes(L, dv, lane);
		if (lane < 27) reinterpret_cast<float*>(L.out + p)[lane] = v;
	}
}

/* Persistent VA13 over (ang xyz, pos xyz, modesRec[0..Mr), modesLig[0..Ml)):
 * the minimizer of minimize.cu generalised to 6 + Mr + Ml DOF (minfor.f is
 * fixed at 6, src/apps/em/minfor.f:16,33). */
__global__ void __launch_bounds__(256) minimize_modes_kernel(const ModesMinLaunch M) {
	const int lane = threadIdx.x & 31;
	const ModesLaunch& L = M.m;
	const uint32_t Mr = L.rec.n_modes, Ml = L.lig.n_modes;
	const int jn = 6 + (int)Mr + (int)Ml;
	for (;;) {
		unsigned long long slot = 0;
		if (lane == 0) slot = atomicAdd(M.counter, 1ull);
		slot = __shfl_sync(GBA_FULL_MASK, slot, 0);
		if (slot >= M.n) break;
		const size_t p = (size_t)slot;
		VA13<6 + 2 * GBA_MODES_MAX> va;
		/* lane k holds DOF float k (pos, ang, modesRec[10], modesLig[10]) */
		float dv = lane < 26 ? __ldg(reinterpret_cast<const float*>(M.start + p) + lane) : 0.f;
		if (lane == 0) {
			double x0[6 + 2 * GBA_MODES_MAX];
			const float* s = reinterpret_cast<const float*>(M.start + p);
			for (int k = 0; k < 3; ++k) { x0[k] = s[3 + k]; x0[3 + k] = s[k]; }
			for (uint32_t m = 0; m < Mr; ++m) x0[6 + m] = s[6 + m];
			for (uint32_t m = 0; m < Ml; ++m) x0[6 + Mr + m] = s[16 + m];
			va.start(x0, jn, M.max_evals);
		}
		float v = 0.f;
		int nev = 0;
		for (;;) {
			/* lane 0 scatters the point to be evaluated into the record layout */
			float rec[26];
			if (lane == 0) {
				const double* pt = va.point();
				for (int k = 0; k < 26; ++k) rec[k] = 0.f;
				for (int k = 0; k < 3; ++k) { rec[3 + k] = (float)pt[k]; rec[k] = (float)pt[3 + k]; }
				for (uint32_t m = 0; m < Mr; ++m) rec[6 + m] = (float)pt[6 + m];
				for (uint32_t m = 0; m < Ml; ++m) rec[16 + m] = (float)pt[6 + Mr + m];
			}
#pragma unroll
			for (int k = 0; k < 26; ++k) {
				const float t = __shfl_sync(GBA_FULL_MASK, lane == 0 ? rec[k] : 0.f, 0);
				if (lane == k) dv = t;
			}
			v = eval_pose_modes(L, dv, lane);
			++nev;
			/* gather the result record on lane 0 */
			float res[27];
#pragma unroll
			for (int k = 0; k < 27; ++k) res[k] = __shfl_sync(GBA_FULL_MASK, v, k);
			int done = 0;
			if (lane == 0) {
				double g[6 + 2 * GBA_MODES_MAX];
				for (int k = 0; k < 3; ++k) { g[k] = -(double)res[4 + k]; g[3 + k] = -(double)res[1 + k]; }
				for (uint32_t m = 0; m < Mr; ++m) g[6 + m] = -(double)res[7 + m];
				for (uint32_t m = 0; m < Ml; ++m) g[6 + Mr + m] = -(double)res[17 + m];
				va.provide((double)res[0], g);
				done = va.done();
			}
			if (__shfl_sync(GBA_FULL_MASK, done, 0)) break;
		}
		if (lane < 27) reinterpret_cast<float*>(M.out_result + p)[lane] = v;
		if (lane < 26) reinterpret_cast<float*>(M.out_state + p)[lane] = dv;
		if (lane == 0 && M.out_nevals) M.out_nevals[p] = nev;
	}
}

cudaError_t launch_minimize_modes(const ModesMinLaunch& M, int blocks, int threads, cudaStream_t s) {
	minimize_modes_kernel<<<blocks, threads, 0, s>>>(M);
	return cudaGetLastError();
}

int minimize_modes_blocks_per_sm(int threads) {
	int nb = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, minimize_modes_kernel, threads, 0);
	return nb > 0 ? nb : 1;
}

cudaError_t launch_modes_energy(const ModesLaunch& L, int blocks, int threads, cudaStream_t s) {
	modes_energy_kernel<<<blocks, threads, 0, s>>>(L);
	return cudaGetLastError();
}

int modes_blocks_per_sm(int threads) {
	int nb = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, modes_energy_kernel, threads, 0);
	return nb > 0 ? nb : 1;
}

}  // namespace gba
