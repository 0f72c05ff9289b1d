/*
 * energy_modes.cu -- fused normal-mode (flexible) docking energy + gradients.
 *
 * CPU semantics followed: CPUEnergyService6DModes::createItemProcessor
 * (src/service/CPUEnergyService6DModes.tpp:121-327).  One warp owns one pose
 * and works in rounds of 64 beads staged in shared memory, like the rigid
 * kernel (rigid_pose.cuh), in two passes:
 *   receptor pass  deform by the receptor amplitudes (rotate_translate_deform,
 *                  src/model/transform_modes.h:54-93), move into the ligand
 *                  frame with the "inverted" DOF (invertDOF, :27-41: angles
 *                  negated, t' = R^T (-t)), interpolate in the LIGAND grid,
 *                  rotate the force back by R (rotate_forces, :146-166) and
 *                  project it on the receptor modes (reduceModeForce without
 *                  rotation, src/model/reduction_modes.h:68-90);
 *   ligand pass    deform + transform the ligand, interpolate in the receptor
 *                  grid, add the NL pair term against the DEFORMED receptor
 *                  (neighborlist_modes.h:21-206) whose reaction forces are
 *                  projected on the receptor modes pair by pair; energy, force,
 *                  torque (undeformed ligand coordinates, reduceTorque) and the
 *                  ligand mode projection of R^T f (reduceModeForce with
 *                  rotation, reduction_modes.h:29-57) are summed per lookup
 *                  and per pair (all linear in the bead forces);
 *   epilogue       warp sums, correctModeForce (delta += 4 k delta^4,
 *                  reduction_modes.h:101-115), ForceLim, TorqueMat.
 * The energy holds only the ligand-side terms, as in the reference.
 * Neighbour receptor positions are re-deformed per pair with the same unfused
 * operation sequence as the receptor pass, so no per-pose scratch is needed.
 *
 * Every mode projection is linear in the force: f . (R^T v) replaces
 * (R f) . v and f . (R v) replaces (R^T f) . v, so each staged bead's mode
 * vectors are rotated once per round into shared memory (ModeStage) and a
 * projection costs no global load and no rotation.  On octet grids the grid
 * lookups of both passes take the rigid kernel's 8-lane cooperative form
 * (CoopStep): the lane holding force component c adds f_c times component
 * c of the staged vector.  Kernels are compiled for mode capacities 5 and 10
 * (arrays sized to the capacity, not to GBA_MODES_MAX).
 * The reference's own GPU modes kernels are not followed: they mis-index the
 * deformed receptor and mode buffers (src/model/neighborlist_modes.cu:81-83,
 * src/model/transform_modes.cu:154, src/model/reduction_modes.cu:68-69).
 */
#include <algorithm>

#include "rigid_pose.cuh"
#include "va13.cuh"

namespace gba {

namespace {

/* Floats of a bead's mode record held in registers (mode_stride(MM)). */
template <int MM>
constexpr int kModeWords = (3 * MM + 3) / 4;

/* The bead's M mode vectors from its 16-byte aligned record v (padded to
 * whole float4s): one 16-byte load per four floats instead of one load per
 * float -- the records of a warp's beads lie apart, so every load is a
 * separate L1 wavefront. */
template <int MM>
__device__ __forceinline__ void load_modes(const float* __restrict__ v, uint32_t M, float (&w)[4 * kModeWords<MM>]) {
	const float4* q = reinterpret_cast<const float4*>(v);
#pragma unroll
	for (int k = 0; k < kModeWords<MM>; ++k) {
		const float4 t = 4 * k < 3 * (int)M ? __ldg(q + k) : make_float4(0.f, 0.f, 0.f, 0.f);
		w[4 * k] = t.x; w[4 * k + 1] = t.y; w[4 * k + 2] = t.z; w[4 * k + 3] = t.w;
	}
}

/* x + sum_m a_m v_m, unfused in mode order (rotate_translate_deform), with
 * the bead's vectors w already loaded. */
template <int MM>
__device__ __forceinline__ void deform_w(const float (&w)[4 * kModeWords<MM>], uint32_t M, const float* amp,
		float& x, float& y, float& z) {
#pragma unroll
	for (int m = 0; m < MM; ++m)
		if (m < (int)M) {
			x = fadd(x, fmul(amp[m], w[3 * m]));
			y = fadd(y, fmul(amp[m], w[3 * m + 1]));
			z = fadd(z, fmul(amp[m], w[3 * m + 2]));
		}
}

template <int MM>
__device__ __forceinline__ void deform(const float* __restrict__ v, uint32_t M, const float* amp,
		float& x, float& y, float& z) {
	float w[4 * kModeWords<MM>];
	load_modes<MM>(v, M, w);
	deform_w<MM>(w, M, amp, x, y, z);
}

/* acc[m] += sign * (f . v_m) */
template <int MM>
__device__ __forceinline__ void project(const float* __restrict__ v, uint32_t M, float fx, float fy,
		float fz, float sign, float* acc) {
	float w[4 * kModeWords<MM>];
	load_modes<MM>(v, M, w);
#pragma unroll
	for (int m = 0; m < MM; ++m)
		if (m < (int)M)
			acc[m] = ffma(sign, ffma(fz, w[3 * m + 2], ffma(fy, w[3 * m + 1], fmul(fx, w[3 * m]))), acc[m]);
}

/* Per warp and round: each staged bead's mode vectors, rotated into the frame
 * of the forces they are projected on, component-major. */
template <int MM>
struct ModeStage {
	float w[kBeadsPerRound][3][MM];
};

/* Rotated mode vectors of slot s: w_m = R v_m (transpose = false) or R^T v_m,
 * from the bead's loaded vectors w. */
template <int MM>
__device__ __forceinline__ void stage_modes(ModeStage<MM>& S, int s, const float (&w)[4 * kModeWords<MM>],
		uint32_t M, const float m9[9], bool transpose) {
#pragma unroll
	for (int m = 0; m < MM; ++m)
		if (m < (int)M) {
			const float vx = w[3 * m], vy = w[3 * m + 1], vz = w[3 * m + 2];
			float a, b, c;
			if (transpose) rot_apply_t(m9, vx, vy, vz, a, b, c);
			else rot_apply(m9, vx, vy, vz, a, b, c);
			S.w[s][0][m] = a;
			S.w[s][1][m] = b;
			S.w[s][2][m] = c;
		}
}

/* acc[m] += sign * (f . w_m) with the staged vectors of slot s */
template <int MM>
__device__ __forceinline__ void project_staged(const ModeStage<MM>& S, uint32_t s, uint32_t M, float fx,
		float fy, float fz, float sign, float* acc) {
#pragma unroll
	for (int m = 0; m < MM; ++m)
		if (m < (int)M)
			acc[m] = ffma(sign, ffma(fz, S.w[s][2][m], ffma(fy, S.w[s][1][m], fmul(fx, S.w[s][0][m]))), acc[m]);
}

/* acc[m] -= f_c * w_m[c]: the cooperative lane holding force component c */
template <int MM>
__device__ __forceinline__ void project_component(const ModeStage<MM>& S, uint32_t s, int c, uint32_t M,
		float f, float* acc) {
#pragma unroll
	for (int m = 0; m < MM; ++m)
		if (m < (int)M) acc[m] = ffma(-f, S.w[s][c][m], acc[m]);
}

}  // namespace

/* The pose frame of both passes: the rotation, its "inverted" counterpart
 * R(-ang) and t' = R^T (-t) (invertDOF, src/model/transform_modes.h:27-41),
 * and the translation. */
struct ModesFrame {
	PoseRot R;
	float Ri[9];
	float ip[3];
	float t[3];
};

/* Lane k (k < 26) brings the k-th float of the DOF_6D_Modes record; every
 * lane gets the frame and the amplitudes. */
template <int MM>
__device__ __forceinline__ ModesFrame modes_frame(const float dv, const int lane, float ampR[MM], float ampL[MM],
		const DevTrig& T) {
	ModesFrame F;
	F.t[0] = __shfl_sync(GBA_FULL_MASK, dv, 0);
	F.t[1] = __shfl_sync(GBA_FULL_MASK, dv, 1);
	F.t[2] = __shfl_sync(GBA_FULL_MASK, dv, 2);
	const float a0 = __shfl_sync(GBA_FULL_MASK, dv, 3);
	const float a1 = __shfl_sync(GBA_FULL_MASK, dv, 4);
	const float a2 = __shfl_sync(GBA_FULL_MASK, dv, 5);
#pragma unroll
	for (int m = 0; m < MM; ++m) {
		ampR[m] = __shfl_sync(GBA_FULL_MASK, dv, 6 + m);
		ampL[m] = __shfl_sync(GBA_FULL_MASK, dv, 16 + m);
	}
	F.R = pose_rotation(a0, a1, a2, lane, T);
	const PoseRot& R = F.R;
	/* R(-ang): same sin/cos with the sines negated (exact sign flips) */
	{
		const float cphi = R.cphi, sphi = -R.sphi, cssi = R.cssi, sssi = -R.sssi;
		const float crot = R.crot, srot = -R.srot;
		const float cSSI_cPHI = fmul(cssi, cphi), cSSI_sPHI = fmul(cssi, sphi);
		const float sSSI_cPHI = fmul(sssi, cphi), sSSI_sPHI = fmul(sssi, sphi);
		F.Ri[0] = fadd(fmul(crot, cSSI_cPHI), fmul(srot, sphi));
		F.Ri[1] = fsub(fmul(srot, cSSI_cPHI), fmul(crot, sphi));
		F.Ri[2] = sSSI_cPHI;
		F.Ri[3] = fsub(fmul(crot, cSSI_sPHI), fmul(srot, cphi));
		F.Ri[4] = fadd(fmul(srot, cSSI_sPHI), fmul(crot, cphi));
		F.Ri[5] = sSSI_sPHI;
		F.Ri[6] = fmul(-crot, sssi);
		F.Ri[7] = fmul(-srot, sssi);
		F.Ri[8] = cssi;
	}
	/* t' = R^T * (-t), RotMat * Vec3 on the transposed matrix */
	const float tx = F.t[0], ty = F.t[1], tz = F.t[2];
	F.ip[0] = fadd(fadd(fmul(R.m[0], -tx), fmul(R.m[3], -ty)), fmul(R.m[6], -tz));
	F.ip[1] = fadd(fadd(fmul(R.m[1], -tx), fmul(R.m[4], -ty)), fmul(R.m[7], -tz));
	F.ip[2] = fadd(fadd(fmul(R.m[2], -tx), fmul(R.m[5], -ty)), fmul(R.m[8], -tz));
	return F;
}

/* Receptor pass: the receptor beads, deformed and moved into the ligand
 * frame, in the LIGAND grid; each force rotated back by R and projected on
 * the receptor modes into the lane sums gR. */
template <int MM>
__device__ __forceinline__ void modes_rec_pass(const ModesLaunch& L, const ModesFrame& F, const float ampR[MM],
		const int lane, WarpStage& W, ModeStage<MM>& MS, float gR[MM]) {
	const uint32_t Mr = L.rec.n_modes;
	const PoseRot& R = F.R;
	const float* Ri = F.Ri;
	const float ipx = F.ip[0], ipy = F.ip[1], ipz = F.ip[2];
	const int comp = coop_component(lane);
	for (uint32_t j0 = 0; j0 < L.rec.n; j0 += kBeadsPerRound) {
		uint32_t nlk[2];
		BeadGrid bg[2];
#pragma unroll
		for (int h = 0; h < 2; ++h) {
			const int s = lane + 32 * h;
			const uint32_t j = j0 + s;
			nlk[h] = 0;
			bg[h] = BeadGrid{0u, 0u};
			if (j < L.rec.n) {
				const float4 r = __ldg(&L.rec.xyzq[j]);
				const uint32_t mapped = __ldg(&L.rec.tm[j]) >> 16;
				float vw[4 * kModeWords<MM>];
				load_modes<MM>(L.rec_modes + (size_t)j * L.rec_ms, Mr, vw);
				float x = r.x, y = r.y, z = r.z;
				deform_w<MM>(vw, Mr, ampR, x, y, z);
				float px, py, pz;
				rot_apply(Ri, x, y, z, px, py, pz);
				px = fadd(px, ipx); py = fadd(py, ipy); pz = fadd(pz, ipz);
				put_bead(W, s, 0.f, 0.f, 0.f, px, py, pz, r.w, j);
				nlk[h] = stage_grid(L.grid_lig, px, py, pz, mapped, r.w, s, W, bg[h]);
				/* the ligand-frame force f is rotated back by R before the
				 * projection: (R f) . v = f . (R^T v); staged for the
				 * cooperative lookups only (one lookup per bead or two: the
				 * per-lane form rotates f instead) */
				if (nlk[h] && L.grid_lig.coop_lookup) stage_modes<MM>(MS, s, vw, Mr, R.m, true);
			}
		}
		const uint32_t n_look = queue_lookups(W, nlk, bg, lane);
		__syncwarp();
		if (L.grid_lig.coop_lookup) {
			for (uint32_t k0 = 0; k0 < n_look; k0 += 16) {
				CoopStep<2> st;
				st.load(L.grid_lig, W, k0, n_look, lane);
#pragma unroll
				for (int b = 0; b < 2; ++b) {
					const float v = st.component(b, lane);
					if (st.ok[b] && comp < 3) project_component<MM>(MS, st.sl[b], comp, Mr, fmul(v, st.sc[b]), gR);
				}
			}
		} else {
			for (uint32_t q = lane; q < n_look; q += 32) {
				const uint32_t s = lookup_slot(W, q);
				const float4 v = grid_lookup(L.grid_lig, W, q);
				/* back into the receptor frame, then -(force . mode) */
				float fx, fy, fz;
				rot_apply(R.m, v.x, v.y, v.z, fx, fy, fz);
				project<MM>(L.rec_modes + (size_t)__float_as_uint(W.ut[s].w) * L.rec_ms, Mr, fx, fy, fz, -1.f, gR);
			}
		}
		__syncwarp();
	}

}

/* Ligand pass: the ligand beads, deformed and moved into the receptor frame,
 * in the receptor grid, plus the NL pairs against the deformed receptor:
 * energy, force and torque into S and C, ligand mode projections into gL,
 * the pairs' reaction forces projected on the receptor modes into gR. */
template <int MM>
__device__ __forceinline__ void modes_lig_pass(const ModesLaunch& L, const ModesFrame& F, const float ampR[MM],
		const float ampL[MM], const int lane, WarpStage& W, ModeStage<MM>& MS, PoseSums& S, CoopSums& C,
		float gL[MM], float gR[MM]) {
	const uint32_t Mr = L.rec.n_modes, Ml = L.lig.n_modes;
	const PoseRot& R = F.R;
	const float tx = F.t[0], ty = F.t[1], tz = F.t[2];
	const int comp = coop_component(lane);
	for (uint32_t i0 = 0; i0 < L.lig.n; i0 += kBeadsPerRound) {
		uint32_t nlk[2], nln[2];
		BeadGrid bg[2];
#pragma unroll
		for (int h = 0; h < 2; ++h) {
			const int s = lane + 32 * h;
			const uint32_t i = i0 + s;
			nlk[h] = 0;
			nln[h] = 0;
			bg[h] = BeadGrid{0u, 0u};
			if (i < L.lig.n) {
				const float4 b = __ldg(&L.lig.xyzq[i]);
				const uint32_t tm = __ldg(&L.lig.tm[i]);
				const uint32_t type = tm & 0xffffu, mapped = tm >> 16;
				float vw[4 * kModeWords<MM>];
				load_modes<MM>(L.lig_modes + (size_t)i * L.lig_ms, Ml, vw);
				float x = b.x, y = b.y, z = b.z;
				deform_w<MM>(vw, Ml, ampL, x, y, z);
				float px, py, pz;
				rot_apply(R.m, x, y, z, px, py, pz);
				px = fadd(px, tx); py = fadd(py, ty); pz = fadd(pz, tz);
				put_bead(W, s, b.x, b.y, b.z, px, py, pz, b.w, type);
				nlk[h] = stage_grid(L.grid_rec, px, py, pz, mapped, b.w, s, W, bg[h]);
				bool in_nl;
				if (type != 0) nln[h] = stage_nl(L.grid_rec.nl, px, py, pz, s, W, in_nl);
				/* the global-frame force f is projected in the ligand frame:
				 * (R^T f) . v = f . (R v) */
				if (nlk[h] | nln[h]) stage_modes<MM>(MS, s, vw, Ml, R.m, false);
			}
		}
		const uint32_t n_look = queue_lookups(W, nlk, bg, lane);
		uint32_t start[2];
		const uint32_t n_pair = queue_pairs(W, nln, lane, start);
		__syncwarp();
		if (L.grid_rec.coop_lookup) {
			for (uint32_t k0 = 0; k0 < n_look; k0 += 16) {
				CoopStep<2> st;
				st.load(L.grid_rec, W, k0, n_look, lane);
#pragma unroll
				for (int b = 0; b < 2; ++b) {
					const float v = st.component(b, lane);
					if (st.ok[b]) {
						const float f = fmul(v, st.sc[b]);
						C.f = fadd(C.f, f);
						if (comp != 3) {
							const float4 u = W.ut[st.sl[b]];
							C.t0 = ffma(u.x, f, C.t0);
							C.t1 = ffma(u.y, f, C.t1);
							C.t2 = ffma(u.z, f, C.t2);
							project_component<MM>(MS, st.sl[b], comp, Ml, f, gL);
						}
					}
				}
			}
		} else {
			for (uint32_t q = lane; q < n_look; q += 32) {
				const uint32_t s = lookup_slot(W, q);
				const float4 v = grid_lookup(L.grid_rec, W, q);
				const float4 u = W.ut[s];
				S.add(v.w, v.x, v.y, v.z, u.x, u.y, u.z);
				project_staged<MM>(MS, s, Ml, v.x, v.y, v.z, -1.f, gL);
			}
		}
		/* neighbour pairs after the lookups: measured faster here (the rigid
		 * kernel measured the opposite) */
		PairWindow win;
		for (uint32_t w = 0; w < n_pair; w += 64) {
			uint32_t so[2];
			win.owners(W, w, start, nln, lane, so[0], so[1]);
#pragma unroll
			for (int h = 0; h < 2; ++h) {
				const uint32_t q = w + 32 * h + lane;
				if (q >= n_pair) continue;
				const uint32_t s = so[h];
				const uint32_t j = __ldg(&L.grid_rec.nl.list[W.lbase[s] + q]);
				const float4 r = __ldg(&L.rec.xyzq[j]);
				float rx = r.x, ry = r.y, rz = r.z;
				float vw[4 * kModeWords<MM>];
				load_modes<MM>(L.rec_modes + (size_t)j * L.rec_ms, Mr, vw);
				deform_w<MM>(vw, Mr, ampR, rx, ry, rz);
				const uint32_t trec = __ldg(&L.rec.tm[j]) & 0xffffu;
				const float4 b = W.pq[s];
				const float4 u = W.ut[s];
				float fx, fy, fz, e;
				if (!nl_pair(L.grid_rec.nl, L.par, __float_as_uint(u.w), b.w, b.x, b.y, b.z, rx, ry, rz,
						r.w, trec, fx, fy, fz, e))
					continue;
				S.add(e, fx, fy, fz, u.x, u.y, u.z);
				/* reaction on receptor bead j is -f: its mode gradient gets -(-f . v) */
#pragma unroll
				for (int m = 0; m < MM; ++m)
					if (m < (int)Mr)
						gR[m] = ffma(1.f, ffma(fz, vw[3 * m + 2], ffma(fy, vw[3 * m + 1], fmul(fx, vw[3 * m]))), gR[m]);
				project_staged<MM>(MS, s, Ml, fx, fy, fz, -1.f, gL);
			}
		}
		__syncwarp();
	}
}

/* The Result_6D_Modes record from the ligand pass's sums and the two passes'
 * receptor-mode gradients (warp-summed, receptor pass first): warp sums,
 * correctModeForce (delta += 4 k delta^4, src/model/reduction_modes.h:101-115),
 * ForceLim, TorqueMat.  Lane k (k < 27) returns float k of the record. */
template <int MM>
__device__ __forceinline__ float modes_epilogue(const ModesLaunch& L, const ModesFrame& F, PoseSums& S,
		const CoopSums& C, float gL[MM], const float gR_rec[MM], float gR_nl[MM], const int lane) {
	const uint32_t Mr = L.rec.n_modes, Ml = L.lig.n_modes;
	fold_coop(C, S, lane);
	float sE = warp_sum(S.E), sFx = warp_sum(S.Fx), sFy = warp_sum(S.Fy), sFz = warp_sum(S.Fz);
	float T[9];
#pragma unroll
	for (int k = 0; k < 9; ++k) T[k] = warp_sum(S.T[k]);
	float gR[MM];
#pragma unroll
	for (int m = 0; m < MM; ++m) {
		gR[m] = 0.f;
		if (m < (int)Mr) gR[m] = fadd(gR_rec[m], warp_sum(gR_nl[m]));
		if (m < (int)Ml) gL[m] = warp_sum(gL[m]);
	}
	force_lim(sFx, sFy, sFz);
	float ang[3];
	torque_reduce(F.R, T, ang);
	/* correctModeForce: delta += (float)(4 k * delta^4) */
#pragma unroll
	for (int m = 0; m < MM; ++m) {
		if (m < (int)Mr) {
			const double dl = gR[m];
			gR[m] = fadd(gR[m], (float)__dmul_rn(__dmul_rn((double)fmul(4.0f, L.rec.mode_force[m]),
					__dmul_rn(dl, dl)), __dmul_rn(dl, dl)));
		}
		if (m < (int)Ml) {
			const double dl = gL[m];
			gL[m] = fadd(gL[m], (float)__dmul_rn(__dmul_rn((double)fmul(4.0f, L.lig.mode_force[m]),
					__dmul_rn(dl, dl)), __dmul_rn(dl, dl)));
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
	for (int m = 0; m < MM; ++m) {
		if (lane == 7 + m) v = m < (int)Mr ? gR[m] : 0.f;
		if (lane == 17 + m) v = m < (int)Ml ? gL[m] : 0.f;
	}
	return v;
}

/* Warp sums of the receptor pass's mode gradients (every lane). */
template <int MM>
__device__ __forceinline__ void sum_rec_modes(uint32_t Mr, float gR[MM]) {
#pragma unroll
	for (int m = 0; m < MM; ++m)
		if (m < (int)Mr) gR[m] = warp_sum(gR[m]);
}

/* One pose of the modes energy, both passes in one warp (the minimizer's
 * form).  Lane k (k < 26) brings the k-th float of the DOF_6D_Modes record;
 * returns on lane k (k < 27) the k-th float of the Result_6D_Modes record.
 * Only the model fields of L are read.  MM >= the receptor's and the
 * ligand's mode counts.  Bit for bit the result of the split scoring
 * kernels (modes_rec_kernel then modes_lig_kernel). */
template <int MM>
__device__ __forceinline__ float eval_pose_modes(const ModesLaunch& L, const float dv, const int lane,
		WarpStage& W, ModeStage<MM>& MS) {
	float ampR[MM], ampL[MM];
	const ModesFrame F = modes_frame<MM>(dv, lane, ampR, ampL, L.trig);
	float gRr[MM], gRn[MM], gL[MM];
#pragma unroll
	for (int m = 0; m < MM; ++m) { gRr[m] = 0.f; gRn[m] = 0.f; gL[m] = 0.f; }
	modes_rec_pass<MM>(L, F, ampR, lane, W, MS, gRr);
	sum_rec_modes<MM>(L.rec.n_modes, gRr);
	PoseSums S;
	CoopSums C;
	modes_lig_pass<MM>(L, F, ampR, ampL, lane, W, MS, S, C, gL, gRn);
	return modes_epilogue<MM>(L, F, S, C, gL, gRr, gRn, lane);
}

/* ---- the reference CPU path's order (GBA_KOPT_REFERENCE_ORDER) ----------
 *
 * CPUEnergyService6DModes evaluates a pose array by array
 * (src/service/CPUEnergyService6DModes.tpp:121-327): the receptor deformed
 * and moved into the ligand frame, its grid forces (ligand grid) rotated back
 * per bead; the ligand deformed and moved, its grid forces (receptor grid);
 * the NL term bead by bead in list order, adding each pair's four sub-terms
 * to the ligand bead and their reaction to the receptor bead; then sums in
 * bead order: energy and force, the ligand mode projections of R^T f, the
 * receptor mode projections, correctModeForce, the torque.  The rigid
 * reference order's pieces (ref_grid_term, ref_pair_terms, ref_fold,
 * ref_accumulate) follow it operation for operation; the receptor bead
 * forces need a per-pose array (scratch in global memory, one per warp,
 * float4 per receptor bead), and each receptor reaction is added to it in
 * the reference's pair order by three lanes, one per component. */

/* Receptor bead index of each window position (the reactions' scatter). */
struct RefModesExtra {
	uint32_t j[32];
};

/* x^4 correctly rounded, standing in for std::pow(x, 4) of
 * correctModeForce: x^2 = p + e and p^2 = hi + lo exactly (Dekker's
 * products through fma), x^4 = hi + (lo + 2 p e + e^2). */
__device__ __forceinline__ double pow4_rn(double x) {
	const double p = __dmul_rn(x, x);
	const double e = __fma_rn(x, x, -p);
	const double hi = __dmul_rn(p, p);
	const double lo = __fma_rn(p, p, -hi);
	return __dadd_rn(hi, __fma_rn(__dmul_rn(2.0, p), e, __fma_rn(e, e, lo)));
}

/* One pose in the reference's order; rf: this warp's receptor array.  Lane
 * k (k < 26) brings the k-th float of the DOF_6D_Modes record; returns on
 * lane k (k < 27) the k-th float of the Result_6D_Modes record. */
template <int MM>
__device__ __forceinline__ float eval_pose_modes_ref(const ModesLaunch& L, const float dv, const int lane,
		WarpStage& W, RefModesExtra& X, float4* __restrict__ rf) {
	const uint32_t Mr = L.rec.n_modes, Ml = L.lig.n_modes;
	const float tx = __shfl_sync(GBA_FULL_MASK, dv, 0);
	const float ty = __shfl_sync(GBA_FULL_MASK, dv, 1);
	const float tz = __shfl_sync(GBA_FULL_MASK, dv, 2);
	const float a0 = __shfl_sync(GBA_FULL_MASK, dv, 3);
	const float a1 = __shfl_sync(GBA_FULL_MASK, dv, 4);
	const float a2 = __shfl_sync(GBA_FULL_MASK, dv, 5);
	float ampR[MM], ampL[MM];
#pragma unroll
	for (int m = 0; m < MM; ++m) {
		ampR[m] = __shfl_sync(GBA_FULL_MASK, dv, 6 + m);
		ampL[m] = __shfl_sync(GBA_FULL_MASK, dv, 16 + m);
	}
	const PoseRot R0 = pose_rotation(a0, a1, a2, lane, L.trig);

	/* receptor: invertDOF (src/model/transform_modes.h:27-41) -- R(-ang)
	 * from the sin/cos of the negated angles, t' = R^T (-t) -- then per bead
	 * the ligand-grid force rotated back by R */
	{
		const PoseRot Rn = pose_rotation(-a0, -a1, -a2, lane, L.trig);
		const float ipx = fadd(fadd(fmul(R0.m[0], -tx), fmul(R0.m[3], -ty)), fmul(R0.m[6], -tz));
		const float ipy = fadd(fadd(fmul(R0.m[1], -tx), fmul(R0.m[4], -ty)), fmul(R0.m[7], -tz));
		const float ipz = fadd(fadd(fmul(R0.m[2], -tx), fmul(R0.m[5], -ty)), fmul(R0.m[8], -tz));
		for (uint32_t j0 = 0; j0 < L.rec.n; j0 += kBeadsPerRound) {
#pragma unroll
			for (int h = 0; h < 2; ++h) {
				const int s = lane + 32 * h;
				const uint32_t j = j0 + s;
				if (j >= L.rec.n) continue;
				const float4 r = __ldg(&L.rec.xyzq[j]);
				const uint32_t mapped = __ldg(&L.rec.tm[j]) >> 16;
				float x = r.x, y = r.y, z = r.z;
				deform<MM>(L.rec_modes + (size_t)j * L.rec_ms, Mr, ampR, x, y, z);
				float px, py, pz;
				rot_apply(Rn.m, x, y, z, px, py, pz);
				px = fadd(px, ipx); py = fadd(py, ipy); pz = fadd(pz, ipz);
				const float4 pot = ref_grid_term(L.grid_lig, px, py, pz, mapped, r.w, s, W);
				float fx, fy, fz;
				rot_apply(R0.m, pot.x, pot.y, pot.z, fx, fy, fz);
				rf[j] = make_float4(fx, fy, fz, 0.f);
			}
		}
	}
	__syncwarp();

	/* ligand: grid term, NL term with the receptor reactions, sums in bead
	 * order -- lanes 0..12 energy, force, torque; lanes 16 + m the ligand
	 * mode projections */
	const uint32_t* lst = L.grid_rec.nl.typed_list ? L.grid_rec.nl.typed_list : L.grid_rec.nl.list;
	const bool typed = L.grid_rec.nl.typed_list != nullptr;
	float acc = 0.f;
	for (uint32_t i0 = 0; i0 < L.lig.n; i0 += kBeadsPerRound) {
		float4 pot[2];
		uint32_t nln[2];
		bool in_nl[2];
#pragma unroll
		for (int h = 0; h < 2; ++h) {
			const int s = lane + 32 * h;
			const uint32_t i = i0 + s;
			pot[h] = make_float4(0.f, 0.f, 0.f, 0.f);
			nln[h] = 0;
			in_nl[h] = false;
			if (i >= L.lig.n) continue;
			const float4 b = __ldg(&L.lig.xyzq[i]);
			const uint32_t tm = __ldg(&L.lig.tm[i]);
			const uint32_t type = tm & 0xffffu, mapped = tm >> 16;
			float x = b.x, y = b.y, z = b.z;
			deform<MM>(L.lig_modes + (size_t)i * L.lig_ms, Ml, ampL, x, y, z);
			float px, py, pz;
			rot_apply(R0.m, x, y, z, px, py, pz);
			px = fadd(px, tx); py = fadd(py, ty); pz = fadd(pz, tz);
			put_bead(W, s, b.x, b.y, b.z, px, py, pz, b.w, type);
			pot[h] = ref_grid_term(L.grid_rec, px, py, pz, mapped, b.w, s, W);
			if (type != 0) nln[h] = stage_nl(L.grid_rec.nl, px, py, pz, s, W, in_nl[h]);
		}
		uint32_t start[2];
		const uint32_t n_pair = queue_pairs(W, nln, lane, start);
		__syncwarp();   /* weights read, list bases final: the overlay may be written */
		RefTerms& T = ref_terms(W);
		if (n_pair > 0) {
#pragma unroll
			for (int k = 0; k < 8; ++k) (&T.acc[0][0])[lane + 32 * k] = 0.f;
		}
		PairWindow win;
		for (uint32_t w = 0; w < n_pair; w += 64) {
			uint32_t sa, sb, ea = 0, eb = 0;
			win.owners(W, w, start, nln, lane, sa, sb);
			if (w + lane < n_pair) ea = __ldg(&lst[W.lbase[sa] + w + lane]);
			if (w + 32 + lane < n_pair) eb = __ldg(&lst[W.lbase[sb] + w + 32 + lane]);
#pragma unroll
			for (int half = 0; half < 2; ++half) {
				const uint32_t wb = w + 32 * half;
				if (wb >= n_pair) break;
				if (wb + lane < n_pair) {
					const uint32_t ent = half ? eb : ea;
					const uint32_t j = typed ? ent & 0xffffffu : ent;
					const uint32_t trec = typed ? ent >> 24 : __ldg(&L.rec.tm[j]) & 0xffffu;
					const float4 r = __ldg(&L.rec.xyzq[j]);
					float rx = r.x, ry = r.y, rz = r.z;
					deform<MM>(L.rec_modes + (size_t)j * L.rec_ms, Mr, ampR, rx, ry, rz);
					ref_pair_terms(L.grid_rec.nl, L.par, W, half ? sb : sa, make_float4(rx, ry, rz, r.w), trec,
							lane);
					X.j[lane] = j;
				}
				__syncwarp();
				const uint32_t n = min(n_pair - wb, 32u);
				ref_fold(T, n, half ? sb : sa, lane);
				/* each pair's reaction on its receptor bead (0 - LJ(r) + LJ(plateau)
				 * [- Coulomb(r) + Coulomb(plateau)]), added pair by pair */
				if (lane < 3) {
					for (uint32_t k = 0; k < n; ++k) {
						const uint32_t f = T.flags[k];
						if (!(f & 1u)) continue;
						const float* t = reinterpret_cast<const float*>(T.t[k]);
						float v = fsub(0.f, t[lane]);
						v = fadd(v, t[4 + lane]);
						if (f & 2u) {
							v = fsub(v, t[8 + lane]);
							v = fadd(v, t[12 + lane]);
						}
						float* d = reinterpret_cast<float*>(rf + X.j[k]) + lane;
						*d = fadd(*d, v);
					}
				}
				__syncwarp();
			}
		}
		float4 a[2];
#pragma unroll
		for (int h = 0; h < 2; ++h) {
			const int s = lane + 32 * h;
			a[h] = n_pair > 0 ? make_float4(T.acc[s][0], T.acc[s][1], T.acc[s][2], T.acc[s][3])
			                  : make_float4(0.f, 0.f, 0.f, 0.f);
		}
		__syncwarp();   /* accumulators read: the totals may overwrite them */
#pragma unroll
		for (int h = 0; h < 2; ++h) {
			const int s = lane + 32 * h;
			if (i0 + s >= L.lig.n) continue;
			float4 v = pot[h];
			if (in_nl[h]) {
				v.x = fadd(v.x, a[h].x); v.y = fadd(v.y, a[h].y); v.z = fadd(v.z, a[h].z); v.w = fadd(v.w, a[h].w);
			}
			float* cw = W.cw + kCornerStride * s;
			cw[0] = v.x; cw[1] = v.y; cw[2] = v.z; cw[3] = v.w;
		}
		__syncwarp();
		const uint32_t nb = min((uint32_t)kBeadsPerRound, L.lig.n - i0);
		acc = ref_accumulate(W, nb, lane, acc);
		if (lane >= 16 && (uint32_t)(lane - 16) < Ml) {
			/* reduceModeForce with rotation (src/model/reduction_modes.h:29-57):
			 * -= (R^T f) . v */
			const int m = lane - 16;
			for (uint32_t s = 0; s < nb; ++s) {
				const float* f = W.cw + kCornerStride * s;
				float ox, oy, oz;
				rot_apply_t(R0.m, f[0], f[1], f[2], ox, oy, oz);
				const float* v = L.lig_modes + (size_t)(i0 + s) * L.lig_ms + 3 * m;
				acc = fsub(acc, fadd(fadd(fmul(ox, __ldg(v)), fmul(oy, __ldg(v + 1))), fmul(oz, __ldg(v + 2))));
			}
		}
		__syncwarp();
	}
	float c[13];
#pragma unroll
	for (int k = 0; k < 13; ++k) c[k] = __shfl_sync(GBA_FULL_MASK, acc, k);
	float gL[MM], gR[MM];
#pragma unroll
	for (int m = 0; m < MM; ++m) gL[m] = __shfl_sync(GBA_FULL_MASK, acc, 16 + m);
	/* reduceModeForce without rotation over the receptor forces, bead order */
	float g = 0.f;
	if ((uint32_t)lane < Mr) {
		for (uint32_t j = 0; j < L.rec.n; ++j) {
			const float4 f = rf[j];
			const float* v = L.rec_modes + (size_t)j * L.rec_ms + 3 * lane;
			g = fsub(g, fadd(fadd(fmul(f.x, __ldg(v)), fmul(f.y, __ldg(v + 1))), fmul(f.z, __ldg(v + 2))));
		}
	}
#pragma unroll
	for (int m = 0; m < MM; ++m) gR[m] = __shfl_sync(GBA_FULL_MASK, g, m);
	__syncwarp();   /* rf read: the next pose may overwrite it */
	float sFx = c[1], sFy = c[2], sFz = c[3];
	force_lim(sFx, sFy, sFz);
	float ang[3];
	torque_reduce(R0, c + 4, ang);
	/* correctModeForce (src/model/reduction_modes.h:101-115):
	 * delta + (float)((double)(4 k) * pow(delta, 4)) */
#pragma unroll
	for (int m = 0; m < MM; ++m) {
		if (m < (int)Mr)
			gR[m] = fadd(gR[m], (float)__dmul_rn((double)fmul(4.0f, L.rec.mode_force[m]), pow4_rn((double)gR[m])));
		if (m < (int)Ml)
			gL[m] = fadd(gL[m], (float)__dmul_rn((double)fmul(4.0f, L.lig.mode_force[m]), pow4_rn((double)gL[m])));
	}
	float v = 0.f;
	if (lane == 0) v = c[0];
	else if (lane == 1) v = sFx;
	else if (lane == 2) v = sFy;
	else if (lane == 3) v = sFz;
	else if (lane == 4) v = ang[0];
	else if (lane == 5) v = ang[1];
	else if (lane == 6) v = ang[2];
#pragma unroll
	for (int m = 0; m < MM; ++m) {
		if (lane == 7 + m) v = m < (int)Mr ? gR[m] : 0.f;
		if (lane == 17 + m) v = m < (int)Ml ? gL[m] : 0.f;
	}
	return v;
}

namespace {

constexpr int kModesThreads = 256;       /* ligand-pass scoring kernel's block */
constexpr int kModesRecThreads = 128;    /* receptor-pass kernel: block, */
constexpr int kModesRecBlocks = 5;       /* resident blocks per SM (shared memory allows five) */
constexpr int kModesMinThreads = 128;    /* minimizer kernel block */
constexpr int kModesRefThreads = 128;    /* reference-order scoring kernel block */

/* mode capacity compiled for a launch: 5 or GBA_MODES_MAX */
int mode_capacity(const ModesLaunch& L) {
	return (L.rec.n_modes <= 5 && L.lig.n_modes <= 5) ? 5 : GBA_MODES_MAX;
}

}  // namespace

extern __shared__ float4 modes_dyn_smem[];

/* Scoring in two kernels, so that each runs at the occupancy its own
 * registers allow: the receptor pass (most of the grid lookups) parks its
 * warp-summed receptor-mode gradients in the result record's modesRec slots;
 * the ligand pass reads them back, adds its own and writes the record. */
template <int MM>
__global__ void __launch_bounds__(kModesRecThreads, kModesRecBlocks) modes_rec_kernel(const ModesLaunch L) {
	__shared__ WarpStage stage[kModesRecThreads / 32];
	ModeStage<MM>* ms = reinterpret_cast<ModeStage<MM>*>(modes_dyn_smem);
	const int lane = threadIdx.x & 31;
	const int wib = threadIdx.x >> 5;
	const uint32_t Mr = L.rec.n_modes;
	PoseFeed feed(L.next);
	for (size_t p = feed.take(lane); p < L.n; p = feed.take(lane)) {
		const float* d = reinterpret_cast<const float*>(L.dofs + p);
		const float dv = lane < 26 ? __ldg(d + lane) : 0.f;
		float ampR[MM], ampL[MM];
		const ModesFrame F = modes_frame<MM>(dv, lane, ampR, ampL, L.trig);
		float gR[MM];
#pragma unroll
		for (int m = 0; m < MM; ++m) gR[m] = 0.f;
		modes_rec_pass<MM>(L, F, ampR, lane, stage[wib], ms[wib], gR);
		sum_rec_modes<MM>(Mr, gR);
		float v = 0.f;
#pragma unroll
		for (int m = 0; m < MM; ++m) v = lane == m ? gR[m] : v;
		if ((uint32_t)lane < Mr) reinterpret_cast<float*>(L.out + p)[7 + lane] = v;
	}
}

template <int MM>
__global__ void __launch_bounds__(kModesThreads, 2) modes_lig_kernel(const ModesLaunch L) {
	__shared__ WarpStage stage[kModesThreads / 32];
	ModeStage<MM>* ms = reinterpret_cast<ModeStage<MM>*>(modes_dyn_smem);
	const int lane = threadIdx.x & 31;
	const int wib = threadIdx.x >> 5;
	const uint32_t Mr = L.rec.n_modes;
	PoseFeed feed(L.next2);
	for (size_t p = feed.take(lane); p < L.n; p = feed.take(lane)) {
		const float* d = reinterpret_cast<const float*>(L.dofs + p);
		const float dv = lane < 26 ? __ldg(d + lane) : 0.f;
		float ampR[MM], ampL[MM];
		const ModesFrame F = modes_frame<MM>(dv, lane, ampR, ampL, L.trig);
		float gRr[MM], gRn[MM], gL[MM];
		const float* o = reinterpret_cast<const float*>(L.out + p);
#pragma unroll
		for (int m = 0; m < MM; ++m) {
			gRr[m] = m < (int)Mr ? o[7 + m] : 0.f;
			gRn[m] = 0.f;
			gL[m] = 0.f;
		}
		__syncwarp();
		PoseSums S;
		CoopSums C;
		modes_lig_pass<MM>(L, F, ampR, ampL, lane, stage[wib], ms[wib], S, C, gL, gRn);
		const float v = modes_epilogue<MM>(L, F, S, C, gL, gRr, gRn, lane);
		if (lane < 27) reinterpret_cast<float*>(L.out + p)[lane] = v;
	}
}

/* GBA_KOPT_REFERENCE_ORDER scoring: a warp takes whole poses
 * (eval_pose_modes_ref) with its own receptor array in L.ref_rf. */
template <int MM>
__global__ void __launch_bounds__(kModesRefThreads) modes_ref_kernel(const ModesLaunch L) {
	__shared__ WarpStage stage[kModesRefThreads / 32];
	__shared__ RefModesExtra extra[kModesRefThreads / 32];
	const int lane = threadIdx.x & 31;
	const int wib = threadIdx.x >> 5;
	float4* rf = L.ref_rf + (((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * L.rec.n;
	PoseFeed feed(L.next);
	for (size_t p = feed.take(lane); p < L.n; p = feed.take(lane)) {
		const float* d = reinterpret_cast<const float*>(L.dofs + p);
		const float dv = lane < 26 ? __ldg(d + lane) : 0.f;
		const float v = eval_pose_modes_ref<MM>(L, dv, lane, stage[wib], extra[wib], rf);
		if (lane < 27) reinterpret_cast<float*>(L.out + p)[lane] = v;
	}
}

/* Persistent VA13 over (ang xyz, pos xyz, modesRec[0..Mr), modesLig[0..Ml)):
 * the minimizer of minimize.cu generalised to 6 + Mr + Ml DOF (minfor.f is
 * fixed at 6, src/apps/em/minfor.f:16,33). */
__device__ __forceinline__ unsigned long long modes_global_ns() {
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

template <int MM, bool REF>
__global__ void __launch_bounds__(kModesMinThreads) minimize_modes_kernel(const ModesMinLaunch M) {
	__shared__ WarpStage stage[kModesMinThreads / 32];
	ModeStage<MM>* ms = reinterpret_cast<ModeStage<MM>*>(modes_dyn_smem);
	/* per warp, after the mode staging areas: its pose's VA13 state, which
	 * every lane of the warp steps (the warp form) */
	static_assert(sizeof(ModeStage<MM>) % 16 == 0, "VA13 states follow the staging areas");
	VA13<6 + 2 * MM>* vas = reinterpret_cast<VA13<6 + 2 * MM>*>(ms + kModesMinThreads / 32);
	const int lane = threadIdx.x & 31;
	const int wib = threadIdx.x >> 5;
	const ModesLaunch& L = M.m;
	const uint32_t Mr = L.rec.n_modes, Ml = L.lig.n_modes;
	const int jn = 6 + (int)Mr + (int)Ml;
	unsigned long long t_start = 0;
	if (lane == 0) t_start = modes_global_ns();
	t_start = __shfl_sync(GBA_FULL_MASK, t_start, 0);
	/* lane 0 reads the clock, the warp decides together */
	auto over_cap = [&]() {
		int over = 0;
		if (lane == 0) over = modes_global_ns() - t_start > kMinimizeHardCapNs;
		return __shfl_sync(GBA_FULL_MASK, over, 0) != 0;
	};
	for (;;) {
		unsigned long long slot = 0;
		if (lane == 0) slot = atomicAdd(M.counter, 1ull);
		slot = __shfl_sync(GBA_FULL_MASK, slot, 0);
		if (slot >= M.n) break;
		if (over_cap()) {
			if (lane == 0) atomicExch(M.status, GBA_ERR_TIMEOUT);
			break;
		}
		const size_t p = (size_t)slot;
		VA13<6 + 2 * MM>& va = vas[wib];
		/* lane k holds DOF float k (pos, ang, modesRec[10], modesLig[10]) */
		float dv = lane < 26 ? __ldg(reinterpret_cast<const float*>(M.start + p) + lane) : 0.f;
		if (lane == 0) {
			double x0[6 + 2 * MM];
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
			if (REF)
				v = eval_pose_modes_ref<MM>(L, dv, lane, stage[wib], *reinterpret_cast<RefModesExtra*>(&ms[wib]),
						L.ref_rf + (((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * L.rec.n);
			else
				v = eval_pose_modes<MM>(L, dv, lane, stage[wib], ms[wib]);
			++nev;
			/* lane j takes gradient element j from the lane holding its entry
			 * of the result record: -(ang), -(pos), then the mode entries,
			 * which are gradients already (reduceModeForce) */
			const int k = lane - 1;
			int src = 0;
			bool neg = false;
			if (lane >= 1 && lane <= jn) {
				if (k < 3) { src = 4 + k; neg = true; }
				else if (k < 6) { src = k - 2; neg = true; }
				else if (k < 6 + (int)Mr) src = 7 + (k - 6);
				else src = 17 + (k - 6 - (int)Mr);
			}
			const float gv = __shfl_sync(GBA_FULL_MASK, v, src);
			const double gl = neg ? -(double)gv : (double)gv;
			const float e = __shfl_sync(GBA_FULL_MASK, v, 0);
			va.provide_w((double)e, [&](int) { return gl; }, VaWarp{lane});
			/* lane 0's reading for all: no lane may see a state that lane 0,
			 * gone on to the next pose, has already restarted */
			if (__shfl_sync(GBA_FULL_MASK, (int)va.done(), 0)) break;
			if (nev > M.max_evals + 1) {
				if (lane == 0) atomicExch(M.status, GBA_ERR_DEVICE_CHECK);
				break;
			}
			if ((nev & 15) == 0 && over_cap()) {
				if (lane == 0) atomicExch(M.status, GBA_ERR_TIMEOUT);
				break;
			}
		}
		if (lane < 27) reinterpret_cast<float*>(M.out_result + p)[lane] = v;
		if (lane < 26) reinterpret_cast<float*>(M.out_state + p)[lane] = dv;
		if (lane == 0 && M.out_nevals) M.out_nevals[p] = nev;
	}
}

namespace {

template <int MM>
size_t mode_stage_bytes(int threads) {
	return (size_t)(threads / 32) * sizeof(ModeStage<MM>);
}

/* dynamic shared memory beyond the 48 KB default needs the opt-in */
template <class K>
cudaError_t allow_smem(K kernel, size_t dyn) {
	return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
}

template <class K>
int resident_blocks(K kernel, int threads, size_t dyn) {
	if (allow_smem(kernel, dyn) != cudaSuccess) return 1;
	int nb = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, dyn);
	return nb > 0 ? nb : 1;
}

template <int MM>
cudaError_t launch_modes_mm(const ModesLaunch& L, int num_sms, cudaStream_t s) {
	const size_t dyn_r = mode_stage_bytes<MM>(kModesRecThreads);
	const size_t want_r = (L.n + kModesRecThreads / 32 - 1) / (kModesRecThreads / 32);
	const size_t br = std::max<size_t>(1, std::min<size_t>(want_r,
			(size_t)num_sms * resident_blocks(modes_rec_kernel<MM>, kModesRecThreads, dyn_r)));
	modes_rec_kernel<MM><<<(unsigned)br, kModesRecThreads, dyn_r, s>>>(L);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	const size_t dyn = mode_stage_bytes<MM>(kModesThreads);
	const size_t want = (L.n + kModesThreads / 32 - 1) / (kModesThreads / 32);
	const size_t bl = std::max<size_t>(1, std::min<size_t>(want,
			(size_t)num_sms * resident_blocks(modes_lig_kernel<MM>, kModesThreads, dyn)));
	modes_lig_kernel<MM><<<(unsigned)bl, kModesThreads, dyn, s>>>(L);
	return cudaGetLastError();
}

template <int MM>
size_t ref_blocks_mm(const ModesLaunch& L, int num_sms) {
	const size_t want = (L.n + kModesRefThreads / 32 - 1) / (kModesRefThreads / 32);
	return std::max<size_t>(1, std::min<size_t>(want,
			(size_t)num_sms * resident_blocks(modes_ref_kernel<MM>, kModesRefThreads, 0)));
}

template <int MM>
cudaError_t launch_ref_mm(const ModesLaunch& L, int num_sms, cudaStream_t s) {
	modes_ref_kernel<MM><<<(unsigned)ref_blocks_mm<MM>(L, num_sms), kModesRefThreads, 0, s>>>(L);
	return cudaGetLastError();
}

/* the minimizer's: staging areas and VA13 states, one each per warp */
template <int MM>
size_t min_modes_bytes(int threads) {
	return (size_t)(threads / 32) * (sizeof(ModeStage<MM>) + sizeof(VA13<6 + 2 * MM>));
}

template <int MM, bool REF>
cudaError_t launch_min_mm(const ModesMinLaunch& M, int blocks, int threads, cudaStream_t s) {
	const size_t dyn = min_modes_bytes<MM>(threads);
	cudaError_t e = allow_smem(minimize_modes_kernel<MM, REF>, dyn);
	if (e != cudaSuccess) return e;
	minimize_modes_kernel<MM, REF><<<blocks, threads, dyn, s>>>(M);
	return cudaGetLastError();
}

template <int MM, bool REF>
int min_bps_mm(int threads) {
	const size_t dyn = min_modes_bytes<MM>(threads);
	if (allow_smem(minimize_modes_kernel<MM, REF>, dyn) != cudaSuccess) return 1;
	int nb = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, minimize_modes_kernel<MM, REF>, threads, dyn);
	return nb > 0 ? nb : 1;
}

}  // namespace

cudaError_t launch_modes_energy(const ModesLaunch& L, int num_sms, cudaStream_t s) {
	if (L.ref_order) {
		if (!L.ref_rf) return cudaErrorInvalidValue;
		return mode_capacity(L) == 5 ? launch_ref_mm<5>(L, num_sms, s) : launch_ref_mm<GBA_MODES_MAX>(L, num_sms, s);
	}
	return mode_capacity(L) == 5 ? launch_modes_mm<5>(L, num_sms, s)
	                             : launch_modes_mm<GBA_MODES_MAX>(L, num_sms, s);
}

size_t modes_ref_warps(const ModesLaunch& L, int num_sms) {
	const size_t blocks = mode_capacity(L) == 5 ? ref_blocks_mm<5>(L, num_sms)
	                                            : ref_blocks_mm<GBA_MODES_MAX>(L, num_sms);
	return blocks * (kModesRefThreads / 32);
}

cudaError_t launch_minimize_modes(const ModesMinLaunch& M, int blocks, int threads, cudaStream_t s) {
	if (threads != kModesMinThreads || (M.m.ref_order && !M.m.ref_rf)) return cudaErrorInvalidValue;
	if (M.m.ref_order)
		return mode_capacity(M.m) == 5 ? launch_min_mm<5, true>(M, blocks, threads, s)
		                               : launch_min_mm<GBA_MODES_MAX, true>(M, blocks, threads, s);
	return mode_capacity(M.m) == 5 ? launch_min_mm<5, false>(M, blocks, threads, s)
	                               : launch_min_mm<GBA_MODES_MAX, false>(M, blocks, threads, s);
}

int minimize_modes_blocks_per_sm(int threads, const ModesLaunch& L) {
	if (L.ref_order)
		return mode_capacity(L) == 5 ? min_bps_mm<5, true>(threads) : min_bps_mm<GBA_MODES_MAX, true>(threads);
	return mode_capacity(L) == 5 ? min_bps_mm<5, false>(threads) : min_bps_mm<GBA_MODES_MAX, false>(threads);
}

}  // namespace gba
