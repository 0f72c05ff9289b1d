/*
 * rigid_pose.cuh -- one warp evaluates one rigid pose.
 *
 * Shared by the scoring kernel (energy_rigid.cu), the multi-pair kernel and
 * the persistent minimizer (minimize.cu).  The per-bead work of the reference
 * -- transform (src/model/transform.h:22-44), inner/outer grid term
 * (src/model/interpolation.h:57-101) and neighbour-list term
 * (src/model/neighborlist.h:29-168) -- is reorganised for the SIMT machine:
 *
 *   1. lane-per-bead, 64 beads per round (two per lane): rotate/translate,
 *      bounds tests, voxel indices and trilinear weights, NL voxel lookup;
 *      the bead's geometry goes to per-warp shared memory and each bead
 *      enqueues one grid lookup per channel it reads (type, and charge when
 *      |q| > 0.001) and its NL list length;
 *   2. the warp drains the lookup queue, one lookup per lane (8 gathered
 *      float4 corners, trilinear sum);
 *   3. the warp drains the flattened (bead, neighbour) pair list, one pair
 *      per lane (owner found by binary search over the 64 prefix sums).
 * Every lookup and pair contributes straight to the pose sums: energy,
 * force and the torque matrix sum_i x_i (x) f_i are linear in the bead
 * forces, so no per-bead force is kept.  The warp then reduces with
 * shuffles (reducePotForce / reduceTorque, src/model/reduction.h:40-103) and
 * every lane ends with the 7 result values.
 */
#ifndef GBA_RIGID_POSE_CUH_
#define GBA_RIGID_POSE_CUH_

#include "energy_dev.cuh"

namespace gba {

constexpr int kBeadsPerRound = 64;

/* Per-warp staging of one round of beads (SoA, bank-conflict free). */
struct WarpStage {
	float ux[kBeadsPerRound], uy[kBeadsPerRound], uz[kBeadsPerRound];   /* unrotated (torque) */
	float px[kBeadsPerRound], py[kBeadsPerRound], pz[kBeadsPerRound];   /* transformed */
	float q[kBeadsPerRound];
	float wnx[kBeadsPerRound], wny[kBeadsPerRound], wnz[kBeadsPerRound]; /* pos - voxel min */
	float wxx[kBeadsPerRound], wxy[kBeadsPerRound], wxz[kBeadsPerRound]; /* voxel max - pos */
	uint32_t off[kBeadsPerRound];      /* octet offset inside a channel */
	uint32_t chan[kBeadsPerRound];     /* mapped channel | outer grid flag << 31 */
	uint32_t type[kBeadsPerRound];     /* raw type (NL parameters) */
	uint32_t nl_idx[kBeadsPerRound];   /* list start */
	uint32_t nl_pre[kBeadsPerRound + 1];  /* exclusive prefix of list lengths */
	uint8_t look[2 * kBeadsPerRound];  /* lookup queue: bead << 1 | is_charge */
};

struct RigidRecPos {
	const float4* __restrict__ xyzq;
	__device__ __forceinline__ void operator()(uint32_t j, float& x, float& y, float& z, float& q) const {
		const float4 r = __ldg(&xyzq[j]);
		x = r.x; y = r.y; z = r.z; q = r.w;
	}
};

/* Inclusive warp scan of v. */
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const uint32_t t = __shfl_up_sync(GBA_FULL_MASK, v, o);
		if (lane >= o) v += t;
	}
	return v;
}

/* Stage bead i (or an empty slot when i >= n) into slot s; returns the
 * number of grid lookups (0..2) and the NL list length of the bead. */
__device__ __forceinline__ void stage_bead(const RigidModel& M, const PoseRot& R, float tx,
		float ty, float tz, uint32_t i, int s, WarpStage& W, uint32_t& nlook, uint32_t& nlen,
		bool& in_nl) {
	nlook = 0;
	nlen = 0;
	in_nl = false;
	if (i >= M.lig.n) return;
	const float4 b = __ldg(&M.lig.xyzq[i]);
	const uint32_t tm = __ldg(&M.lig.tm[i]);
	const uint32_t type = tm & 0xffffu, mapped = tm >> 16;
	float px, py, pz;
	rot_apply(R.m, b.x, b.y, b.z, px, py, pz);
	px = fadd(px, tx); py = fadd(py, ty); pz = fadd(pz, tz);
	W.ux[s] = b.x; W.uy[s] = b.y; W.uz[s] = b.z;
	W.px[s] = px; W.py[s] = py; W.pz[s] = pz;
	W.q[s] = b.w;
	W.type[s] = type;
	/* potForce's grid selection, src/model/interpolation.h:66-76 */
	if (mapped != 0) {
		const bool inner = !grid_out(M.grid.inner, px, py, pz);
		const bool outer = !inner && !grid_out(M.grid.outer, px, py, pz);
		if (inner | outer) {
			const DevIntrpl& g = inner ? M.grid.inner : M.grid.outer;
			/* getIndex / getVoxelByIndex, src/model/IntrplGrid.h:96-104,130-163 */
			const uint32_t ix = min((uint32_t)floorf(fmul(fsub(px, g.pos[0]), g.dVox_inv)), g.dimN[0] - 2);
			const uint32_t iy = min((uint32_t)floorf(fmul(fsub(py, g.pos[1]), g.dVox_inv)), g.dimN[1] - 2);
			const uint32_t iz = min((uint32_t)floorf(fmul(fsub(pz, g.pos[2]), g.dVox_inv)), g.dimN[2] - 2);
			const float minx = fadd(fmul((float)ix, g.dVox), g.pos[0]);
			const float miny = fadd(fmul((float)iy, g.dVox), g.pos[1]);
			const float minz = fadd(fmul((float)iz, g.dVox), g.pos[2]);
			W.wnx[s] = fsub(px, minx); W.wny[s] = fsub(py, miny); W.wnz[s] = fsub(pz, minz);
			W.wxx[s] = fsub(fadd(minx, g.dVox), px);
			W.wxy[s] = fsub(fadd(miny, g.dVox), py);
			W.wxz[s] = fsub(fadd(minz, g.dVox), pz);
			W.off[s] = g.oct ? (g.dimN[0] - 1) * (iz * (g.dimN[1] - 1) + iy) + ix
			                 : g.dimN[0] * (iz * g.dimN[1] + iy) + ix;
			W.chan[s] = mapped | (outer ? 0x80000000u : 0u);
			nlook = fabsf(b.w) > 0.001f ? 2u : 1u;
		}
	}
	/* NLPotForce's voxel lookup, src/model/neighborlist.h:59-66 */
	if (type != 0 && !nl_out(M.grid.nl, px, py, pz)) {
		const DevNL& nl = M.grid.nl;
		const int ix = min(max((int)roundf(fmul(fsub(px, nl.pos[0]), nl.dVox_inv)), 0), (int)nl.dimN[0] - 1);
		const int iy = min(max((int)roundf(fmul(fsub(py, nl.pos[1]), nl.dVox_inv)), 0), (int)nl.dimN[1] - 1);
		const int iz = min(max((int)roundf(fmul(fsub(pz, nl.pos[2]), nl.dVox_inv)), 0), (int)nl.dimN[2] - 1);
		const uint2 d = __ldg(&nl.grid[nl.dimN[0] * (iz * nl.dimN[1] + iy) + ix]);
		W.nl_idx[s] = d.y;
		nlen = d.x;
		in_nl = true;
	}
}

/* Grid bookkeeping of a staged bead at position (px, py, pz): picks inner or
 * outer grid, stores octet offset and trilinear weights in slot s and returns
 * the number of lookups (0, 1, or 2 with the charge channel). */
__device__ __forceinline__ uint32_t stage_grid(const DevGrid& G, float px, float py, float pz,
		uint32_t mapped, float q, int s, WarpStage& W) {
	if (mapped == 0) return 0;
	const bool inner = !grid_out(G.inner, px, py, pz);
	const bool outer = !inner && !grid_out(G.outer, px, py, pz);
	if (!(inner | outer)) return 0;
	const DevIntrpl& g = inner ? G.inner : G.outer;
	const uint32_t ix = min((uint32_t)floorf(fmul(fsub(px, g.pos[0]), g.dVox_inv)), g.dimN[0] - 2);
	const uint32_t iy = min((uint32_t)floorf(fmul(fsub(py, g.pos[1]), g.dVox_inv)), g.dimN[1] - 2);
	const uint32_t iz = min((uint32_t)floorf(fmul(fsub(pz, g.pos[2]), g.dVox_inv)), g.dimN[2] - 2);
	const float minx = fadd(fmul((float)ix, g.dVox), g.pos[0]);
	const float miny = fadd(fmul((float)iy, g.dVox), g.pos[1]);
	const float minz = fadd(fmul((float)iz, g.dVox), g.pos[2]);
	W.wnx[s] = fsub(px, minx); W.wny[s] = fsub(py, miny); W.wnz[s] = fsub(pz, minz);
	W.wxx[s] = fsub(fadd(minx, g.dVox), px);
	W.wxy[s] = fsub(fadd(miny, g.dVox), py);
	W.wxz[s] = fsub(fadd(minz, g.dVox), pz);
	W.off[s] = g.oct ? (g.dimN[0] - 1) * (iz * (g.dimN[1] - 1) + iy) + ix
	                 : g.dimN[0] * (iz * g.dimN[1] + iy) + ix;
	W.chan[s] = mapped | (outer ? 0x80000000u : 0u);
	return fabsf(q) > 0.001f ? 2u : 1u;
}

/* One queued lookup: the channel's interpolated (fx, fy, fz, E), scaled by
 * 1/voxelVol and, for the charge channel, by the bead charge. */
__device__ __forceinline__ float4 grid_lookup(const DevGrid& G, const WarpStage& W, uint32_t e) {
	const uint32_t s = e >> 1;
	const bool is_q = e & 1u;
	const uint32_t ch = W.chan[s];
	const DevIntrpl& g = (ch & 0x80000000u) ? G.outer : G.inner;
	const uint32_t c = is_q ? 0u : (ch & 0x7fffffffu);
	float4 v;
	if (g.oct) {
		const size_t nocts = (size_t)(g.dimN[0] - 1) * (g.dimN[1] - 1) * (g.dimN[2] - 1);
		v = octet_lerp(g.oct + 8 * ((size_t)c * nocts + W.off[s]), 2, 4, W.wnx[s], W.wny[s], W.wnz[s],
				W.wxx[s], W.wxy[s], W.wxz[s]);
	} else {
		const uint32_t sx = g.dimN[0], sxy = g.dimN[0] * g.dimN[1];
		v = octet_lerp(g.data + (size_t)c * (sxy * g.dimN[2]) + W.off[s], sx, sxy, W.wnx[s], W.wny[s],
				W.wnz[s], W.wxx[s], W.wxy[s], W.wxz[s]);
	}
	const float sc = is_q ? g.voxelVol_inv * W.q[s] : g.voxelVol_inv;
	v.x *= sc; v.y *= sc; v.z *= sc; v.w *= sc;
	return v;
}

/* Writes the lookup queue entries of slot s (n = 0..2) at position k. */
__device__ __forceinline__ void enqueue_lookups(WarpStage& W, uint32_t& k, int s, uint32_t n) {
	if (n > 0) W.look[k++] = (uint8_t)(s << 1);
	if (n > 1) W.look[k++] = (uint8_t)((s << 1) | 1);
}

/* Owner slot of flattened pair k: the last s with nl_pre[s] <= k. */
__device__ __forceinline__ uint32_t pair_owner(const WarpStage& W, uint32_t k) {
	uint32_t lo = 0, hi = kBeadsPerRound;
#pragma unroll
	for (int it = 0; it < 6; ++it) {
		const uint32_t mid = (lo + hi) >> 1;
		if (W.nl_pre[mid] <= k) lo = mid; else hi = mid;
	}
	return lo;
}

/* NL voxel lookup of a staged bead (type != 0), NLPotForce's
 * src/model/neighborlist.h:59-66; returns the list length (0 outside). */
__device__ __forceinline__ uint32_t stage_nl(const DevNL& nl, float px, float py, float pz, int s,
		WarpStage& W, bool& in_nl) {
	in_nl = false;
	if (nl_out(nl, px, py, pz)) return 0;
	const int ix = min(max((int)roundf(fmul(fsub(px, nl.pos[0]), nl.dVox_inv)), 0), (int)nl.dimN[0] - 1);
	const int iy = min(max((int)roundf(fmul(fsub(py, nl.pos[1]), nl.dVox_inv)), 0), (int)nl.dimN[1] - 1);
	const int iz = min(max((int)roundf(fmul(fsub(pz, nl.pos[2]), nl.dVox_inv)), 0), (int)nl.dimN[2] - 1);
	const uint2 d = __ldg(&nl.grid[nl.dimN[0] * (iz * nl.dimN[1] + iy) + ix]);
	W.nl_idx[s] = d.y;
	in_nl = true;
	return d.x;
}

/* Accumulates f into the pose sums with the bead's unrotated coordinates. */
struct PoseSums {
	float E = 0.f, Fx = 0.f, Fy = 0.f, Fz = 0.f;
	float T[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
	__device__ __forceinline__ void add(float e, float fx, float fy, float fz, float ux, float uy,
			float uz) {
		E += e; Fx += fx; Fy += fy; Fz += fz;
		T[0] += ux * fx; T[1] += uy * fx; T[2] += uz * fx;
		T[3] += ux * fy; T[4] += uy * fy; T[5] += uz * fy;
		T[6] += ux * fz; T[7] += uy * fz; T[8] += uz * fz;
	}
};

/* One NL pair term (plateau-subtracted LJ + Coulomb), the body of the
 * neighbour loop of src/model/neighborlist.h:70-158.  Returns false when
 * the pair lies outside the plateau. */
__device__ __forceinline__ bool nl_pair(const DevNL& nl, const DevParams& P, uint32_t lig_type,
		float qlig, float px, float py, float pz, float rx, float ry, float rz, float rq,
		uint32_t trec, float& fx, float& fy, float& fz, float& e) {
	float dx = fsub(px, rx), dy = fsub(py, ry), dz = fsub(pz, rz);
	const float dr2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
	if (!(dr2 <= nl.dPlateau2) || trec == 0) return false;
	const float dr2_inv = __frcp_rn(dr2);
	dx *= dr2_inv; dy *= dr2_inv; dz *= dr2_inv;
	const bool shape86 = P.potshape == GBA_POTSHAPE_8_6;
	const size_t k = (size_t)P.num_types * (trec - 1) + (lig_type - 1);
	const float4 p = __ldg(&P.lj[k]);
	const float iv = __ldg(&P.ivor[k]);
	float f1x, f1y, f1z, e1;
	lj_pot_force(dr2, dr2_inv, dx, dy, dz, p, iv, shape86, f1x, f1y, f1z, e1);
	const float ratio = __ldg(&nl.ratio[(int)fmul(dr2, 10000.0f)]);
	const float rdx = ratio * dx, rdy = ratio * dy, rdz = ratio * dz;
	float f2x, f2y, f2z, e2;
	lj_pot_force(nl.dPlateau2, nl.dPlateau2_inv, rdx, rdy, rdz, p, iv, shape86, f2x, f2y, f2z, e2);
	fx = f1x - f2x; fy = f1y - f2y; fz = f1z - f2z; e = e1 - e2;
	const float qq = fmul(fmul(qlig, rq), P.ffelec);
	if (fabsf(qq) > 0.001f) {
		const bool cdiel = P.dielec == GBA_DIELEC_CONSTANT;
		float c1x, c1y, c1z, c1e, c2x, c2y, c2z, c2e;
		charge_pot_force(dr2_inv, dx, dy, dz, qq, cdiel, c1x, c1y, c1z, c1e);
		charge_pot_force(nl.dPlateau2_inv, rdx, rdy, rdz, qq, cdiel, c2x, c2y, c2z, c2e);
		fx += c1x - c2x; fy += c1y - c2y; fz += c1z - c2z; e += c1e - c2e;
	}
	return true;
}

/* res: E, force xyz, Euler gradient xyz (Result_6D order); identical on all
 * lanes.  W is this warp's shared staging area. */
template <bool CENSUS>
__device__ __forceinline__ void eval_pose_rigid(const RigidModel& M, float tx, float ty, float tz,
		float a0, float a1, float a2, int lane, WarpStage& W, float res[7], PoseCensus* census) {
	const PoseRot R = pose_rotation(a0, a1, a2, lane);
	PoseSums S;
	uint32_t c_grid = 0, c_charged = 0, c_nl = 0, c_ent = 0;
	for (uint32_t i0 = 0; i0 < M.lig.n; i0 += kBeadsPerRound) {
		/* 1. stage 64 beads, two per lane */
		uint32_t nlk0, nlk1, nl0, nl1;
		bool in0, in1;
		stage_bead(M, R, tx, ty, tz, i0 + lane, lane, W, nlk0, nl0, in0);
		stage_bead(M, R, tx, ty, tz, i0 + lane + 32, lane + 32, W, nlk1, nl1, in1);
		if (CENSUS) {
			c_grid += (nlk0 > 0) + (nlk1 > 0);
			c_charged += (nlk0 > 1) + (nlk1 > 1);
			c_nl += in0 + in1;
			c_ent += nl0 + nl1;
		}
		/* queue positions: lookups of bead lane, then bead lane+32 */
		const uint32_t lk_incl = warp_incl_scan(nlk0 + nlk1, lane);
		const uint32_t n_look = __shfl_sync(GBA_FULL_MASK, lk_incl, 31);
		uint32_t lk = lk_incl - nlk0 - nlk1;
		if (nlk0 > 0) W.look[lk++] = (uint8_t)(lane << 1);
		if (nlk0 > 1) W.look[lk++] = (uint8_t)((lane << 1) | 1);
		if (nlk1 > 0) W.look[lk++] = (uint8_t)((lane + 32) << 1);
		if (nlk1 > 1) W.look[lk++] = (uint8_t)(((lane + 32) << 1) | 1);
		/* NL prefix over slots: slot s < 32 first, then s + 32 */
		const uint32_t a_incl = warp_incl_scan(nl0, lane);
		const uint32_t a_tot = __shfl_sync(GBA_FULL_MASK, a_incl, 31);
		const uint32_t b_incl = warp_incl_scan(nl1, lane);
		W.nl_pre[lane] = a_incl - nl0;
		W.nl_pre[lane + 32] = a_tot + b_incl - nl1;
		const uint32_t n_pair = a_tot + __shfl_sync(GBA_FULL_MASK, b_incl, 31);
		if (lane == 0) W.nl_pre[kBeadsPerRound] = n_pair;
		__syncwarp();

		/* 2. grid lookups, one per lane */
		for (uint32_t k = lane; k < n_look; k += 32) {
			const uint32_t e = W.look[k];
			const uint32_t s = e >> 1;
			const bool is_q = e & 1u;
			const uint32_t ch = W.chan[s];
			const DevIntrpl& g = (ch & 0x80000000u) ? M.grid.outer : M.grid.inner;
			const uint32_t sx = g.dimN[0], sxy = g.dimN[0] * g.dimN[1];
			const uint32_t c = is_q ? 0u : (ch & 0x7fffffffu);
			float4 v;
			if (g.oct) {
				const size_t nocts = (size_t)(g.dimN[0] - 1) * (g.dimN[1] - 1) * (g.dimN[2] - 1);
				const float4* base = g.oct + 8 * ((size_t)c * nocts + W.off[s]);
				v = octet_lerp(base, 2, 4, W.wnx[s], W.wny[s], W.wnz[s], W.wxx[s], W.wxy[s], W.wxz[s]);
			} else {
				const float4* base = g.data + (size_t)c * (sxy * g.dimN[2]) + W.off[s];
				v = octet_lerp(base, sx, sxy, W.wnx[s], W.wny[s], W.wnz[s], W.wxx[s], W.wxy[s], W.wxz[s]);
			}
			float sc = g.voxelVol_inv;
			v.x *= sc; v.y *= sc; v.z *= sc; v.w *= sc;
			if (is_q) {
				const float q = W.q[s];
				v.x *= q; v.y *= q; v.z *= q; v.w *= q;
			}
			S.add(v.w, v.x, v.y, v.z, W.ux[s], W.uy[s], W.uz[s]);
		}

		/* 3. neighbour pairs, one per lane */
		for (uint32_t k = lane; k < n_pair; k += 32) {
			/* owner slot: last s with nl_pre[s] <= k */
			uint32_t lo = 0, hi = kBeadsPerRound;
#pragma unroll
			for (int it = 0; it < 6; ++it) {
				const uint32_t mid = (lo + hi) >> 1;
				if (W.nl_pre[mid] <= k) lo = mid; else hi = mid;
			}
			const uint32_t s = lo;
			const uint32_t j = __ldg(&M.grid.nl.list[W.nl_idx[s] + (k - W.nl_pre[s])]);
			const float4 r = __ldg(&M.rec.xyzq[j]);
			const uint32_t trec = __ldg(&M.rec.tm[j]) & 0xffffu;
			float fx, fy, fz, e;
			if (nl_pair(M.grid.nl, M.par, W.type[s], W.q[s], W.px[s], W.py[s], W.pz[s], r.x, r.y,
					r.z, r.w, trec, fx, fy, fz, e))
				S.add(e, fx, fy, fz, W.ux[s], W.uy[s], W.uz[s]);
		}
		__syncwarp();
	}
	float sE = warp_sum(S.E), sFx = warp_sum(S.Fx), sFy = warp_sum(S.Fy), sFz = warp_sum(S.Fz);
	float T[9];
#pragma unroll
	for (int k = 0; k < 9; ++k) T[k] = warp_sum(S.T[k]);
	force_lim(sFx, sFy, sFz);
	float ang[3];
	torque_reduce(R, T, ang);
	res[0] = sE; res[1] = sFx; res[2] = sFy; res[3] = sFz;
	res[4] = ang[0]; res[5] = ang[1]; res[6] = ang[2];
	if (CENSUS) {
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			c_grid += __shfl_xor_sync(GBA_FULL_MASK, c_grid, o);
			c_charged += __shfl_xor_sync(GBA_FULL_MASK, c_charged, o);
			c_nl += __shfl_xor_sync(GBA_FULL_MASK, c_nl, o);
			c_ent += __shfl_xor_sync(GBA_FULL_MASK, c_ent, o);
		}
		if (lane == 0) *census = PoseCensus{c_grid, c_charged, c_nl, c_ent};
	}
}

/* Lanes 0..6 store the 7 result floats (one coalesced 28-byte write). */
__device__ __forceinline__ void store_result7(float* dst, const float res[7], int lane) {
	float v = 0.f;
#pragma unroll
	for (int k = 0; k < 7; ++k) v = lane == k ? res[k] : v;
	if (lane < 7) dst[lane] = v;
}

}  // namespace gba

#endif
