/*
 * rigid_pose.cuh -- one warp evaluates one rigid pose.
 *
 * Shared by the scoring kernel (energy_rigid.cu), the multi-pair kernel and
 * the persistent minimizer (minimize.cu); the staging helpers also serve the
 * normal-mode kernel (energy_modes.cu).  The per-bead work of the reference
 * -- transform (src/model/transform.h:22-44), inner/outer grid term
 * (src/model/interpolation.h:57-101) and neighbour-list term
 * (src/model/neighborlist.h:29-168) -- is reorganised for the SIMT machine:
 *
 *   1. lane-per-bead, 64 beads per round (two per lane): rotate/translate,
 *      bounds tests, voxel indices and trilinear weights, NL voxel lookup;
 *      the bead's geometry goes to per-warp shared memory and each bead
 *      enqueues one grid lookup per channel it reads (type, and charge when
 *      |q| > 0.001) and its NL list length;
 *   2. the warp drains the lookup queue: one lookup per lane (8 gathered
 *      float4 corners), or with the octet layout and GBA_KOPT_COOP_LOOKUP
 *      eight lanes per lookup, one corner each (one 128-byte line per
 *      lookup, four lookups per warp instruction, loaded without L1
 *      allocation so that L1 keeps the receptor and parameter data);
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
	/* the pose: rotation matrix [0, 9), sin/cos of phi, ssi, rot [9, 15),
	 * translation [15, 18); kept here rather than in registers */
	float pose[18];
};

/* Stores the pose rotation and translation in the warp's staging area. */
__device__ __forceinline__ void put_pose(WarpStage& W, const PoseRot& R, float tx, float ty, float tz,
		int lane) {
	if (lane == 0) {
#pragma unroll
		for (int k = 0; k < 9; ++k) W.pose[k] = R.m[k];
		W.pose[9] = R.cphi; W.pose[10] = R.sphi; W.pose[11] = R.cssi;
		W.pose[12] = R.sssi; W.pose[13] = R.crot; W.pose[14] = R.srot;
		W.pose[15] = tx; W.pose[16] = ty; W.pose[17] = tz;
	}
	__syncwarp();
}

/* Reads back what put_pose stored; the volatile reads keep the compiler from
 * holding these 18 values in registers across the bead rounds. */
__device__ __forceinline__ PoseRot get_pose(const WarpStage& W, float& tx, float& ty, float& tz) {
	const volatile float* v = W.pose;
	PoseRot R;
#pragma unroll
	for (int k = 0; k < 9; ++k) R.m[k] = v[k];
	R.cphi = v[9]; R.sphi = v[10]; R.cssi = v[11]; R.sssi = v[12]; R.crot = v[13]; R.srot = v[14];
	tx = v[15]; ty = v[16]; tz = v[17];
	return R;
}

/* Inclusive warp scan of v. */
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const uint32_t t = __shfl_up_sync(GBA_FULL_MASK, v, o);
		if (lane >= o) v += t;
	}
	return v;
}

/* potForce's grid selection for a staged bead at (px, py, pz),
 * src/model/interpolation.h:66-76, with getIndex / getVoxelByIndex
 * (src/model/IntrplGrid.h:96-104,130-163): picks inner or outer grid, stores
 * the octet offset and trilinear weights in slot s and returns the number of
 * lookups (0, 1, or 2 with the charge channel). */
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

/* Grid and first corner of queued lookup e (bead << 1 | is_charge). */
__device__ __forceinline__ const float4* lookup_base(const DevGrid& G, const WarpStage& W, uint32_t e,
		const DevIntrpl*& gp) {
	const uint32_t s = e >> 1;
	const uint32_t ch = W.chan[s];
	gp = (ch & 0x80000000u) ? &G.outer : &G.inner;
	const uint32_t c = (e & 1u) ? 0u : (ch & 0x7fffffffu);
	if (gp->oct) {
		const size_t nocts = (size_t)(gp->dimN[0] - 1) * (gp->dimN[1] - 1) * (gp->dimN[2] - 1);
		return gp->oct + 8 * ((size_t)c * nocts + W.off[s]);
	}
	const size_t sxy = (size_t)gp->dimN[0] * gp->dimN[1];
	return gp->data + (size_t)c * (sxy * gp->dimN[2]) + W.off[s];
}

/* One queued lookup by one lane: the channel's interpolated (fx, fy, fz, E),
 * scaled by 1/voxelVol and, for the charge channel, by the bead charge. */
__device__ __forceinline__ float4 grid_lookup(const DevGrid& G, const WarpStage& W, uint32_t e) {
	const uint32_t s = e >> 1;
	const DevIntrpl* gp;
	const float4* base = lookup_base(G, W, e, gp);
	float4 v;
	if (gp->oct)
		v = octet_lerp(base, 2, 4, W.wnx[s], W.wny[s], W.wnz[s], W.wxx[s], W.wxy[s], W.wxz[s]);
	else
		v = octet_lerp(base, gp->dimN[0], gp->dimN[0] * gp->dimN[1], W.wnx[s], W.wny[s], W.wnz[s],
				W.wxx[s], W.wxy[s], W.wxz[s]);
	const float sc = (e & 1u) ? fmul(gp->voxelVol_inv, W.q[s]) : gp->voxelVol_inv;
	v.x = fmul(v.x, sc); v.y = fmul(v.y, sc); v.z = fmul(v.z, sc); v.w = fmul(v.w, sc);
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

/* Accumulates f into the pose sums with the bead's unrotated coordinates. */
struct PoseSums {
	float E = 0.f, Fx = 0.f, Fy = 0.f, Fz = 0.f;
	float T[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
	__device__ __forceinline__ void add(float e, float fx, float fy, float fz, float ux, float uy,
			float uz) {
		E = fadd(E, e); Fx = fadd(Fx, fx); Fy = fadd(Fy, fy); Fz = fadd(Fz, fz);
		T[0] = ffma(ux, fx, T[0]); T[1] = ffma(uy, fx, T[1]); T[2] = ffma(uz, fx, T[2]);
		T[3] = ffma(ux, fy, T[3]); T[4] = ffma(uy, fy, T[4]); T[5] = ffma(uz, fy, T[5]);
		T[6] = ffma(ux, fz, T[6]); T[7] = ffma(uy, fz, T[7]); T[8] = ffma(uz, fz, T[8]);
	}
};

/* One lane's share of cooperative lookup k: its corner times its trilinear
 * weight, and the lookup's scale. */
struct CoopPart {
	float4 v;
	float sc;
	uint32_t e;
	bool valid;
};

__device__ __forceinline__ CoopPart coop_part(const DevGrid& G, const WarpStage& W, uint32_t k,
		uint32_t n_look, int cor) {
	CoopPart r;
	r.v = make_float4(0.f, 0.f, 0.f, 0.f);
	r.sc = 0.f;
	r.e = 0;
	r.valid = k < n_look;
	if (r.valid) {
		r.e = W.look[k];
		const uint32_t s = r.e >> 1;
		const DevIntrpl* gp;
		const float4* p = lookup_base(G, W, r.e, gp) + cor;
		const float4 d = ldg_no_l1(p);
		const float w = corner_weight(cor, W.wnx[s], W.wny[s], W.wnz[s], W.wxx[s], W.wxy[s], W.wxz[s]);
		r.v.x = fmul(d.x, w); r.v.y = fmul(d.y, w); r.v.z = fmul(d.z, w); r.v.w = fmul(d.w, w);
		r.sc = (r.e & 1u) ? fmul(gp->voxelVol_inv, W.q[s]) : gp->voxelVol_inv;
	}
	return r;
}

/* Drains the lookup queue of a round into S.  Cooperative form: lane group
 * grp = lane / 8 takes lookup k0 + grp and lane cor = lane % 8 loads octet
 * corner cor (x = bit 0, y = bit 1, z = bit 2; the octet record stores d000
 * d100 d010 d110 d001 d101 d011 d111) times its trilinear weight
 * (src/model/trilinIntrpl.h:29-66); a three-step butterfly sums the eight
 * products.  The sum order differs from the reference's left-to-right sum
 * (FP32 rounding only). */
__device__ __forceinline__ void drain_lookups(const DevGrid& G, const WarpStage& W, uint32_t n_look,
		int lane, PoseSums& S) {
	if (!G.coop_lookup) {
		for (uint32_t k = lane; k < n_look; k += 32) {
			const uint32_t e = W.look[k];
			const uint32_t s = e >> 1;
			const float4 v = grid_lookup(G, W, e);
			S.add(v.w, v.x, v.y, v.z, W.ux[s], W.uy[s], W.uz[s]);
		}
		return;
	}
	const int grp = lane >> 3, cor = lane & 7;
	/* two lookups per lane group and iteration: both corner loads are in
	 * flight before the butterflies */
	for (uint32_t k0 = 0; k0 < n_look; k0 += 8) {
		CoopPart a = coop_part(G, W, k0 + grp, n_look, cor);
		CoopPart b = coop_part(G, W, k0 + 4 + grp, n_look, cor);
#pragma unroll
		for (int o = 1; o < 8; o <<= 1) {
			a.v.x = fadd(a.v.x, __shfl_xor_sync(GBA_FULL_MASK, a.v.x, o));
			a.v.y = fadd(a.v.y, __shfl_xor_sync(GBA_FULL_MASK, a.v.y, o));
			a.v.z = fadd(a.v.z, __shfl_xor_sync(GBA_FULL_MASK, a.v.z, o));
			a.v.w = fadd(a.v.w, __shfl_xor_sync(GBA_FULL_MASK, a.v.w, o));
			b.v.x = fadd(b.v.x, __shfl_xor_sync(GBA_FULL_MASK, b.v.x, o));
			b.v.y = fadd(b.v.y, __shfl_xor_sync(GBA_FULL_MASK, b.v.y, o));
			b.v.z = fadd(b.v.z, __shfl_xor_sync(GBA_FULL_MASK, b.v.z, o));
			b.v.w = fadd(b.v.w, __shfl_xor_sync(GBA_FULL_MASK, b.v.w, o));
		}
		if (cor == 0) {
			if (a.valid) {
				const uint32_t s = a.e >> 1;
				S.add(fmul(a.v.w, a.sc), fmul(a.v.x, a.sc), fmul(a.v.y, a.sc), fmul(a.v.z, a.sc), W.ux[s],
						W.uy[s], W.uz[s]);
			}
			if (b.valid) {
				const uint32_t s = b.e >> 1;
				S.add(fmul(b.v.w, b.sc), fmul(b.v.x, b.sc), fmul(b.v.y, b.sc), fmul(b.v.z, b.sc), W.ux[s],
						W.uy[s], W.uz[s]);
			}
		}
	}
}

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
	dx = fmul(dx, dr2_inv); dy = fmul(dy, dr2_inv); dz = fmul(dz, dr2_inv);
	const bool shape86 = P.potshape == GBA_POTSHAPE_8_6;
	const size_t k = (size_t)P.num_types * (trec - 1) + (lig_type - 1);
	const float4 p = __ldg(&P.lj[k]);
	const float iv = __ldg(&P.ivor[k]);
	float f1x, f1y, f1z, e1;
	lj_pot_force(dr2, dr2_inv, dx, dy, dz, p, iv, shape86, f1x, f1y, f1z, e1);
	/* getRatio's table bin, src/model/NLGrid.h:141-143 */
	const int bin = (int)fmul(dr2, 10000.0f);
	const float ratio = nl.ratio_computed
			? __fsqrt_rn(fmul(fadd((float)bin, 0.5f), nl.ratio_scale))
			: __ldg(&nl.ratio[bin]);
	const float rdx = fmul(ratio, dx), rdy = fmul(ratio, dy), rdz = fmul(ratio, dz);
	float f2x, f2y, f2z, e2;
	lj_pot_force(nl.dPlateau2, nl.dPlateau2_inv, rdx, rdy, rdz, p, iv, shape86, f2x, f2y, f2z, e2);
	fx = fsub(f1x, f2x); fy = fsub(f1y, f2y); fz = fsub(f1z, f2z); e = fsub(e1, e2);
	const float qq = fmul(fmul(qlig, rq), P.ffelec);
	if (fabsf(qq) > 0.001f) {
		const bool cdiel = P.dielec == GBA_DIELEC_CONSTANT;
		float c1x, c1y, c1z, c1e, c2x, c2y, c2z, c2e;
		charge_pot_force(dr2_inv, dx, dy, dz, qq, cdiel, c1x, c1y, c1z, c1e);
		charge_pot_force(nl.dPlateau2_inv, rdx, rdy, rdz, qq, cdiel, c2x, c2y, c2z, c2e);
		fx = fadd(fx, fsub(c1x, c2x)); fy = fadd(fy, fsub(c1y, c2y)); fz = fadd(fz, fsub(c1z, c2z));
		e = fadd(e, fsub(c1e, c2e));
	}
	return true;
}

/* res: E, force xyz, Euler gradient xyz (Result_6D order); identical on all
 * lanes.  W is this warp's shared staging area. */
template <bool CENSUS>
__device__ __forceinline__ void eval_pose_rigid(const RigidModel& M, float tx, float ty, float tz,
		float a0, float a1, float a2, int lane, WarpStage& W, float res[7], PoseCensus* census) {
	put_pose(W, pose_rotation(a0, a1, a2, lane), tx, ty, tz, lane);
	PoseSums S;
	uint32_t c_grid = 0, c_charged = 0, c_nl = 0, c_ent = 0;
	for (uint32_t i0 = 0; i0 < M.lig.n; i0 += kBeadsPerRound) {
		/* 1. stage 64 beads, two per lane: lane, then lane + 32 */
		float ttx, tty, ttz;
		const PoseRot R = get_pose(W, ttx, tty, ttz);
		uint32_t nlk[2], nln[2];
#pragma unroll
		for (int h = 0; h < 2; ++h) {
			const int s = lane + 32 * h;
			const uint32_t i = i0 + s;
			nlk[h] = 0;
			nln[h] = 0;
			bool in_nl = false;
			if (i < M.lig.n) {
				const float4 b = __ldg(&M.lig.xyzq[i]);
				const uint32_t tm = __ldg(&M.lig.tm[i]);
				const uint32_t type = tm & 0xffffu, mapped = tm >> 16;
				float px, py, pz;
				rot_apply(R.m, b.x, b.y, b.z, px, py, pz);
				px = fadd(px, ttx); py = fadd(py, tty); pz = fadd(pz, ttz);
				W.ux[s] = b.x; W.uy[s] = b.y; W.uz[s] = b.z;
				W.px[s] = px; W.py[s] = py; W.pz[s] = pz;
				W.q[s] = b.w;
				W.type[s] = type;
				nlk[h] = stage_grid(M.grid, px, py, pz, mapped, b.w, s, W);
				if (type != 0) nln[h] = stage_nl(M.grid.nl, px, py, pz, s, W, in_nl);
			}
			if (CENSUS) {
				c_grid += nlk[h] > 0;
				c_charged += nlk[h] > 1;
				c_nl += in_nl;
				c_ent += nln[h];
			}
		}
		/* queue positions: lookups of bead lane, then bead lane+32 */
		const uint32_t lk_incl = warp_incl_scan(nlk[0] + nlk[1], lane);
		const uint32_t n_look = __shfl_sync(GBA_FULL_MASK, lk_incl, 31);
		uint32_t lk = lk_incl - nlk[0] - nlk[1];
		enqueue_lookups(W, lk, lane, nlk[0]);
		enqueue_lookups(W, lk, lane + 32, nlk[1]);
		/* NL prefix over slots: slot s < 32 first, then s + 32 */
		const uint32_t a_incl = warp_incl_scan(nln[0], lane);
		const uint32_t a_tot = __shfl_sync(GBA_FULL_MASK, a_incl, 31);
		const uint32_t b_incl = warp_incl_scan(nln[1], lane);
		W.nl_pre[lane] = a_incl - nln[0];
		W.nl_pre[lane + 32] = a_tot + b_incl - nln[1];
		const uint32_t n_pair = a_tot + __shfl_sync(GBA_FULL_MASK, b_incl, 31);
		if (lane == 0) W.nl_pre[kBeadsPerRound] = n_pair;
		__syncwarp();

		/* 2. grid lookups */
		drain_lookups(M.grid, W, n_look, lane, S);

		/* 3. neighbour pairs, one per lane; two per lane and iteration so that
		 * both gather chains (list entry -> receptor bead -> parameters) are
		 * in flight together */
		for (uint32_t k = lane; k < n_pair; k += 64) {
			const uint32_t k2 = k + 32;
			const bool has2 = k2 < n_pair;
			const uint32_t sa = pair_owner(W, k);
			const uint32_t sb = has2 ? pair_owner(W, k2) : sa;
			const uint32_t ja = __ldg(&M.grid.nl.list[W.nl_idx[sa] + (k - W.nl_pre[sa])]);
			const uint32_t jb = has2 ? __ldg(&M.grid.nl.list[W.nl_idx[sb] + (k2 - W.nl_pre[sb])]) : ja;
			const float4 ra = __ldg(&M.rec.xyzq[ja]);
			const float4 rb = __ldg(&M.rec.xyzq[jb]);
			const uint32_t ta = __ldg(&M.rec.tm[ja]) & 0xffffu;
			const uint32_t tb = __ldg(&M.rec.tm[jb]) & 0xffffu;
			float fx, fy, fz, e;
			if (nl_pair(M.grid.nl, M.par, W.type[sa], W.q[sa], W.px[sa], W.py[sa], W.pz[sa], ra.x, ra.y,
					ra.z, ra.w, ta, fx, fy, fz, e))
				S.add(e, fx, fy, fz, W.ux[sa], W.uy[sa], W.uz[sa]);
			if (has2 && nl_pair(M.grid.nl, M.par, W.type[sb], W.q[sb], W.px[sb], W.py[sb], W.pz[sb], rb.x,
					rb.y, rb.z, rb.w, tb, fx, fy, fz, e))
				S.add(e, fx, fy, fz, W.ux[sb], W.uy[sb], W.uz[sb]);
		}
		__syncwarp();
	}
	float sE = warp_sum(S.E), sFx = warp_sum(S.Fx), sFy = warp_sum(S.Fy), sFz = warp_sum(S.Fz);
	float T[9];
#pragma unroll
	for (int k = 0; k < 9; ++k) T[k] = warp_sum(S.T[k]);
	force_lim(sFx, sFy, sFz);
	float ang[3];
	float ttx, tty, ttz;
	torque_reduce(get_pose(W, ttx, tty, ttz), T, ang);
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
