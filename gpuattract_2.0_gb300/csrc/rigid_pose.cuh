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
 *   2. the warp drains the flattened (bead, neighbour) pair list in windows
 *      of 64 pairs, two per lane (owners from per-window start masks);
 *   3. the warp drains the lookup queue: one lookup per lane (8 gathered
 *      float4 corners), or with the octet layout and GBA_KOPT_COOP_LOOKUP
 *      eight lanes per lookup, one corner each (one 128-byte line per
 *      lookup, sixteen lookups per step, loaded without L1 allocation so
 *      that L1 keeps the receptor and parameter data).  Pairs come first:
 *      measured on GB300, this order is faster.
 * Every lookup and pair contributes straight to the pose sums: energy,
 * force and the torque matrix sum_i x_i (x) f_i are linear in the bead
 * forces, so no per-bead force is kept (reducePotForce / reduceTorque,
 * src/model/reduction.h:40-103).  Two summation orders exist:
 *   per pose   (scoring kernels) each lane accumulates over all rounds and
 *              the warp reduces once per pose;
 *   round-wise (minimizer kernels and the plain per-step form's launches)
 *              each 64-bead round is reduced on its own by a fixed 16-value
 *              reduce-scatter (round_reduce) and the round totals are added
 *              in round order, so a pose's result does not depend on which
 *              warp evaluates which round: a team of warps splitting one
 *              pose (eval_pose_rigid_team) gives the same bits as one warp.
 * Both are deterministic; they differ from each other in the last bits.  The
 * per-pose order stays in the scoring kernels because the round-wise
 * reduction costs them registers at their 64-register bound (it spills and
 * measured 13 % slower on config 1).
 */
#ifndef GBA_RIGID_POSE_CUH_
#define GBA_RIGID_POSE_CUH_

#include <cstddef>

#include "energy_dev.cuh"

namespace gba {

constexpr int kBeadsPerRound = 64;
constexpr int kCornerStride = 9;   /* corner weights per slot, padded: 9 is odd, so
                                      consecutive slots start in different banks */

/* Per-warp staging of one round of beads.  Consumers read whole records:
 * one 16-byte load gives a bead's transformed position and charge, another
 * its unrotated coordinates and type. */
struct WarpStage {
	float4 pq[kBeadsPerRound];         /* transformed x, y, z; charge */
	float4 ut[kBeadsPerRound];         /* unrotated x, y, z (torque); type (bits) */
	uint32_t lbase[kBeadsPerRound];    /* list start - first flattened pair of the slot */
	float cw[kBeadsPerRound * kCornerStride];   /* trilinear weight of octet corner c */
	uint2 look[2 * kBeadsPerRound];    /* lookup queue: {element | outer << 31, slot | is_charge << 7} */
	uint8_t own[64];                   /* PairWindow: slot of the bead starting at window position b */
	/* the pose: rotation matrix [0, 9), sin/cos of phi, ssi, rot [9, 15),
	 * translation [15, 18); kept here rather than in registers */
	float pose[18];
	/* round-wise order: running total of the rounds, component c in tot[c]
	 * (written by lane 2c) */
	float tot[16];
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

/* Staged bead record of slot s: positions, charge, torque lever, type. */
__device__ __forceinline__ void put_bead(WarpStage& W, int s, float ux, float uy, float uz, float px,
		float py, float pz, float q, uint32_t type) {
	W.pq[s] = make_float4(px, py, pz, q);
	W.ut[s] = make_float4(ux, uy, uz, __uint_as_float(type));
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

/* Element indices of a bead's grid lookups: type channel and charge channel,
 * each | outer grid << 31.  An element addresses a 128-byte octet record on
 * octet grids and the first corner float4 otherwise. */
struct BeadGrid {
	uint32_t t, q;
};

/* potForce's grid selection for a staged bead at (px, py, pz),
 * src/model/interpolation.h:66-76, with getIndex / getVoxelByIndex
 * (src/model/IntrplGrid.h:96-104,130-163): picks inner or outer grid, stores
 * the eight trilinear corner weights of slot s, sets the element indices and
 * returns the number of lookups (0, 1, or 2 with the charge channel). */
__device__ __forceinline__ uint32_t stage_grid(const DevGrid& G, float px, float py, float pz,
		uint32_t mapped, float q, int s, WarpStage& W, BeadGrid& bg) {
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
	const float pmn_x = fsub(px, minx), pmn_y = fsub(py, miny), pmn_z = fsub(pz, minz);
	const float pmx_x = fsub(fadd(minx, g.dVox), px);
	const float pmx_y = fsub(fadd(miny, g.dVox), py);
	const float pmx_z = fsub(fadd(minz, g.dVox), pz);
	float* cw = W.cw + kCornerStride * s;
#pragma unroll
	for (int c = 0; c < 8; ++c) cw[c] = corner_weight(c, pmn_x, pmn_y, pmn_z, pmx_x, pmx_y, pmx_z);
	uint32_t off, cells;
	if (g.oct) {
		cells = (g.dimN[0] - 1) * (g.dimN[1] - 1) * (g.dimN[2] - 1);
		off = (g.dimN[0] - 1) * (iz * (g.dimN[1] - 1) + iy) + ix;
	} else {
		cells = g.dimN[0] * g.dimN[1] * g.dimN[2];
		off = g.dimN[0] * (iz * g.dimN[1] + iy) + ix;
	}
	const uint32_t og = outer ? 0x80000000u : 0u;
	bg.t = (mapped * cells + off) | og;
	bg.q = off | og;
	return fabsf(q) > 0.001f ? 2u : 1u;
}

/* NL voxel lookup of a staged bead (type != 0), NLPotForce's
 * src/model/neighborlist.h:59-66: stores the list start (queue_pairs turns it
 * into the slot's list base) and returns the list length (0 outside). */
template <class Stage>
__device__ __forceinline__ uint32_t stage_nl(const DevNL& nl, float px, float py, float pz, int s,
		Stage& W, bool& in_nl) {
	in_nl = false;
	if (nl_out(nl, px, py, pz)) return 0;
	const int ix = min(max((int)roundf(fmul(fsub(px, nl.pos[0]), nl.dVox_inv)), 0), (int)nl.dimN[0] - 1);
	const int iy = min(max((int)roundf(fmul(fsub(py, nl.pos[1]), nl.dVox_inv)), 0), (int)nl.dimN[1] - 1);
	const int iz = min(max((int)roundf(fmul(fsub(pz, nl.pos[2]), nl.dVox_inv)), 0), (int)nl.dimN[2] - 1);
	const uint2 d = __ldg(&nl.grid[nl.dimN[0] * (iz * nl.dimN[1] + iy) + ix]);
	W.lbase[s] = d.y;
	in_nl = true;
	return d.x;
}

/* Bead slot of queued lookup k. */
__device__ __forceinline__ uint32_t lookup_slot(const WarpStage& W, uint32_t k) { return W.look[k].y & 0x7fu; }

/* Grid, element, slot and scale of queued lookup k: 1/voxelVol, times the
 * bead charge for the charge channel. */
__device__ __forceinline__ const DevIntrpl& lookup_grid(const DevGrid& G, const WarpStage& W, uint32_t k,
		uint32_t& elem, uint32_t& s, float& sc) {
	const uint2 e = W.look[k];
	const DevIntrpl& g = (e.x & 0x80000000u) ? G.outer : G.inner;
	elem = e.x & 0x7fffffffu;
	s = e.y & 0x7fu;
	sc = (e.y & 0x80u) ? fmul(g.voxelVol_inv, W.pq[s].w) : g.voxelVol_inv;
	return g;
}

/* One queued lookup by one lane: the channel's interpolated (fx, fy, fz, E),
 * scaled. */
__device__ __forceinline__ float4 grid_lookup(const DevGrid& G, const WarpStage& W, uint32_t k) {
	uint32_t elem, s;
	float sc;
	const DevIntrpl& g = lookup_grid(G, W, k, elem, s, sc);
	const float* cw = W.cw + kCornerStride * s;
	float w[8];
#pragma unroll
	for (int c = 0; c < 8; ++c) w[c] = cw[c];
	const float4 v = g.oct ? octet_lerp_w(g.oct + 8 * (size_t)elem, 2, 4, w)
	                       : octet_lerp_w(g.data + elem, g.dimN[0], g.dimN[0] * g.dimN[1], w);
	return make_float4(fmul(v.x, sc), fmul(v.y, sc), fmul(v.z, sc), fmul(v.w, sc));
}

/* Writes the lookup queue entries of slot s (n = 0..2) at position k. */
__device__ __forceinline__ void enqueue_lookups(WarpStage& W, uint32_t k, int s, uint32_t n, const BeadGrid& bg) {
	if (n > 0) W.look[k] = make_uint2(bg.t, (uint32_t)s);
	if (n > 1) W.look[k + 1] = make_uint2(bg.q, (uint32_t)s | 0x80u);
}

/* Fills the lookup queue of a round from the per-lane counts (nlk[0] for
 * bead slot lane, nlk[1] for slot lane + 32): slots 0..31 first, then 32..63,
 * so that neighbouring queue entries belong to neighbouring slots.  Returns
 * the queue length. */
__device__ __forceinline__ uint32_t queue_lookups(WarpStage& W, const uint32_t nlk[2], const BeadGrid bg[2],
		int lane) {
	const uint32_t incl = warp_incl_scan(nlk[0] | (nlk[1] << 16), lane);
	const uint32_t tot = __shfl_sync(GBA_FULL_MASK, incl, 31);
	const uint32_t tot_a = tot & 0xffffu;
	enqueue_lookups(W, (incl & 0xffffu) - nlk[0], lane, nlk[0], bg[0]);
	enqueue_lookups(W, tot_a + (incl >> 16) - nlk[1], lane + 32, nlk[1], bg[1]);
	return tot_a + (tot >> 16);
}

/* Exclusive prefix of the NL list lengths over slots 0..63 (slot lane, then
 * lane + 32); turns each slot's list start into its list base (list index of
 * flattened pair k = lbase + k) and returns the number of pairs of the round
 * and, per lane, the first flattened pair of its two slots. */
template <class Stage>
__device__ __forceinline__ uint32_t queue_pairs(Stage& W, const uint32_t nln[2], int lane,
		uint32_t start[2]) {
	const uint32_t a_incl = warp_incl_scan(nln[0], lane);
	const uint32_t a_tot = __shfl_sync(GBA_FULL_MASK, a_incl, 31);
	const uint32_t b_incl = warp_incl_scan(nln[1], lane);
	start[0] = a_incl - nln[0];
	start[1] = a_tot + b_incl - nln[1];
	if (nln[0]) W.lbase[lane] -= start[0];
	if (nln[1]) W.lbase[lane + 32] -= start[1];
	return a_tot + __shfl_sync(GBA_FULL_MASK, b_incl, 31);
}

/* Owners of the 64 pairs [w, w + 64) of a round, window by window: every
 * non-empty bead starting inside the window sets bit (start - w) and records
 * its slot in W.own; the owner of pair w + b is the bead of the highest set
 * bit <= b, or, with none, the bead that covered pair w - 1 (carry).  Two
 * warp OR-reductions per window replace a search per pair. */
struct PairWindow {
	uint32_t carry = 0;
	/* lane gets the owners of pairs w + lane and w + 32 + lane */
	template <class Stage>
	__device__ __forceinline__ void owners(Stage& W, uint32_t w, const uint32_t start[2],
			const uint32_t len[2], int lane, uint32_t& sa, uint32_t& sb) {
		uint32_t lo = 0, hi = 0;
#pragma unroll
		for (int h = 0; h < 2; ++h)
			if (len[h] > 0 && start[h] >= w && start[h] - w < 64u) {
				const uint32_t b = start[h] - w;
				W.own[b] = (uint8_t)(lane + 32 * h);
				if (b < 32) lo |= 1u << b; else hi |= 1u << (b - 32);
			}
		lo = __reduce_or_sync(GBA_FULL_MASK, lo);
		hi = __reduce_or_sync(GBA_FULL_MASK, hi);
		__syncwarp();
		const uint32_t upto = 0xffffffffu >> (31 - lane);   /* bits 0..lane */
		const uint32_t last_lo = lo ? W.own[31 - __clz(lo)] : carry;   /* owner of pair w + 31 */
		const uint32_t mlo = lo & upto, mhi = hi & upto;
		sa = mlo ? W.own[31 - __clz(mlo)] : carry;
		sb = mhi ? W.own[63 - __clz(mhi)] : last_lo;
		carry = hi ? W.own[63 - __clz(hi)] : last_lo;              /* owner of pair w + 63 */
		__syncwarp();
	}
};

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

/* Cooperative accumulators of one lane: the lane always ends a butterfly
 * holding the same component (x, y, z of the force or E) of one of the two
 * lookups of its group, so it accumulates that component and, for a force
 * component, its three torque-matrix entries u (x) f. */
struct CoopSums {
	float f = 0.f, t0 = 0.f, t1 = 0.f, t2 = 0.f;
	/* adds the lane's role into S: comp 0..2 = force x, y, z, 3 = energy
	 * (static indices only, so S stays in registers) */
	__device__ __forceinline__ void fold(PoseSums& S, int comp) const {
		const float z = 0.f;
		S.E = fadd(S.E, comp == 3 ? f : z);
		S.Fx = fadd(S.Fx, comp == 0 ? f : z);
		S.Fy = fadd(S.Fy, comp == 1 ? f : z);
		S.Fz = fadd(S.Fz, comp == 2 ? f : z);
#pragma unroll
		for (int r = 0; r < 3; ++r) {
			S.T[3 * r] = fadd(S.T[3 * r], comp == r ? t0 : z);
			S.T[3 * r + 1] = fadd(S.T[3 * r + 1], comp == r ? t1 : z);
			S.T[3 * r + 2] = fadd(S.T[3 * r + 2], comp == r ? t2 : z);
		}
	}
};

/* Drains the lookup queue of a round.  Per-lane form: one lookup per lane
 * into S.  Cooperative form (octet layout), sixteen lookups per step in two
 * blocks of eight: in block b, lane group g = lane / 8 takes lookups
 * k0 + 8 b + g and k0 + 8 b + 4 + g, lane c = lane % 8 loads octet corner c
 * of both (one 128-byte line per lookup, read without L1 allocation) times
 * its trilinear weight (src/model/trilinIntrpl.h:29-66); all four loads of a
 * lane are issued before the first is used.  A three-step reduce-scatter over
 * the group leaves lane c holding one finished component -- lookup (c & 1),
 * component 2 * ((c >> 1) & 1) + (c >> 2) -- summed in octet_sum's pairwise
 * order, so both forms give the same value per lookup.  Each lane loads its
 * own lookup first, which makes the first step select-free.  The lane scales
 * the component and adds it to its CoopSums role. */
/* One cooperative step of drain_lookups: the loads and the reduce-scatter of
 * lookups k0 .. k0 + 8 NB - 1, kept apart so that other work can run between
 * them. */
template <int NB>
struct CoopStep {
	float c[NB][8];   /* per block b: own lookup x y z w, partner's x y z w */
	uint32_t sl[NB];
	float sc[NB];
	bool ok[NB];

	/* block b, lane (g, c): own lookup k0 + 8 b + 4 mine + g, then the partner's */
	__device__ __forceinline__ void load(const DevGrid& G, const WarpStage& W, uint32_t k0, uint32_t n_look,
			int lane) {
		const int grp = lane >> 3, cor = lane & 7, mine = cor & 1;
#pragma unroll
		for (int b = 0; b < NB; ++b) {
			sl[b] = 0;
			sc[b] = 0.f;
			ok[b] = false;
#pragma unroll
			for (int h = 0; h < 2; ++h) {
				const uint32_t k = k0 + 8 * b + 4 * (h ^ mine) + grp;
				float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
				float w = 0.f;
				if (k < n_look) {
					uint32_t elem, s;
					float scale;
					const DevIntrpl& g = lookup_grid(G, W, k, elem, s, scale);
					d = ldg_no_l1(g.oct + 8 * (size_t)elem + cor);
					w = W.cw[kCornerStride * s + cor];
					if (h == 0) { sl[b] = s; sc[b] = scale; ok[b] = true; }
				}
				c[b][4 * h] = fmul(d.x, w); c[b][4 * h + 1] = fmul(d.y, w);
				c[b][4 * h + 2] = fmul(d.z, w); c[b][4 * h + 3] = fmul(d.w, w);
			}
		}
	}

	/* the reduce-scatter of block b: the lane's finished, unscaled component
	 * (lane c: lookup c & 1, component 2 * ((c >> 1) & 1) + (c >> 2)) */
	__device__ __forceinline__ float component(int b, int lane) const {
		const int cor = lane & 7;
		const int hi2 = (cor >> 1) & 1, hi4 = cor >> 2;
		/* step 1 (partner c ^ 1): keep the own lookup */
		float m4[4];
#pragma unroll
		for (int j = 0; j < 4; ++j) m4[j] = fadd(c[b][j], __shfl_xor_sync(GBA_FULL_MASK, c[b][4 + j], 1));
		/* step 2 (partner c ^ 2): keep components {0,1} or {2,3} */
		float m2[2];
#pragma unroll
		for (int j = 0; j < 2; ++j) {
			const float keep = hi2 ? m4[2 + j] : m4[j];
			const float send = hi2 ? m4[j] : m4[2 + j];
			m2[j] = fadd(keep, __shfl_xor_sync(GBA_FULL_MASK, send, 2));
		}
		/* step 3 (partner c ^ 4): keep one */
		const float keep = hi4 ? m2[1] : m2[0];
		const float send = hi4 ? m2[0] : m2[1];
		return fadd(keep, __shfl_xor_sync(GBA_FULL_MASK, send, 4));
	}

	__device__ __forceinline__ void reduce(const WarpStage& W, int lane, CoopSums& C) const {
		const int cor = lane & 7;
		const int comp = 2 * ((cor >> 1) & 1) + (cor >> 2);     /* which component */
#pragma unroll
		for (int b = 0; b < NB; ++b) {
			const float v = component(b, lane);
			if (ok[b]) {
				const float f = fmul(v, sc[b]);
				C.f = fadd(C.f, f);
				if (comp != 3) {
					const float4 u = W.ut[sl[b]];
					C.t0 = ffma(u.x, f, C.t0);
					C.t1 = ffma(u.y, f, C.t1);
					C.t2 = ffma(u.z, f, C.t2);
				}
			}
		}
	}
};

/* Component (0..3 = force x, y, z, energy) that lane holds after
 * CoopStep::component. */
__device__ __forceinline__ int coop_component(int lane) {
	const int cor = lane & 7;
	return 2 * ((cor >> 1) & 1) + (cor >> 2);
}

__device__ __forceinline__ void drain_lookups(const DevGrid& G, const WarpStage& W, uint32_t n_look,
		int lane, PoseSums& S, CoopSums& C) {
	if (!G.coop_lookup) {
		for (uint32_t k = lane; k < n_look; k += 32) {
			const uint32_t s = lookup_slot(W, k);
			const float4 v = grid_lookup(G, W, k);
			const float4 u = W.ut[s];
			S.add(v.w, v.x, v.y, v.z, u.x, u.y, u.z);
		}
		return;
	}
	for (uint32_t k0 = 0; k0 < n_look; k0 += 16) {
		CoopStep<2> st;
		st.load(G, W, k0, n_look, lane);
		st.reduce(W, lane, C);
	}
}

/* Fold of the cooperative accumulators into the pose sums (component of the lane). */
__device__ __forceinline__ void fold_coop(const CoopSums& C, PoseSums& S, int lane) {
	const int cor = lane & 7;
	C.fold(S, 2 * ((cor >> 1) & 1) + (cor >> 2));
}

/* One NL pair term (plateau-subtracted LJ + Coulomb), the body of the
 * neighbour loop of src/model/neighborlist.h:70-158.  Returns false when
 * the pair lies outside the plateau.
 *
 * Every force the reference adds for a pair -- LJPotForce at r, minus
 * LJPotForce at the plateau along the same direction, ChargePotForce at r,
 * minus ChargePotForce at the plateau (src/model/neighborlist.h:105-141,
 * src/model/forcefield.h:30-146) -- is a scalar times d / r^2 (the plateau
 * terms use ratio * d / r^2).  The scalars are summed first and the
 * direction is applied once: the same force up to rounding order.  Every
 * decision (plateau test, rmin2 branch, ratio bin, Coulomb switches) uses
 * the reference's quantities computed in the reference's order. */
__device__ __forceinline__ bool nl_pair(const DevNL& nl, const DevParams& P, uint32_t lig_type,
		float qlig, float px, float py, float pz, float rx, float ry, float rz, float rq,
		uint32_t trec, float& fx, float& fy, float& fz, float& e) {
	const float dx = fsub(px, rx), dy = fsub(py, ry), dz = fsub(pz, rz);
	const float dr2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
	if (!(dr2 <= nl.dPlateau2) || trec == 0) return false;
	/* 1/r^2 only scales smooth terms: its one decision, the Coulomb cutoff
	 * at 1/r^2 = 1/50^2 (src/model/forcefield.h:104-113), lies outside any
	 * plateau below 50 A, where nl.approx_inv allows the hardware reciprocal */
	const float dr2_inv = nl.approx_inv ? frcp_approx(dr2) : __frcp_rn(dr2);
	const bool shape86 = P.potshape == GBA_POTSHAPE_8_6;
	const size_t k = (size_t)P.num_types * (lig_type - 1) + (trec - 1);
	const float4 p = __ldg(&P.pair[2 * k]);
	const float4 pl = __ldg(&P.pair[2 * k + 1]);   /* ipon, plateau force factor, plateau energy */
	/* LJPotForce: energy and the radial factor fb (force = fb * d / r^2) */
	const float rr23 = fmul(fmul(dr2_inv, dr2_inv), dr2_inv);
	const float rep = fmul(p.x, shape86 ? dr2_inv : rr23);
	const float vlj = fmul(fsub(rep, p.y), rr23);
	float fb = ffma(6.0f, vlj, fmul(shape86 ? 2.0f : 6.0f, fmul(rep, rr23)));
	if (dr2 < p.z) {
		e = ffma(fsub(pl.x, 1.0f), p.w, vlj);
	} else {
		e = fmul(pl.x, vlj);
		fb = fmul(pl.x, fb);
	}
	/* getRatio's table bin, src/model/NLGrid.h:141-143 */
	const int bin = (int)fmul(dr2, 10000.0f);
	const float ratio = nl.ratio_computed
			? fsqrt_approx(fmul(fadd((float)bin, 0.5f), nl.ratio_scale))
			: __ldg(&nl.ratio[bin]);
	/* minus LJPotForce at the plateau (per type pair, precomputed) */
	float s = ffma(-pl.y, ratio, fb);
	e = fsub(e, pl.z);
	const float qq = fmul(fmul(qlig, rq), P.ffelec);
	if (fabsf(qq) > 0.001f) {
		/* ChargePotForce at r minus at the plateau: energy qq * dd when
		 * dd > 0, radial factor 2 qq / r^2 (distance-dependent dielectric)
		 * or qq / r (constant dielectric) */
		float d1, f1, d2, f2;
		if (P.dielec == GBA_DIELEC_CONSTANT) {
			const float sr = __fsqrt_rn(dr2_inv), sp = __fsqrt_rn(nl.dPlateau2_inv);
			d1 = fsub(sr, 0.02f); f1 = sr;
			d2 = fsub(sp, 0.02f); f2 = sp;
		} else {
			d1 = fsub(dr2_inv, 4.0e-4f); f1 = fmul(2.0f, dr2_inv);
			d2 = fsub(nl.dPlateau2_inv, 4.0e-4f); f2 = fmul(2.0f, nl.dPlateau2_inv);
		}
		if (d1 > 0.0f) {
			e = fadd(e, fmul(qq, d1));
			s = ffma(qq, f1, s);
		}
		if (d2 > 0.0f) {
			e = fsub(e, fmul(qq, d2));
			s = ffma(-fmul(qq, f2), ratio, s);
		}
	}
	const float sr2 = fmul(s, dr2_inv);
	fx = fmul(sr2, dx); fy = fmul(sr2, dy); fz = fmul(sr2, dz);
	return true;
}

/* Pair term of a flattened pair owned by slot s against receptor bead record
 * r (x, y, z, q) of type trec: adds it to S. */
__device__ __forceinline__ void pair_term(const RigidModel& M, const WarpStage& W, uint32_t s, float4 r,
		uint32_t trec, PoseSums& S) {
	const float4 b = W.pq[s];
	const float4 u = W.ut[s];
	float fx, fy, fz, e;
	if (nl_pair(M.grid.nl, M.par, __float_as_uint(u.w), b.w, b.x, b.y, b.z, r.x, r.y, r.z, r.w, trec, fx, fy,
			fz, e))
		S.add(e, fx, fy, fz, u.x, u.y, u.z);
}

/* Per-pose counters of the census (CENSUS instantiations only). */
struct RoundCensus {
	uint32_t grid = 0, charged = 0, nl = 0, ent = 0;
};

/* One round: beads [i0, i0 + 64) of the pose staged in W, added to the
 * lane sums S. */
template <bool CENSUS>
__device__ __forceinline__ void eval_round(const RigidModel& M, uint32_t i0, int lane, WarpStage& W,
		RoundCensus& cen, PoseSums& S) {
	/* 1. stage 64 beads, two per lane: lane, then lane + 32 */
	float ttx, tty, ttz;
	const PoseRot R = get_pose(W, ttx, tty, ttz);
	uint32_t nlk[2], nln[2];
	BeadGrid bg[2];
#pragma unroll
	for (int h = 0; h < 2; ++h) {
		const int s = lane + 32 * h;
		const uint32_t i = i0 + s;
		nlk[h] = 0;
		nln[h] = 0;
		bg[h] = BeadGrid{0u, 0u};
		bool in_nl = false;
		if (i < M.lig.n) {
			const float4 b = __ldg(&M.lig.xyzq[i]);
			const uint32_t tm = __ldg(&M.lig.tm[i]);
			const uint32_t type = tm & 0xffffu, mapped = tm >> 16;
			float px, py, pz;
			rot_apply(R.m, b.x, b.y, b.z, px, py, pz);
			px = fadd(px, ttx); py = fadd(py, tty); pz = fadd(pz, ttz);
			put_bead(W, s, b.x, b.y, b.z, px, py, pz, b.w, type);
			nlk[h] = stage_grid(M.grid, px, py, pz, mapped, b.w, s, W, bg[h]);
			if (type != 0) nln[h] = stage_nl(M.grid.nl, px, py, pz, s, W, in_nl);
		}
		if (CENSUS) {
			cen.grid += nlk[h] > 0;
			cen.charged += nlk[h] > 1;
			cen.nl += in_nl;
			cen.ent += nln[h];
		}
	}
	const uint32_t n_look = queue_lookups(W, nlk, bg, lane);
	uint32_t start[2];
	const uint32_t n_pair = queue_pairs(W, nln, lane, start);
	__syncwarp();

	/* 2. neighbour pairs, two per lane and window so that both gather
	 * chains (list entry -> receptor bead -> parameters) are in flight
	 * together, the next window's list entries already on their way */
	PairWindow win;
	/* list entries of the next window are loaded while this one is
	 * computed; typed entries carry the receptor type in bits 24..31 */
	const uint32_t* lst = M.grid.nl.typed_list ? M.grid.nl.typed_list : M.grid.nl.list;
	const bool typed = M.grid.nl.typed_list != nullptr;
	uint32_t sa = 0, sb = 0, ea = 0, eb = 0;
	if (n_pair > 0) {
		win.owners(W, 0, start, nln, lane, sa, sb);
		if ((uint32_t)lane < n_pair) ea = __ldg(&lst[W.lbase[sa] + lane]);
		if ((uint32_t)lane + 32 < n_pair) eb = __ldg(&lst[W.lbase[sb] + lane + 32]);
	}
	for (uint32_t w = 0; w < n_pair; w += 64) {
		const uint32_t k = w + lane, k2 = k + 32;
		const uint32_t csa = sa, csb = sb, cea = ea, ceb = eb;
		if (w + 64 < n_pair) {
			win.owners(W, w + 64, start, nln, lane, sa, sb);
			if (k + 64 < n_pair) ea = __ldg(&lst[W.lbase[sa] + k + 64]);
			if (k2 + 64 < n_pair) eb = __ldg(&lst[W.lbase[sb] + k2 + 64]);
		}
		if (k >= n_pair) continue;
		const bool has2 = k2 < n_pair;
		const uint32_t eb2 = has2 ? ceb : cea;
		const uint32_t ja = typed ? cea & 0xffffffu : cea;
		const uint32_t jb = typed ? eb2 & 0xffffffu : eb2;
		const float4 ra = __ldg(&M.rec.xyzq[ja]);
		const float4 rb = __ldg(&M.rec.xyzq[jb]);
		const uint32_t ta = typed ? cea >> 24 : __ldg(&M.rec.tm[ja]) & 0xffffu;
		const uint32_t tb = typed ? eb2 >> 24 : __ldg(&M.rec.tm[jb]) & 0xffffu;
		pair_term(M, W, csa, ra, ta, S);
		if (has2) pair_term(M, W, csb, rb, tb, S);
	}

	/* 3. grid lookups (cooperative sums folded per round) */
	{
		CoopSums Cr;
		drain_lookups(M.grid, W, n_look, lane, S, Cr);
		fold_coop(Cr, S, lane);
	}
	__syncwarp();
}

/* Reduce-scatter of a round's lane sums over the warp in a fixed butterfly:
 * lane l returns component l >> 1 of (E, Fx, Fy, Fz, T[0..8], 0, 0, 0)
 * summed over all 32 lanes (lanes 2c and 2c + 1 hold the same value). */
__device__ __forceinline__ float round_reduce(const PoseSums& S, int lane) {
	const float v[16] = {S.E, S.Fx, S.Fy, S.Fz, S.T[0], S.T[1], S.T[2], S.T[3], S.T[4], S.T[5], S.T[6],
			S.T[7], S.T[8], 0.f, 0.f, 0.f};
	const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4, b1 = lane & 2;
	float m8[8];
#pragma unroll
	for (int j = 0; j < 8; ++j)
		m8[j] = fadd(b4 ? v[8 + j] : v[j], __shfl_xor_sync(GBA_FULL_MASK, b4 ? v[j] : v[8 + j], 16));
	float m4[4];
#pragma unroll
	for (int j = 0; j < 4; ++j)
		m4[j] = fadd(b3 ? m8[4 + j] : m8[j], __shfl_xor_sync(GBA_FULL_MASK, b3 ? m8[j] : m8[4 + j], 8));
	float m2[2];
#pragma unroll
	for (int j = 0; j < 2; ++j)
		m2[j] = fadd(b2 ? m4[2 + j] : m4[j], __shfl_xor_sync(GBA_FULL_MASK, b2 ? m4[j] : m4[2 + j], 4));
	const float m1 = fadd(b1 ? m2[1] : m2[0], __shfl_xor_sync(GBA_FULL_MASK, b1 ? m2[0] : m2[1], 2));
	return fadd(m1, __shfl_xor_sync(GBA_FULL_MASK, m1, 1));
}

/* Clears the warp's round totals. */
__device__ __forceinline__ void clear_totals(WarpStage& W, int lane) {
	if (lane < 16) W.tot[lane] = 0.f;
	__syncwarp();
}

/* Adds a round's component (lane 2c holds component c) to the totals. */
__device__ __forceinline__ void add_round(WarpStage& W, float v, int lane) {
	if ((lane & 1) == 0) W.tot[lane >> 1] = fadd(W.tot[lane >> 1], v);
}

/* The pose result from the round totals: ForceLim on the force sum and the
 * TorqueMat contraction, on every lane. */
__device__ __forceinline__ void finish_pose(const WarpStage& W, float res[7]) {
	__syncwarp();
	const volatile float* t = W.tot;
	float c[13];
#pragma unroll
	for (int k = 0; k < 13; ++k) c[k] = t[k];
	float sFx = c[1], sFy = c[2], sFz = c[3];
	force_lim(sFx, sFy, sFz);
	float ang[3];
	float ttx, tty, ttz;
	torque_reduce(get_pose(W, ttx, tty, ttz), c + 4, ang);
	res[0] = c[0]; res[1] = sFx; res[2] = sFy; res[3] = sFz;
	res[4] = ang[0]; res[5] = ang[1]; res[6] = ang[2];
}

/* res: E, force xyz, Euler gradient xyz (Result_6D order); identical on all
 * lanes.  W is this warp's shared staging area.  ROUNDWISE selects the
 * round-wise summation order (see the file comment). */
template <bool CENSUS, bool ROUNDWISE = false>
__device__ __forceinline__ void eval_pose_rigid(const RigidModel& M, float tx, float ty, float tz,
		float a0, float a1, float a2, int lane, WarpStage& W, float res[7], PoseCensus* census) {
	put_pose(W, pose_rotation(a0, a1, a2, lane, M.trig), tx, ty, tz, lane);
	RoundCensus cen;
	if (ROUNDWISE) {
		clear_totals(W, lane);
		for (uint32_t i0 = 0; i0 < M.lig.n; i0 += kBeadsPerRound) {
			PoseSums S;
			eval_round<CENSUS>(M, i0, lane, W, cen, S);
			add_round(W, round_reduce(S, lane), lane);
		}
		finish_pose(W, res);
	} else {
		PoseSums S;
		for (uint32_t i0 = 0; i0 < M.lig.n; i0 += kBeadsPerRound) eval_round<CENSUS>(M, i0, lane, W, cen, S);
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
	}
	if (CENSUS) {
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			cen.grid += __shfl_xor_sync(GBA_FULL_MASK, cen.grid, o);
			cen.charged += __shfl_xor_sync(GBA_FULL_MASK, cen.charged, o);
			cen.nl += __shfl_xor_sync(GBA_FULL_MASK, cen.nl, o);
			cen.ent += __shfl_xor_sync(GBA_FULL_MASK, cen.ent, o);
		}
		if (lane == 0) *census = PoseCensus{cen.grid, cen.charged, cen.nl, cen.ent};
	}
}

/* ---- the reference CPU path's operation order (GBA_KOPT_REFERENCE_ORDER) ----
 *
 * CPUEnergyService6D evaluates a pose bead by bead: the bead's grid term
 * (type channel, then the charge channel times the charge), then its
 * neighbour list in list order, each pair adding LJPotForce at r, minus it at
 * the plateau, and (charged pairs) ChargePotForce at r, minus it at the
 * plateau, partly in double (src/model/neighborlist.h:70-158,
 * src/model/forcefield.h:30-146); then the bead forces and energies summed in
 * bead order (reducePotForce, reduceTorque, src/model/reduction.h:40-103).
 * These functions repeat that arithmetic operation for operation, so with the
 * same sin/cos the result equals the reference's bit for bit.  A lane walks a
 * bead's list by itself (no flattened pair windows) and the bead sums run on
 * 13 lanes sequentially, so this order is slower than the others; it is used
 * by the minimizers, the plain per-step form and gba_energy_6d when
 * GBA_KOPT_REFERENCE_ORDER is set. */

/* One channel of trilinearInterpolation (src/model/trilinIntrpl.h:29-66):
 * the corner products summed left to right in the order d000, d100, d010,
 * d001, d101, d011, d110, d111, then times 1/voxelVol.  elem as the lookup
 * queue encodes it (octet record, or first corner of the native layout). */
__device__ __forceinline__ float4 ref_channel(const DevIntrpl& g, uint32_t elem, const float* cw) {
	float4 d[8];
	if (g.oct) {
		const float4* b = g.oct + 8 * (size_t)elem;
#pragma unroll
		for (int c = 0; c < 8; ++c) d[c] = __ldg(b + c);
	} else {
		const float4* b = g.data + elem;
		const uint32_t sx = g.dimN[0], sxy = g.dimN[0] * g.dimN[1];
#pragma unroll
		for (int c = 0; c < 8; ++c) d[c] = __ldg(b + (c & 1) + sx * ((c >> 1) & 1) + sxy * (c >> 2));
	}
	/* corner c = x + 2 y + 4 z; the reference's order as corner indices */
	constexpr int ord[8] = {0, 1, 2, 4, 5, 6, 3, 7};
	float4 o = make_float4(fmul(d[0].x, cw[0]), fmul(d[0].y, cw[0]), fmul(d[0].z, cw[0]), fmul(d[0].w, cw[0]));
#pragma unroll
	for (int k = 1; k < 8; ++k) {
		const int c = ord[k];
		o.x = fadd(o.x, fmul(d[c].x, cw[c]));
		o.y = fadd(o.y, fmul(d[c].y, cw[c]));
		o.z = fadd(o.z, fmul(d[c].z, cw[c]));
		o.w = fadd(o.w, fmul(d[c].w, cw[c]));
	}
	return make_float4(fmul(o.x, g.voxelVol_inv), fmul(o.y, g.voxelVol_inv), fmul(o.z, g.voxelVol_inv),
			fmul(o.w, g.voxelVol_inv));
}

/* potForce of one bead at (px, py, pz) staged in slot s (its corner weights
 * go to the slot): the type channel, plus the charge channel times q when
 * |q| > 0.001, summed as interpolate does (src/model/interpolation.h:27-53);
 * zero outside both grids or for mapped type 0. */
__device__ __forceinline__ float4 ref_grid_term(const DevGrid& G, float px, float py, float pz, uint32_t mapped,
		float q, int s, WarpStage& W) {
	BeadGrid bg{0u, 0u};
	const uint32_t nlk = stage_grid(G, px, py, pz, mapped, q, s, W, bg);
	float4 pot = make_float4(0.f, 0.f, 0.f, 0.f);
	if (nlk > 0) {
		const float* cw = W.cw + kCornerStride * s;
		const DevIntrpl& g = (bg.t & 0x80000000u) ? G.outer : G.inner;
		pot = ref_channel(g, bg.t & 0x7fffffffu, cw);
		if (nlk > 1) {
			float4 el = ref_channel(g, bg.q & 0x7fffffffu, cw);
			el.x = fmul(el.x, q); el.y = fmul(el.y, q); el.z = fmul(el.z, q); el.w = fmul(el.w, q);
			pot.x = fadd(pot.x, el.x); pot.y = fadd(pot.y, el.y); pot.z = fadd(pot.z, el.z);
			pot.w = fadd(pot.w, el.w);
		}
	}
	return pot;
}

/* LJPotForce (swi = 1) as the reference computes it: the force factor in
 * double, rounded to float. */
__device__ __forceinline__ void ref_lj(float dr2, float dr2_inv, float dx, float dy, float dz, const float4 p,
		float ivor, bool shape86, float& fx, float& fy, float& fz, float& e) {
	const float rr23 = fmul(fmul(dr2_inv, dr2_inv), dr2_inv);
	const float rrd = shape86 ? dr2_inv : rr23;
	const float sd = shape86 ? 2.0f : 6.0f;
	const float rep = fmul(p.x, rrd);
	const float vlj = fmul(fsub(rep, p.y), rr23);
	const double sum = __dadd_rn(__dmul_rn(6.0, (double)vlj), (double)fmul(sd, fmul(rep, rr23)));
	float fb;
	if (dr2 < p.z) {
		e = fadd(vlj, fmul(fsub(ivor, 1.0f), p.w));
		fb = (float)sum;
	} else {
		e = fmul(ivor, vlj);
		fb = (float)__dmul_rn((double)ivor, sum);
	}
	fx = fmul(fb, dx); fy = fmul(fb, dy); fz = fmul(fb, dz);
}

/* ChargePotForce (swi = 1) as the reference computes it. */
__device__ __forceinline__ void ref_coulomb(float dr2_inv, float dx, float dy, float dz, float qq, bool cdiel,
		float& fx, float& fy, float& fz, float& e) {
	float dd;
	if (cdiel) dd = (float)__dsub_rn((double)__fsqrt_rn(dr2_inv), 1.0 / 50.0);
	else dd = (float)__dsub_rn((double)dr2_inv, 1.0 / (50.0 * 50.0));
	if (dd < 0.0f) dd = 0.0f;
	e = fmul(qq, dd);
	if (dd <= 0.0f) {
		fx = fy = fz = 0.0f;
		return;
	}
	/* (float)(et2 * (double)d) of two floats is the single-precision product
	 * (the double product is exact); the distance-dependent 2 et2 likewise
	 * wherever 2 et2 is finite in single precision */
	if (cdiel) {
		const float et2 = fmul(qq, __fsqrt_rn(dr2_inv));
		fx = fmul(et2, dx); fy = fmul(et2, dy); fz = fmul(et2, dz);
	} else {
		const float et2 = fmul(2.0f, fmul(qq, dr2_inv));
		if (isfinite(et2)) {
			fx = fmul(et2, dx); fy = fmul(et2, dy); fz = fmul(et2, dz);
		} else {
			const double d2 = __dmul_rn(2.0, (double)fmul(qq, dr2_inv));
			fx = (float)__dmul_rn(d2, (double)dx);
			fy = (float)__dmul_rn(d2, (double)dy);
			fz = (float)__dmul_rn(d2, (double)dz);
		}
	}
}

/* The four sub-terms NLPotForce adds for one pair -- LJPotForce at r, at the
 * plateau, ChargePotForce at r, at the plateau -- each (fx, fy, fz, E), for
 * the 32 pairs of a window (flags bit 0: the pair is within the plateau,
 * bit 1: its charge product passes the Coulomb test); the neighbour-list
 * accumulator of each of the round's 64 beads, component c in acc[s][c];
 * and the window's segments (runs of pairs of one bead): first position and
 * bead slot of segment j.  Overlaid on the staging area's corner weights and
 * lookup queue, which the reference order does not use once the round's grid
 * terms are taken. */
struct RefTerms {
	float4 t[32][4];
	uint32_t flags[32];
	float acc[64][4];
	uint8_t seg_pos[33];
	uint8_t seg_slot[32];
};
static_assert(sizeof(RefTerms) <= sizeof(WarpStage::cw) + sizeof(WarpStage::look), "RefTerms overlay");
static_assert(offsetof(WarpStage, look) == offsetof(WarpStage, cw) + sizeof(WarpStage::cw), "RefTerms overlay");
static_assert(offsetof(WarpStage, cw) % 16 == 0, "RefTerms overlay");

__device__ __forceinline__ RefTerms& ref_terms(WarpStage& W) { return *reinterpret_cast<RefTerms*>(W.cw); }

/* The sub-terms of one pair -- ligand bead staged in slot sl, receptor bead
 * at r (x, y, z, charge) of type trec -- into window position b (the loop
 * body of NLPotForce, src/model/neighborlist.h:70-158). */
__device__ __forceinline__ void ref_pair_terms(const DevNL& nl, const DevParams& P, WarpStage& W, uint32_t sl,
		const float4 r, uint32_t trec, int b) {
	const float4 bq = W.pq[sl];
	const uint32_t tlig = __float_as_uint(W.ut[sl].w);
	float dx = fsub(bq.x, r.x), dy = fsub(bq.y, r.y), dz = fsub(bq.z, r.z);
	const float dr2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
	RefTerms& T = ref_terms(W);
	/* trec 0: no parameters (the reference would index before its table) */
	if (dr2 > nl.dPlateau2 || trec == 0) {
		T.flags[b] = 0;
		return;
	}
	const bool shape86 = P.potshape == GBA_POTSHAPE_8_6;
	const bool cdiel = P.dielec == GBA_DIELEC_CONSTANT;
	/* (float)(1.0 / (double)dr2): double rounding is harmless here, so this
	 * is the correctly rounded float reciprocal */
	const float inv = __frcp_rn(dr2);
	dx = fmul(dx, inv); dy = fmul(dy, inv); dz = fmul(dz, inv);
	const size_t kp = (size_t)P.num_types * (trec - 1) + (tlig - 1);
	const float4 p = __ldg(&P.lj[kp]);
	const float ivor = __ldg(&P.ivor[kp]);
	const float ratio = __ldg(&nl.ratio[(int)fmul(dr2, 10000.0f)]);
	float4 t;
	ref_lj(dr2, inv, dx, dy, dz, p, ivor, shape86, t.x, t.y, t.z, t.w);
	T.t[b][0] = t;
	const float rdx = fmul(ratio, dx), rdy = fmul(ratio, dy), rdz = fmul(ratio, dz);
	ref_lj(nl.dPlateau2, nl.dPlateau2_inv, rdx, rdy, rdz, p, ivor, shape86, t.x, t.y, t.z, t.w);
	T.t[b][1] = t;
	const float qq = fmul(fmul(bq.w, r.w), P.ffelec);
	/* fabs(qq) > 0.001 in double: 0.001f is the first float above 0.001 */
	const bool charged = fabsf(qq) >= 0.001f;
	if (charged) {
		ref_coulomb(inv, dx, dy, dz, qq, cdiel, t.x, t.y, t.z, t.w);
		T.t[b][2] = t;
		ref_coulomb(nl.dPlateau2_inv, rdx, rdy, rdz, qq, cdiel, t.x, t.y, t.z, t.w);
		T.t[b][3] = t;
	}
	T.flags[b] = charged ? 3u : 1u;
}

/* Folds the n pairs of a window into their beads' accumulators in list
 * order.  Lane p (p < n) holds the slot of the bead owning pair p.  The
 * window's segments are numbered; four lanes take a segment, one component
 * each (the components' sums are independent), eight segments at a time. */
__device__ __forceinline__ void ref_fold(RefTerms& T, uint32_t n, uint32_t owner, int lane) {
	const uint32_t prev = __shfl_up_sync(GBA_FULL_MASK, owner, 1);
	const bool start = (uint32_t)lane < n && (lane == 0 || owner != prev);
	const uint32_t starts = __ballot_sync(GBA_FULL_MASK, start);
	const uint32_t nseg = __popc(starts);
	if (start) {
		const uint32_t j = __popc(starts & ((1u << lane) - 1u));
		T.seg_pos[j] = (uint8_t)lane;
		T.seg_slot[j] = (uint8_t)owner;
	}
	if (lane == 0) T.seg_pos[nseg] = (uint8_t)n;
	__syncwarp();
	const int c = lane & 3;
	for (uint32_t j = lane >> 2; j < nseg; j += 8) {
		const uint32_t lo = T.seg_pos[j], hi = T.seg_pos[j + 1], sl = T.seg_slot[j];
		float a = T.acc[sl][c];
		for (uint32_t k = lo; k < hi; ++k) {
			const uint32_t f = T.flags[k];
			if (!(f & 1u)) continue;
			const float* t = reinterpret_cast<const float*>(T.t[k]);
			a = fadd(a, t[c]);
			a = fsub(a, t[4 + c]);
			if (f & 2u) {
				a = fadd(a, t[8 + c]);
				a = fsub(a, t[12 + c]);
			}
		}
		T.acc[sl][c] = a;
	}
}

/* One round in the reference's order: for each of the 64 staged beads its
 * total (fx, fy, fz, E) -- grid term, plus the neighbour-list term for beads
 * that looked it up -- parked in the slot's first four weight floats
 * (W.cw[9 s .. 9 s + 3]).  The pair sub-terms are computed by the whole warp
 * over the round's flattened pair list, 32 pairs at a time (every lane busy,
 * which matters for the double-precision steps on GB300's narrow FP64 pipe),
 * and the sub-terms are then added to each bead's accumulator in list order,
 * four lanes per bead, one per component (ref_fold). */
__device__ __forceinline__ void eval_round_ref(const RigidModel& M, uint32_t i0, int lane, WarpStage& W) {
	float ttx, tty, ttz;
	const PoseRot R = get_pose(W, ttx, tty, ttz);
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
		if (i >= M.lig.n) continue;
		const float4 b = __ldg(&M.lig.xyzq[i]);
		const uint32_t tm = __ldg(&M.lig.tm[i]);
		const uint32_t type = tm & 0xffffu, mapped = tm >> 16;
		float px, py, pz;
		rot_apply(R.m, b.x, b.y, b.z, px, py, pz);
		px = fadd(px, ttx); py = fadd(py, tty); pz = fadd(pz, ttz);
		put_bead(W, s, b.x, b.y, b.z, px, py, pz, b.w, type);
		pot[h] = ref_grid_term(M.grid, px, py, pz, mapped, b.w, s, W);
		if (type != 0) nln[h] = stage_nl(M.grid.nl, px, py, pz, s, W, in_nl[h]);
	}
	uint32_t start[2];
	const uint32_t n_pair = queue_pairs(W, nln, lane, start);
	__syncwarp();   /* weights read, list bases final: the overlay may be written */
	RefTerms& T = ref_terms(W);
	if (n_pair > 0) {
#pragma unroll
		for (int k = 0; k < 8; ++k) (&T.acc[0][0])[lane + 32 * k] = 0.f;
	}

	const uint32_t* lst = M.grid.nl.typed_list ? M.grid.nl.typed_list : M.grid.nl.list;
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
				const bool typed = M.grid.nl.typed_list != nullptr;
				const uint32_t j = typed ? ent & 0xffffffu : ent;
				const uint32_t trec = typed ? ent >> 24 : __ldg(&M.rec.tm[j]) & 0xffffu;
				ref_pair_terms(M.grid.nl, M.par, W, half ? sb : sa, __ldg(&M.rec.xyzq[j]), trec, lane);
			}
			__syncwarp();
			ref_fold(T, min(n_pair - wb, 32u), half ? sb : sa, lane);
			__syncwarp();
		}
	}
	float4 acc[2];
#pragma unroll
	for (int h = 0; h < 2; ++h) {
		const int s = lane + 32 * h;
		acc[h] = n_pair > 0 ? make_float4(T.acc[s][0], T.acc[s][1], T.acc[s][2], T.acc[s][3])
		                    : make_float4(0.f, 0.f, 0.f, 0.f);
	}
	__syncwarp();   /* accumulators read: the totals may overwrite them */
#pragma unroll
	for (int h = 0; h < 2; ++h) {
		const int s = lane + 32 * h;
		if (i0 + s >= M.lig.n) continue;
		float4 v = pot[h];
		if (in_nl[h]) {
			v.x = fadd(v.x, acc[h].x); v.y = fadd(v.y, acc[h].y); v.z = fadd(v.z, acc[h].z);
			v.w = fadd(v.w, acc[h].w);
		}
		float* cw = W.cw + kCornerStride * s;
		cw[0] = v.x; cw[1] = v.y; cw[2] = v.z; cw[3] = v.w;
	}
	__syncwarp();
}

/* Adds the bead totals of slots 0 .. nb-1 of W to the running sums, in bead
 * order: lane c < 13 owns sum c (0 energy, 1..3 force, 4 + 3 a + b the
 * torque entry x_b f_a).  Returns the lane's updated sum. */
__device__ __forceinline__ float ref_accumulate(const WarpStage& W, uint32_t nb, int lane, float acc) {
	if (lane < 13) {
		const int a = (lane - 4) / 3, bb = (lane - 4) % 3;
		for (uint32_t s = 0; s < nb; ++s) {
			const float* f = W.cw + kCornerStride * s;
			if (lane == 0) {
				acc = fadd(acc, f[3]);
			} else if (lane < 4) {
				acc = fadd(acc, f[lane - 1]);
			} else {
				const float4 u = W.ut[s];
				const float ub = bb == 0 ? u.x : (bb == 1 ? u.y : u.z);
				acc = fadd(acc, fmul(ub, f[a]));
			}
		}
	}
	return acc;
}

/* The pose result from the running sums of lanes 0..12: ForceLim and the
 * TorqueMat contraction, on every lane. */
__device__ __forceinline__ void finish_ref(float acc, const WarpStage& W, float res[7]) {
	float c[13];
#pragma unroll
	for (int k = 0; k < 13; ++k) c[k] = __shfl_sync(GBA_FULL_MASK, acc, k);
	float sFx = c[1], sFy = c[2], sFz = c[3];
	force_lim(sFx, sFy, sFz);
	float ang[3];
	float ttx, tty, ttz;
	torque_reduce(get_pose(W, ttx, tty, ttz), c + 4, ang);
	res[0] = c[0]; res[1] = sFx; res[2] = sFy; res[3] = sFz;
	res[4] = ang[0]; res[5] = ang[1]; res[6] = ang[2];
}

/* A whole pose in the reference's order, one warp. */
__device__ __forceinline__ void eval_pose_rigid_ref(const RigidModel& M, float tx, float ty, float tz,
		float a0, float a1, float a2, int lane, WarpStage& W, float res[7]) {
	put_pose(W, pose_rotation(a0, a1, a2, lane, M.trig), tx, ty, tz, lane);
	float acc = 0.f;
	for (uint32_t i0 = 0; i0 < M.lig.n; i0 += kBeadsPerRound) {
		eval_round_ref(M, i0, lane, W);
		acc = ref_accumulate(W, min((uint32_t)kBeadsPerRound, M.lig.n - i0), lane, acc);
		__syncwarp();
	}
	finish_ref(acc, W, res);
}

/* Barrier of the `nthreads` threads that use barrier `id` (a named barrier:
 * a subset of the block's warps). */
__device__ __forceinline__ void group_sync(int id, int nthreads) {
	asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

/* One pose evaluated by a team of G warps (t = 0..G-1) that synchronize
 * with named barrier bar_id: warp t takes rounds t, t + G, t + 2G, ...;
 * after each group of G rounds the warps park their round components in
 * slots[16 t + c] and warp 0 adds them in round order -- the arithmetic of
 * eval_pose_rigid<_, true>, so the result is the same bit for bit.  Warp 0
 * computes the rotation (double sincos: GB300's FP64 pipe is narrow) and the
 * others copy it.  Every warp of the team must call it; res is valid in
 * warp 0.  stages: the G warps' staging areas. */
__device__ __forceinline__ void eval_pose_rigid_team(const RigidModel& M, float tx, float ty, float tz,
		float a0, float a1, float a2, int lane, int t, int G, WarpStage* stages, float* slots, float res[7],
		int bar_id) {
	const int nthreads = 32 * G;
	WarpStage& W = stages[t];
	if (t == 0) put_pose(W, pose_rotation(a0, a1, a2, lane, M.trig), tx, ty, tz, lane);
	group_sync(bar_id, nthreads);
	if (t != 0) {
		if (lane < 18) W.pose[lane] = stages[0].pose[lane];
		__syncwarp();
	}
	clear_totals(W, lane);
	const uint32_t rounds = (M.lig.n + kBeadsPerRound - 1) / kBeadsPerRound;
	RoundCensus cen;
	for (uint32_t r0 = 0; r0 < rounds; r0 += G) {
		const uint32_t r = r0 + t;
		if (r < rounds) {
			PoseSums S;
			eval_round<false>(M, r * kBeadsPerRound, lane, W, cen, S);
			const float v = round_reduce(S, lane);
			if ((lane & 1) == 0) slots[16 * t + (lane >> 1)] = v;
		}
		group_sync(bar_id, nthreads);
		if (t == 0)
			for (int u = 0; u < G && r0 + u < rounds; ++u) add_round(W, slots[16 * u + (lane >> 1)], lane);
		group_sync(bar_id, nthreads);
	}
	if (t == 0) finish_pose(W, res);
}

/* The reference order by a team of G warps (named barrier bar_id): warp t
 * evaluates rounds t, t + G, ... into its staging area's bead totals
 * (eval_round_ref); after each group of G rounds warp 0 adds them to the 13
 * running sums in round and bead order (ref_accumulate over each warp's
 * staging area) -- the arithmetic of eval_pose_rigid_ref, bit for bit.
 * Every warp of the team must call it; res is valid in warp 0. */
__device__ __forceinline__ void eval_pose_rigid_team_ref(const RigidModel& M, float tx, float ty, float tz,
		float a0, float a1, float a2, int lane, int t, int G, WarpStage* stages, float res[7], int bar_id) {
	const int nthreads = 32 * G;
	WarpStage& W = stages[t];
	if (t == 0) put_pose(W, pose_rotation(a0, a1, a2, lane, M.trig), tx, ty, tz, lane);
	group_sync(bar_id, nthreads);
	if (t != 0) {
		if (lane < 18) W.pose[lane] = stages[0].pose[lane];
		__syncwarp();
	}
	const uint32_t rounds = (M.lig.n + kBeadsPerRound - 1) / kBeadsPerRound;
	float acc = 0.f;
	for (uint32_t r0 = 0; r0 < rounds; r0 += G) {
		const uint32_t r = r0 + t;
		if (r < rounds) eval_round_ref(M, r * kBeadsPerRound, lane, W);
		group_sync(bar_id, nthreads);
		if (t == 0)
			for (int u = 0; u < G && r0 + u < rounds; ++u)
				acc = ref_accumulate(stages[u], min((uint32_t)kBeadsPerRound, M.lig.n - (r0 + u) * kBeadsPerRound),
						lane, acc);
		group_sync(bar_id, nthreads);
	}
	if (t == 0) finish_ref(acc, W, res);
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
