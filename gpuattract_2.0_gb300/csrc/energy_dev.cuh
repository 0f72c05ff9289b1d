/*
 * energy_dev.cuh -- device building blocks of the fused docking energy kernels.
 *
 * Numerical policy.  Every quantity that feeds a discrete decision -- the
 * rotation matrix, the transformed bead position, grid/NL voxel indices, the
 * inner/outer/NL bounds tests, r^2 against the plateau, the ratio-table index
 * and the Coulomb switch -- is computed with explicitly rounded, unfused FP32
 * operations in the reference's operation order, so indices and neighbour
 * sets are bit-identical to the reference CPU path.  The rotation angles go
 * through double-precision sincos rounded to float (the correctly rounded
 * value, which is what the host's sinf/cosf return).  The smooth arithmetic
 * after those decisions (trilinear sums, pair terms, reductions) may fuse.
 */
#ifndef GBA_ENERGY_DEV_CUH_
#define GBA_ENERGY_DEV_CUH_

#include "gba_internal.h"

namespace gba {

#define GBA_FULL_MASK 0xffffffffu

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

/* Rotation matrix and its sin/cos, one pose. */
struct PoseRot {
	float m[9];
	float cphi, sphi, cssi, sssi, crot, srot;
};

/* Lanes 0..2 each take one Euler angle (phi, ssi, rot) through double sincos;
 * the 6 values are broadcast and combined as euler2rotmat does
 * (src/model/matrixFunctions.h:40-77), unfused. */
__device__ __forceinline__ PoseRot pose_rotation(float phi, float ssi, float rot, int lane) {
	float a = lane == 0 ? phi : (lane == 1 ? ssi : rot);
	double sd = 0.0, cd = 1.0;
	if (lane < 3) sincos((double)a, &sd, &cd);
	float s = (float)sd, c = (float)cd;
	PoseRot R;
	R.cphi = __shfl_sync(GBA_FULL_MASK, c, 0);
	R.sphi = __shfl_sync(GBA_FULL_MASK, s, 0);
	R.cssi = __shfl_sync(GBA_FULL_MASK, c, 1);
	R.sssi = __shfl_sync(GBA_FULL_MASK, s, 1);
	R.crot = __shfl_sync(GBA_FULL_MASK, c, 2);
	R.srot = __shfl_sync(GBA_FULL_MASK, s, 2);
	const float cSSI_cPHI = fmul(R.cssi, R.cphi);
	const float cSSI_sPHI = fmul(R.cssi, R.sphi);
	const float sSSI_cPHI = fmul(R.sssi, R.cphi);
	const float sSSI_sPHI = fmul(R.sssi, R.sphi);
	R.m[0] = fadd(fmul(R.crot, cSSI_cPHI), fmul(R.srot, R.sphi));
	R.m[1] = fsub(fmul(R.srot, cSSI_cPHI), fmul(R.crot, R.sphi));
	R.m[2] = sSSI_cPHI;
	R.m[3] = fsub(fmul(R.crot, cSSI_sPHI), fmul(R.srot, R.cphi));
	R.m[4] = fadd(fmul(R.srot, cSSI_sPHI), fmul(R.crot, R.cphi));
	R.m[5] = sSSI_sPHI;
	R.m[6] = fmul(-R.crot, R.sssi);
	R.m[7] = fmul(-R.srot, R.sssi);
	R.m[8] = R.cssi;
	return R;
}

/* RotMat * Vec3 (src/commons/RotMat.h:170-176), unfused, left to right. */
__device__ __forceinline__ void rot_apply(const float m[9], float x, float y, float z,
		float& ox, float& oy, float& oz) {
	ox = fadd(fadd(fmul(m[0], x), fmul(m[1], y)), fmul(m[2], z));
	oy = fadd(fadd(fmul(m[3], x), fmul(m[4], y)), fmul(m[5], z));
	oz = fadd(fadd(fmul(m[6], x), fmul(m[7], y)), fmul(m[8], z));
}

/* outOfBounds_byPos, src/model/IntrplGrid.h:113-117, written as a negated
 * inside test so a NaN position counts as outside (the reference would index
 * with it). */
__device__ __forceinline__ bool grid_out(const DevIntrpl& g, float x, float y, float z) {
	return !((x >= g.pos[0]) & (x <= g.maxDim[0]) & (y >= g.pos[1]) & (y <= g.maxDim[1]) &
			(z >= g.pos[2]) & (z <= g.maxDim[2]));
}

/* NLGrid::outOfBounds(x,y,z), src/model/NLGrid.h:128-133, NaN-safe as above. */
__device__ __forceinline__ bool nl_out(const DevNL& g, float x, float y, float z) {
	return !((x >= g.pos[0]) & (x <= g.maxDim[0]) & (y >= g.pos[1]) & (y <= g.maxDim[1]) &
			(z >= g.pos[2]) & (z <= g.maxDim[2]));
}

/* One channel's trilinear interpolation at a voxel octet (unscaled). */
__device__ __forceinline__ float4 octet_lerp(const float4* __restrict__ base, uint32_t sx,
		uint32_t sxy, float pmn_x, float pmn_y, float pmn_z, float pmx_x, float pmx_y,
		float pmx_z) {
	const float4 d000 = __ldg(base);
	const float4 d100 = __ldg(base + 1);
	const float4 d010 = __ldg(base + sx);
	const float4 d110 = __ldg(base + sx + 1);
	const float4 d001 = __ldg(base + sxy);
	const float4 d101 = __ldg(base + sxy + 1);
	const float4 d011 = __ldg(base + sxy + sx);
	const float4 d111 = __ldg(base + sxy + sx + 1);
	const float tmax_xy = pmx_x * pmx_y;
	const float tmin_xy = pmn_x * pmn_y;
	const float w000 = tmax_xy * pmx_z;
	const float w100 = (pmn_x * pmx_y) * pmx_z;
	const float w010 = (pmx_x * pmn_y) * pmx_z;
	const float w001 = tmax_xy * pmn_z;
	const float w101 = (pmn_x * pmx_y) * pmn_z;
	const float w011 = (pmx_x * pmn_y) * pmn_z;
	const float w110 = tmin_xy * pmx_z;
	const float w111 = tmin_xy * pmn_z;
	float4 v;
#define GBA_TRI(c) v.c = d000.c * w000 + d100.c * w100 + d010.c * w010 + d001.c * w001 + \
		d101.c * w101 + d011.c * w011 + d110.c * w110 + d111.c * w111;
	GBA_TRI(x) GBA_TRI(y) GBA_TRI(z) GBA_TRI(w)
#undef GBA_TRI
	return v;
}

/* interpolate(), src/model/interpolation.h:27-53, with getIndex /
 * getVoxelByIndex of src/model/IntrplGrid.h:96-104,130-163.  Returns the
 * type channel plus (|q| > 0.001) q times the charge channel, scaled by
 * 1/voxelVol. */
__device__ __forceinline__ float4 grid_interpolate(const DevIntrpl& g, float px, float py,
		float pz, uint32_t mapped, float q, bool& charged) {
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
	const uint32_t sx = g.dimN[0];
	const uint32_t sxy = g.dimN[0] * g.dimN[1];
	const uint32_t N = sxy * g.dimN[2];
	const uint32_t off = sx * (iz * g.dimN[1] + iy) + ix;
	float4 pot = octet_lerp(g.data + (size_t)mapped * N + off, sx, sxy, pmn_x, pmn_y, pmn_z,
			pmx_x, pmx_y, pmx_z);
	pot.x *= g.voxelVol_inv; pot.y *= g.voxelVol_inv; pot.z *= g.voxelVol_inv; pot.w *= g.voxelVol_inv;
	charged = fabsf(q) > 0.001f;
	if (charged) {
		float4 el = octet_lerp(g.data + off, sx, sxy, pmn_x, pmn_y, pmn_z, pmx_x, pmx_y, pmx_z);
		pot.x += (el.x * g.voxelVol_inv) * q;
		pot.y += (el.y * g.voxelVol_inv) * q;
		pot.z += (el.z * g.voxelVol_inv) * q;
		pot.w += (el.w * g.voxelVol_inv) * q;
	}
	return pot;
}

/* potForce's inner/outer selection for one bead, src/model/interpolation.h:57-101.
 * Returns false when the bead lies outside both grids or has channel 0. */
__device__ __forceinline__ bool bead_grid_term(const DevGrid& G, float px, float py, float pz,
		uint32_t mapped, float q, float4& pot, bool& charged) {
	charged = false;
	if (mapped == 0) return false;
	if (!grid_out(G.inner, px, py, pz)) {
		pot = grid_interpolate(G.inner, px, py, pz, mapped, q, charged);
		return true;
	}
	if (!grid_out(G.outer, px, py, pz)) {
		pot = grid_interpolate(G.outer, px, py, pz, mapped, q, charged);
		return true;
	}
	return false;
}

/* LJPotForce, src/model/forcefield.h:30-83, swi = 1. */
__device__ __forceinline__ void lj_pot_force(float dr2, float dr2_inv, float dx, float dy,
		float dz, const float4 p, float ivor, bool shape86, float& fx, float& fy, float& fz,
		float& e) {
	const float rr23 = dr2_inv * dr2_inv * dr2_inv;
	const float rrd = shape86 ? dr2_inv : rr23;
	const float sd = shape86 ? 2.0f : 6.0f;
	const float rep = p.x * rrd;
	const float vlj = (rep - p.y) * rr23;
	float fb = 6.0f * vlj + sd * (rep * rr23);
	if (dr2 < p.z) {
		e = vlj + (ivor - 1.0f) * p.w;
	} else {
		e = ivor * vlj;
		fb = ivor * fb;
	}
	fx = fb * dx; fy = fb * dy; fz = fb * dz;
}

/* ChargePotForce, src/model/forcefield.h:87-146, swi = 1. */
__device__ __forceinline__ void charge_pot_force(float dr2_inv, float dx, float dy, float dz,
		float qq, bool constant_dielec, float& fx, float& fy, float& fz, float& e) {
	if (constant_dielec) {
		const float sr = sqrtf(dr2_inv);
		float dd = sr - 0.02f;
		if (dd <= 0.0f) { e = 0.0f; fx = fy = fz = 0.0f; return; }
		e = qq * dd;
		const float et2 = qq * sr;
		fx = et2 * dx; fy = et2 * dy; fz = et2 * dz;
	} else {
		float dd = dr2_inv - 4.0e-4f;
		if (dd <= 0.0f) { e = 0.0f; fx = fy = fz = 0.0f; return; }
		e = qq * dd;
		const float et2 = 2.0f * (qq * dr2_inv);
		fx = et2 * dx; fy = et2 * dy; fz = et2 * dz;
	}
}

/* Neighbour-list pair term of one ligand bead, NLPotForce's body
 * (src/model/neighborlist.h:59-165).  Receptor positions come from
 * rec_xyzq (rigid) or from `defo` when non-null (per-pose deformed receptor,
 * neighborlist_modes.h); receptor reaction forces go through `on_pair` when
 * requested.  Adds into f/e; returns the voxel's numEl (0 when outside). */
struct NoPairHook {
	__device__ __forceinline__ void operator()(uint32_t, float, float, float) const {}
};

template <typename RecPos, typename PairHook>
__device__ __forceinline__ uint32_t bead_nl_term(const DevNL& nl, const DevParams& P,
		const uint32_t* __restrict__ rec_tm, const RecPos& recpos, float px, float py, float pz,
		uint32_t lig_type, float qlig, float& fx, float& fy, float& fz, float& e,
		uint32_t& npairs, const PairHook& hook) {
	if (nl_out(nl, px, py, pz)) return 0;
	/* getIndex (round half away from zero); inside the bounds the result lies in
	 * [0, dimN-1] already, the clamp only guards the index arithmetic */
	const int ix = min(max((int)roundf(fmul(fsub(px, nl.pos[0]), nl.dVox_inv)), 0), (int)nl.dimN[0] - 1);
	const int iy = min(max((int)roundf(fmul(fsub(py, nl.pos[1]), nl.dVox_inv)), 0), (int)nl.dimN[1] - 1);
	const int iz = min(max((int)roundf(fmul(fsub(pz, nl.pos[2]), nl.dVox_inv)), 0), (int)nl.dimN[2] - 1);
	const uint2 d = __ldg(&nl.grid[nl.dimN[0] * (iz * nl.dimN[1] + iy) + ix]);
	const bool shape86 = P.potshape == GBA_POTSHAPE_8_6;
	const bool cdiel = P.dielec == GBA_DIELEC_CONSTANT;
	const float4* __restrict__ ljrow = P.lj + (lig_type - 1);
	const float* __restrict__ ivrow = P.ivor + (lig_type - 1);
	float ax = 0.f, ay = 0.f, az = 0.f, ae = 0.f;
	for (uint32_t j = 0; j < d.x; ++j) {
		const uint32_t nIdx = __ldg(&nl.list[d.y + j]);
		float rx, ry, rz, rq;
		recpos(nIdx, rx, ry, rz, rq);
		float dx = fsub(px, rx), dy = fsub(py, ry), dz = fsub(pz, rz);
		const float dr2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
		/* outOfPlateau (src/model/NLGrid.h:136-138); NaN counts as outside */
		if (!(dr2 <= nl.dPlateau2)) continue;
		const uint32_t trec = __ldg(&rec_tm[nIdx]) & 0xffffu;
		if (trec == 0) continue;   /* the reference asserts atomTypeRec > 0 */
		++npairs;
		const float dr2_inv = __frcp_rn(dr2);
		dx *= dr2_inv; dy *= dr2_inv; dz *= dr2_inv;
		const size_t k = (size_t)P.num_types * (trec - 1);
		const float4 p = __ldg(&ljrow[k]);
		const float iv = __ldg(&ivrow[k]);
		float f1x, f1y, f1z, e1;
		lj_pot_force(dr2, dr2_inv, dx, dy, dz, p, iv, shape86, f1x, f1y, f1z, e1);
		const float ratio = __ldg(&nl.ratio[(int)fmul(dr2, 10000.0f)]);
		const float rdx = ratio * dx, rdy = ratio * dy, rdz = ratio * dz;
		float f2x, f2y, f2z, e2;
		lj_pot_force(nl.dPlateau2, nl.dPlateau2_inv, rdx, rdy, rdz, p, iv, shape86, f2x, f2y, f2z, e2);
		float px_ = f1x - f2x, py_ = f1y - f2y, pz_ = f1z - f2z, pe = e1 - e2;
		const float qq = fmul(fmul(qlig, rq), P.ffelec);
		if (fabsf(qq) > 0.001f) {
			float c1x, c1y, c1z, c1e, c2x, c2y, c2z, c2e;
			charge_pot_force(dr2_inv, dx, dy, dz, qq, cdiel, c1x, c1y, c1z, c1e);
			charge_pot_force(nl.dPlateau2_inv, rdx, rdy, rdz, qq, cdiel, c2x, c2y, c2z, c2e);
			px_ += c1x - c2x; py_ += c1y - c2y; pz_ += c1z - c2z; pe += c1e - c2e;
		}
		ax += px_; ay += py_; az += pz_; ae += pe;
		hook(nIdx, px_, py_, pz_);
	}
	fx += ax; fy += ay; fz += az; e += ae;
	return d.x;
}

/* Butterfly sum across the warp. */
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(GBA_FULL_MASK, v, o);
	return v;
}

/* euler2torquemat (src/model/matrixFunctions.h:81-127) contracted with the
 * torque matrix T (TorqueMat::rotateReduce, src/commons/TorqueMat.h:27-37). */
__device__ __forceinline__ void torque_reduce(const PoseRot& R, const float T[9], float out[3]) {
	const float cSSI_cPHI = R.cssi * R.cphi, cSSI_sPHI = R.cssi * R.sphi;
	const float sSSI_cPHI = R.sssi * R.cphi, sSSI_sPHI = R.sssi * R.sphi;
	const float cROT = R.crot, sROT = R.srot, cPHI = R.cphi, sPHI = R.sphi;
	const float cSSI = R.cssi, sSSI = R.sssi;
	float M[3][3][3];
	M[0][0][0] = -cROT * cSSI_sPHI + sROT * cPHI;
	M[0][0][1] = -sROT * cSSI_sPHI - cROT * cPHI;
	M[0][0][2] = -sSSI_sPHI;
	M[1][0][0] = cROT * cSSI_cPHI + sROT * sPHI;
	M[1][0][1] = sROT * cSSI_cPHI - cROT * sPHI;
	M[1][0][2] = sSSI_cPHI;
	M[2][0][0] = 0.f; M[2][0][1] = 0.f; M[2][0][2] = 0.f;
	M[0][1][0] = -cROT * sSSI_cPHI;
	M[0][1][1] = -sROT * sSSI_cPHI;
	M[0][1][2] = cSSI_cPHI;
	M[1][1][0] = -cROT * sSSI_sPHI;
	M[1][1][1] = -sROT * sSSI_sPHI;
	M[1][1][2] = cSSI_sPHI;
	M[2][1][0] = -cROT * cSSI;
	M[2][1][1] = -sROT * cSSI;
	M[2][1][2] = -sSSI;
	M[0][2][0] = -sROT * cSSI_cPHI + cROT * sPHI;
	M[0][2][1] = cROT * cSSI_cPHI + sROT * sPHI;
	M[0][2][2] = 0.f;
	M[1][2][0] = -sROT * cSSI_sPHI - cROT * cPHI;
	M[1][2][1] = cROT * cSSI_sPHI - sROT * cPHI;
	M[1][2][2] = 0.f;
	M[2][2][0] = sROT * sSSI;
	M[2][2][1] = -cROT * sSSI;
	M[2][2][2] = 0.f;
	float rx = 0.f, ry = 0.f, rz = 0.f;
#pragma unroll
	for (int k = 0; k < 3; ++k)
#pragma unroll
		for (int l = 0; l < 3; ++l) {
			rx += M[k][0][l] * T[3 * k + l];
			ry += M[k][1][l] * T[3 * k + l];
			rz += M[k][2][l] * T[3 * k + l];
		}
	out[0] = rx; out[1] = ry; out[2] = rz;
}

/* ForceLim clamp of reducePotForce, src/model/reduction.h:60-72 (x0.01 in
 * double, at most three times). */
__device__ __forceinline__ void force_lim(float& x, float& y, float& z) {
#pragma unroll
	for (int i = 0; i < 3; ++i) {
		const float magn2 = fadd(fadd(fmul(x, x), fmul(y, y)), fmul(z, z));
		if (magn2 > 1.0e18f) {
			x = (float)((double)x * 0.01);
			y = (float)((double)y * 0.01);
			z = (float)((double)z * 0.01);
		}
	}
}

}  // namespace gba

#endif
