/*
 * energy_dev.cuh -- device building blocks of the fused docking energy kernels.
 *
 * Numerical policy.  Every quantity that feeds a discrete decision -- the
 * rotation matrix, the transformed bead position, grid/NL voxel indices, the
 * inner/outer/NL bounds tests, r^2 against the plateau, the ratio-table index
 * and the Coulomb switch -- is computed with explicitly rounded, unfused FP32
 * operations in the reference's operation order, so indices and neighbour
 * sets are bit-identical to the reference CPU path.  The rotation angles go
 * through double-precision sincos rounded to float: the correctly rounded
 * value, which glibc's sinf/cosf return for all but about 1% of arguments
 * (where they are off by one ulp) -- or, with gba_set_host_sincos, the host
 * C library's own sinf/cosf values read from a table.  The smooth arithmetic after those
 * decisions (trilinear sums, pair terms, reductions) may fuse.
 */
#ifndef GBA_ENERGY_DEV_CUH_
#define GBA_ENERGY_DEV_CUH_

#include "gba_internal.h"

namespace gba {

#define GBA_FULL_MASK 0xffffffffu

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

/* Hardware reciprocal and square root (rcp/sqrt.approx: within about one
 * ulp; deterministic, the same bits in every kernel). */
__device__ __forceinline__ float frcp_approx(float x) {
	float r;
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
	return r;
}
__device__ __forceinline__ float fsqrt_approx(float x) {
	float r;
	asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
	return r;
}

/* Rotation matrix and its sin/cos, one pose. */
struct PoseRot {
	float m[9];
	float cphi, sphi, cssi, sssi, crot, srot;
};

/* Lanes 0..2 each take one Euler angle (phi, ssi, rot) through double sincos
 * -- or, for angles the host table T covers, the host C library's sinf/cosf
 * read from it; the 6 values are broadcast and combined as euler2rotmat does
 * (src/model/matrixFunctions.h:40-77), unfused. */
__device__ __forceinline__ PoseRot pose_rotation(float phi, float ssi, float rot, int lane, const DevTrig& T) {
	float a = lane == 0 ? phi : (lane == 1 ? ssi : rot);
	float s = 0.f, c = 1.f;
	if (lane < 3) {
		const uint32_t b = __float_as_uint(a), mag = b & 0x7fffffffu;
		if (T.sc && mag >= T.lo && mag < T.hi) {
			const float2 v = __ldg(&T.sc[(size_t)(b >> 31) * (T.hi - T.lo) + (mag - T.lo)]);
			s = v.x;
			c = v.y;
		} else {
			double sd, cd;
			sincos((double)a, &sd, &cd);
			s = (float)sd;
			c = (float)cd;
		}
	}
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

/* Transposed RotMat * Vec3 (R^T v), unfused, left to right. */
__device__ __forceinline__ void rot_apply_t(const float m[9], float x, float y, float z,
		float& ox, float& oy, float& oz) {
	ox = fadd(fadd(fmul(m[0], x), fmul(m[3], y)), fmul(m[6], z));
	oy = fadd(fadd(fmul(m[1], x), fmul(m[4], y)), fmul(m[7], z));
	oz = fadd(fadd(fmul(m[2], x), fmul(m[5], y)), fmul(m[8], z));
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

/* Read-only load that does not allocate in L1 (the line still goes through
 * L2): grid corners are streamed, so L1 stays with the receptor and
 * parameter data the pair term re-reads. */
__device__ __forceinline__ float4 ldg_no_l1(const float4* p) {
	float4 v;
	asm("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
			: "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
			: "l"(p));
	return v;
}

/* Trilinear weight of octet corner c (x = bit 0, y = bit 1, z = bit 2), the
 * products of src/model/trilinIntrpl.h:29-66: (wx * wy) * wz with w = pos -
 * min on the corner's high side and max - pos on its low side. */
__device__ __forceinline__ float corner_weight(int c, float pmn_x, float pmn_y, float pmn_z,
		float pmx_x, float pmx_y, float pmx_z) {
	return fmul(fmul((c & 1) ? pmn_x : pmx_x, (c & 2) ? pmn_y : pmx_y), (c & 4) ? pmn_z : pmx_z);
}

/* Sum of the eight corner products p[c] in the fixed pairwise order
 * ((p0 + p1) + (p2 + p3)) + ((p4 + p5) + (p6 + p7)) -- the order the
 * cooperative 8-lane butterfly produces, so both lookup forms give the same
 * value bit for bit. */
__device__ __forceinline__ float octet_sum(const float p[8]) {
	return fadd(fadd(fadd(p[0], p[1]), fadd(p[2], p[3])), fadd(fadd(p[4], p[5]), fadd(p[6], p[7])));
}

/* One channel's trilinear interpolation at a voxel octet (unscaled), with
 * the eight corner weights given: corner c at base + (c & 1) + sx * ((c >> 1)
 * & 1) + sxy * (c >> 2). */
__device__ __forceinline__ float4 octet_lerp_w(const float4* __restrict__ base, uint32_t sx, uint32_t sxy,
		const float w[8]) {
	float px[8], py[8], pz[8], pw[8];
#pragma unroll
	for (int c = 0; c < 8; ++c) {
		const float4 d = __ldg(base + (c & 1) + sx * ((c >> 1) & 1) + sxy * (c >> 2));
		px[c] = fmul(d.x, w[c]); py[c] = fmul(d.y, w[c]); pz[c] = fmul(d.z, w[c]); pw[c] = fmul(d.w, w[c]);
	}
	return make_float4(octet_sum(px), octet_sum(py), octet_sum(pz), octet_sum(pw));
}

/* LJPotForce, src/model/forcefield.h:30-83, swi = 1.  Explicitly rounded
 * FP32 (products and sums are never contracted by the compiler), so every
 * kernel that inlines it computes the same bits. */
__device__ __forceinline__ void lj_pot_force(float dr2, float dr2_inv, float dx, float dy,
		float dz, const float4 p, float ivor, bool shape86, float& fx, float& fy, float& fz,
		float& e) {
	const float rr23 = fmul(fmul(dr2_inv, dr2_inv), dr2_inv);
	const float rrd = shape86 ? dr2_inv : rr23;
	const float sd = shape86 ? 2.0f : 6.0f;
	const float rep = fmul(p.x, rrd);
	const float vlj = fmul(fsub(rep, p.y), rr23);
	float fb = ffma(6.0f, vlj, fmul(sd, fmul(rep, rr23)));
	if (dr2 < p.z) {
		e = ffma(fsub(ivor, 1.0f), p.w, vlj);
	} else {
		e = fmul(ivor, vlj);
		fb = fmul(ivor, fb);
	}
	fx = fmul(fb, dx); fy = fmul(fb, dy); fz = fmul(fb, dz);
}

/* ChargePotForce, src/model/forcefield.h:87-146, swi = 1 (explicitly rounded). */
__device__ __forceinline__ void charge_pot_force(float dr2_inv, float dx, float dy, float dz,
		float qq, bool constant_dielec, float& fx, float& fy, float& fz, float& e) {
	if (constant_dielec) {
		const float sr = __fsqrt_rn(dr2_inv);
		const float dd = fsub(sr, 0.02f);
		if (dd <= 0.0f) { e = 0.0f; fx = fy = fz = 0.0f; return; }
		e = fmul(qq, dd);
		const float et2 = fmul(qq, sr);
		fx = fmul(et2, dx); fy = fmul(et2, dy); fz = fmul(et2, dz);
	} else {
		const float dd = fsub(dr2_inv, 4.0e-4f);
		if (dd <= 0.0f) { e = 0.0f; fx = fy = fz = 0.0f; return; }
		e = fmul(qq, dd);
		const float et2 = fmul(2.0f, fmul(qq, dr2_inv));
		fx = fmul(et2, dx); fy = fmul(et2, dy); fz = fmul(et2, dz);
	}
}

/* Pose indices of one warp, identical on all lanes.  With a counter (zero
 * at launch) the warp takes the next unclaimed index whenever it finishes a
 * pose: per-pose cost varies by orders of magnitude (contact poses walk
 * thousands of neighbour pairs, distant ones none), and a fixed stride left
 * warps idle while others finished their share.  Without one, the fixed
 * stride warp, warp + nwarps, ... */
struct PoseFeed {
	unsigned long long* next;
	size_t k, stride;
	__device__ __forceinline__ PoseFeed(unsigned long long* counter)
		: next(counter),
		  k(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5),
		  stride(((size_t)gridDim.x * blockDim.x) >> 5) {}
	__device__ __forceinline__ size_t take(int lane) {
		if (next) {
			unsigned long long t = 0;
			if (lane == 0) t = atomicAdd(next, 1ull);
			return (size_t)__shfl_sync(GBA_FULL_MASK, t, 0);
		}
		const size_t r = k;
		k += stride;
		return r;
	}
};

/* Butterfly sum across the warp. */
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v = fadd(v, __shfl_xor_sync(GBA_FULL_MASK, v, o));
	return v;
}

/* euler2torquemat (src/model/matrixFunctions.h:81-127) contracted with the
 * torque matrix T (TorqueMat::rotateReduce, src/commons/TorqueMat.h:27-37). */
__device__ __forceinline__ void torque_reduce(const PoseRot& R, const float T[9], float out[3]) {
	const float cSSI_cPHI = fmul(R.cssi, R.cphi), cSSI_sPHI = fmul(R.cssi, R.sphi);
	const float sSSI_cPHI = fmul(R.sssi, R.cphi), sSSI_sPHI = fmul(R.sssi, R.sphi);
	const float cROT = R.crot, sROT = R.srot, cPHI = R.cphi, sPHI = R.sphi;
	const float cSSI = R.cssi, sSSI = R.sssi;
	float M[3][3][3];
	M[0][0][0] = fadd(fmul(-cROT, cSSI_sPHI), fmul(sROT, cPHI));
	M[0][0][1] = fsub(fmul(-sROT, cSSI_sPHI), fmul(cROT, cPHI));
	M[0][0][2] = -sSSI_sPHI;
	M[1][0][0] = fadd(fmul(cROT, cSSI_cPHI), fmul(sROT, sPHI));
	M[1][0][1] = fsub(fmul(sROT, cSSI_cPHI), fmul(cROT, sPHI));
	M[1][0][2] = sSSI_cPHI;
	M[2][0][0] = 0.f; M[2][0][1] = 0.f; M[2][0][2] = 0.f;
	M[0][1][0] = fmul(-cROT, sSSI_cPHI);
	M[0][1][1] = fmul(-sROT, sSSI_cPHI);
	M[0][1][2] = cSSI_cPHI;
	M[1][1][0] = fmul(-cROT, sSSI_sPHI);
	M[1][1][1] = fmul(-sROT, sSSI_sPHI);
	M[1][1][2] = cSSI_sPHI;
	M[2][1][0] = fmul(-cROT, cSSI);
	M[2][1][1] = fmul(-sROT, cSSI);
	M[2][1][2] = -sSSI;
	M[0][2][0] = fadd(fmul(-sROT, cSSI_cPHI), fmul(cROT, sPHI));
	M[0][2][1] = fadd(fmul(cROT, cSSI_cPHI), fmul(sROT, sPHI));
	M[0][2][2] = 0.f;
	M[1][2][0] = fsub(fmul(-sROT, cSSI_sPHI), fmul(cROT, cPHI));
	M[1][2][1] = fsub(fmul(cROT, cSSI_sPHI), fmul(sROT, cPHI));
	M[1][2][2] = 0.f;
	M[2][2][0] = fmul(sROT, sSSI);
	M[2][2][1] = fmul(-cROT, sSSI);
	M[2][2][2] = 0.f;
	float rx = 0.f, ry = 0.f, rz = 0.f;
#pragma unroll
	for (int k = 0; k < 3; ++k)
#pragma unroll
		for (int l = 0; l < 3; ++l) {
			rx = fadd(rx, fmul(M[k][0][l], T[3 * k + l]));
			ry = fadd(ry, fmul(M[k][1][l], T[3 * k + l]));
			rz = fadd(rz, fmul(M[k][2][l], T[3 * k + l]));
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
