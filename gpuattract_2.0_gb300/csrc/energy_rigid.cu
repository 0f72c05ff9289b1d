/*
 * energy_rigid.cu -- fused rigid-body docking energy + DOF gradient.
 *
 * One warp owns one pose at a time (grid-stride over poses).  For its pose the
 * warp builds the rotation once (lanes 0..2 run the sincos), then lanes
 * stride over the ligand beads and, per bead, fuse what the reference runs as
 * five separate stages with global intermediates:
 *   d_DOF2Pos        src/model/transform.cu:18-52        x' = R x + t
 *   d_potForce       src/model/interpolation.cu:18-140   inner/outer trilinear
 *   d_NLPotForce     src/model/neighborlist.cu:21-171    NL pair term
 *   blockReduce      src/model/reduction.cu:50-391       13 sums per pose
 *   h_finalReduce    src/model/reduction.h:160-205       ForceLim + TorqueMat
 * Nothing per bead is written to memory: the warp reduces force, energy and
 * the 3x3 torque matrix with shuffles and lanes 0..6 store the 28-byte
 * Result_6D.  The CPU semantics followed are CPUEnergyService6D's
 * (src/service/CPUEnergyService6D.tpp:100-195).
 */
#include "energy_dev.cuh"

namespace gba {

struct RigidRecPos {
	const float4* __restrict__ xyzq;
	__device__ __forceinline__ void operator()(uint32_t j, float& x, float& y, float& z, float& q) const {
		const float4 r = __ldg(&xyzq[j]);
		x = r.x; y = r.y; z = r.z; q = r.w;
	}
};

template <bool CENSUS>
__global__ void __launch_bounds__(256) rigid_energy_kernel(const RigidLaunch L) {
	const int lane = threadIdx.x & 31;
	const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
	const uint32_t nl_lig = L.lig.n;
	const RigidRecPos recpos{L.rec.xyzq};
	for (size_t p = warp; p < L.n; p += nwarps) {
		const float* dofp = reinterpret_cast<const float*>(L.dofs + p);
		const float dv = lane < 6 ? __ldg(dofp + lane) : 0.f;
		const float tx = __shfl_sync(GBA_FULL_MASK, dv, 0);
		const float ty = __shfl_sync(GBA_FULL_MASK, dv, 1);
		const float tz = __shfl_sync(GBA_FULL_MASK, dv, 2);
		const float a0 = __shfl_sync(GBA_FULL_MASK, dv, 3);
		const float a1 = __shfl_sync(GBA_FULL_MASK, dv, 4);
		const float a2 = __shfl_sync(GBA_FULL_MASK, dv, 5);
		const PoseRot R = pose_rotation(a0, a1, a2, lane);

		float sE = 0.f, sFx = 0.f, sFy = 0.f, sFz = 0.f;
		float T[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
		uint32_t c_grid = 0, c_charged = 0, c_nl = 0, c_ent = 0;
		for (uint32_t i = lane; i < nl_lig; i += 32) {
			const float4 b = __ldg(&L.lig.xyzq[i]);
			const uint32_t tm = __ldg(&L.lig.tm[i]);
			const uint32_t type = tm & 0xffffu, mapped = tm >> 16;
			float px, py, pz;
			rot_apply(R.m, b.x, b.y, b.z, px, py, pz);
			px = fadd(px, tx); py = fadd(py, ty); pz = fadd(pz, tz);
			float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
			bool charged;
			float4 pot;
			if (bead_grid_term(L.grid, px, py, pz, mapped, b.w, pot, charged)) {
				fx = pot.x; fy = pot.y; fz = pot.z; e = pot.w;
				if (CENSUS) { ++c_grid; c_charged += charged; }
			}
			if (type != 0) {
				uint32_t npairs = 0;
				const uint32_t ne = bead_nl_term(L.grid.nl, L.par, L.rec.tm, recpos, px, py, pz,
						type, b.w, fx, fy, fz, e, npairs, NoPairHook());
				if (CENSUS && !nl_out(L.grid.nl, px, py, pz)) {
					++c_nl;
					c_ent += ne;
				}
			}
			sE += e; sFx += fx; sFy += fy; sFz += fz;
			T[0] += b.x * fx; T[1] += b.y * fx; T[2] += b.z * fx;
			T[3] += b.x * fy; T[4] += b.y * fy; T[5] += b.z * fy;
			T[6] += b.x * fz; T[7] += b.y * fz; T[8] += b.z * fz;
		}
		sE = warp_sum(sE); sFx = warp_sum(sFx); sFy = warp_sum(sFy); sFz = warp_sum(sFz);
#pragma unroll
		for (int k = 0; k < 9; ++k) T[k] = warp_sum(T[k]);
		force_lim(sFx, sFy, sFz);
		float ang[3];
		torque_reduce(R, T, ang);
		const float vals[7] = {sE, sFx, sFy, sFz, ang[0], ang[1], ang[2]};
		float v = 0.f;
#pragma unroll
		for (int k = 0; k < 7; ++k) v = lane == k ? vals[k] : v;
		if (lane < 7) reinterpret_cast<float*>(L.out + p)[lane] = v;
		if (CENSUS) {
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) {
				c_grid += __shfl_xor_sync(GBA_FULL_MASK, c_grid, o);
				c_charged += __shfl_xor_sync(GBA_FULL_MASK, c_charged, o);
				c_nl += __shfl_xor_sync(GBA_FULL_MASK, c_nl, o);
				c_ent += __shfl_xor_sync(GBA_FULL_MASK, c_ent, o);
			}
			if (lane == 0) L.census[p] = PoseCensus{c_grid, c_charged, c_nl, c_ent};
		}
	}
}

cudaError_t launch_rigid_energy(const RigidLaunch& L, int blocks, int threads, cudaStream_t s) {
	if (L.census)
		rigid_energy_kernel<true><<<blocks, threads, 0, s>>>(L);
	else
		rigid_energy_kernel<false><<<blocks, threads, 0, s>>>(L);
	return cudaGetLastError();
}

int rigid_blocks_per_sm(int threads, bool census) {
	int nb = 0;
	if (census)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, rigid_energy_kernel<true>, threads, 0);
	else
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, rigid_energy_kernel<false>, threads, 0);
	return nb > 0 ? nb : 1;
}

}  // namespace gba
