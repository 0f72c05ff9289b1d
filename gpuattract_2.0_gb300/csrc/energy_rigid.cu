/*
 * energy_rigid.cu -- fused rigid-body docking energy + DOF gradient, one
 * launch per batch of poses.
 *
 * Replaces the reference GPU pipeline of five launches with global
 * intermediates per 100-pose item (src/service/GPUEnergyService6D.tpp:163-430):
 *   d_DOF2Pos        src/model/transform.cu:18-52        x' = R x + t
 *   d_potForce       src/model/interpolation.cu:18-140   inner/outer trilinear
 *   d_NLPotForce     src/model/neighborlist.cu:21-171    NL pair term
 *   blockReduce      src/model/reduction.cu:50-391       13 sums per pose
 *   h_finalReduce    src/model/reduction.h:160-205       ForceLim + TorqueMat
 * by one kernel in which a warp owns a pose (grid-stride over poses) and
 * nothing per bead leaves the SM; lanes 0..6 store the 28-byte Result_6D.
 */
#include <atomic>

#include "rigid_pose.cuh"

namespace gba {

/* BOUND4: registers capped for four resident 256-thread blocks per SM
 * (GBA_KOPT_FOUR_BLOCKS).  ROUNDWISE: the minimizers' round-wise summation
 * order (the plain per-step minimization form's launches). */
template <bool CENSUS, bool BOUND4, bool ROUNDWISE = false>
__global__ void __launch_bounds__(256, BOUND4 ? 4 : 1) rigid_energy_kernel(const RigidLaunch L) {
	__shared__ WarpStage stage[8];   /* one per warp of a <=256-thread block */
	const int lane = threadIdx.x & 31;
	PoseFeed feed(L.next);
	for (size_t k = feed.take(lane); k < L.n; k = feed.take(lane)) {
		const size_t p = L.order ? (size_t)__ldg(&L.order[k]) : k;
		const float* dofp = reinterpret_cast<const float*>(L.dofs + p);
		const float dv = lane < 6 ? __ldg(dofp + lane) : 0.f;
		const float tx = __shfl_sync(GBA_FULL_MASK, dv, 0);
		const float ty = __shfl_sync(GBA_FULL_MASK, dv, 1);
		const float tz = __shfl_sync(GBA_FULL_MASK, dv, 2);
		const float a0 = __shfl_sync(GBA_FULL_MASK, dv, 3);
		const float a1 = __shfl_sync(GBA_FULL_MASK, dv, 4);
		const float a2 = __shfl_sync(GBA_FULL_MASK, dv, 5);
		float res[7];
		eval_pose_rigid<CENSUS, ROUNDWISE>(L.m, tx, ty, tz, a0, a1, a2, lane, stage[threadIdx.x >> 5], res,
				CENSUS ? L.census + p : nullptr);
		store_result7(reinterpret_cast<float*>(L.out + p), res, lane);
	}
}

/* GBA_KOPT_REFERENCE_ORDER: each pose summed in the reference CPU path's
 * order (eval_pose_rigid_ref).  Compiled for four resident 256-thread blocks
 * per SM (64 registers): it spills 152 bytes there, but the latency of its
 * double-precision chains wants the warps -- config 1 measured 15.4 ms per
 * 100,000 poses at four blocks, 16.7 ms at three (80 registers) and 20.7 ms
 * at two (108, no spills). */
__global__ void __launch_bounds__(256, 4) rigid_energy_ref_kernel(const RigidLaunch L) {
	__shared__ WarpStage stage[8];
	const int lane = threadIdx.x & 31;
	PoseFeed feed(L.next);
	for (size_t k = feed.take(lane); k < L.n; k = feed.take(lane)) {
		const size_t p = L.order ? (size_t)__ldg(&L.order[k]) : k;
		const float* dofp = reinterpret_cast<const float*>(L.dofs + p);
		const float dv = lane < 6 ? __ldg(dofp + lane) : 0.f;
		float c[6];
#pragma unroll
		for (int j = 0; j < 6; ++j) c[j] = __shfl_sync(GBA_FULL_MASK, dv, j);
		float res[7];
		eval_pose_rigid_ref(L.m, c[0], c[1], c[2], c[3], c[4], c[5], lane, stage[threadIdx.x >> 5], res);
		store_result7(reinterpret_cast<float*>(L.out + p), res, lane);
	}
}

/* Poses of many pairs in one launch: pose p belongs to pair pair_of[p]. */
template <bool REF>
__global__ void __launch_bounds__(256) batch_energy_kernel(const BatchEnergyLaunch L) {
	__shared__ WarpStage stage[8];   /* one per warp of a <=256-thread block */
	const int lane = threadIdx.x & 31;
	PoseFeed feed(L.next);
	for (size_t p = feed.take(lane); p < L.n; p = feed.take(lane)) {
		const RigidModel& M = L.models[__ldg(&L.pair_of[p])];
		const float* dofp = reinterpret_cast<const float*>(L.dofs + p);
		const float dv = lane < 6 ? __ldg(dofp + lane) : 0.f;
		float c[6];
#pragma unroll
		for (int k = 0; k < 6; ++k) c[k] = __shfl_sync(GBA_FULL_MASK, dv, k);
		float res[7];
		if (REF)
			eval_pose_rigid_ref(M, c[0], c[1], c[2], c[3], c[4], c[5], lane, stage[threadIdx.x >> 5], res);
		else
			eval_pose_rigid<false>(M, c[0], c[1], c[2], c[3], c[4], c[5], lane, stage[threadIdx.x >> 5], res,
					nullptr);
		store_result7(reinterpret_cast<float*>(L.out + p), res, lane);
	}
}

cudaError_t launch_batch_energy(const BatchEnergyLaunch& L, int blocks, int threads, cudaStream_t s) {
	if (L.ref_order)
		batch_energy_kernel<true><<<blocks, threads, 0, s>>>(L);
	else
		batch_energy_kernel<false><<<blocks, threads, 0, s>>>(L);
	return cudaGetLastError();
}

cudaError_t launch_rigid_energy(const RigidLaunch& L, int blocks, int threads, cudaStream_t s) {
	if (L.census)
		rigid_energy_kernel<true, false><<<blocks, threads, 0, s>>>(L);
	else if (L.ref_order)
		rigid_energy_ref_kernel<<<blocks, threads, 0, s>>>(L);
	else if (L.roundwise && L.bound4)
		rigid_energy_kernel<false, true, true><<<blocks, threads, 0, s>>>(L);
	else if (L.roundwise)
		rigid_energy_kernel<false, false, true><<<blocks, threads, 0, s>>>(L);
	else if (L.bound4)
		rigid_energy_kernel<false, true><<<blocks, threads, 0, s>>>(L);
	else
		rigid_energy_kernel<false, false><<<blocks, threads, 0, s>>>(L);
	return cudaGetLastError();
}

/* resident blocks per SM, queried once per device, instantiation and block
 * size (the query costs host time on every launch otherwise) */
int rigid_blocks_per_sm(int threads, bool census, bool bound4, bool roundwise, bool ref_order) {
	static std::atomic<int> cache[64][6][33];
	int dev = 0;
	cudaGetDevice(&dev);
	const int v = census ? 0 : ref_order ? 5 : (roundwise ? (bound4 ? 3 : 4) : (bound4 ? 1 : 2)), t = threads / 32;
	const bool cacheable = dev >= 0 && dev < 64 && threads % 32 == 0 && t >= 1 && t <= 32;
	if (cacheable) {
		const int c = cache[dev][v][t].load(std::memory_order_relaxed);
		if (c > 0) return c;
	}
	int nb = 0;
	if (census)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, rigid_energy_kernel<true, false>, threads, 0);
	else if (ref_order)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, rigid_energy_ref_kernel, threads, 0);
	else if (roundwise && bound4)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, rigid_energy_kernel<false, true, true>, threads, 0);
	else if (roundwise)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, rigid_energy_kernel<false, false, true>, threads, 0);
	else if (bound4)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, rigid_energy_kernel<false, true>, threads, 0);
	else
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, rigid_energy_kernel<false, false>, threads, 0);
	nb = nb > 0 ? nb : 1;
	if (cacheable) cache[dev][v][t].store(nb, std::memory_order_relaxed);
	return nb;
}

}  // namespace gba
