/*
 * minimize.cu -- device-resident VA13 minimization of rigid poses.
 *
 * The reference minimizes on the host: one coroutine per pose runs
 * minfor/mc11a and every energy evaluation is a round trip through the
 * request server to the GPU service (src/apps/em/RequestHandler.tpp:102-216,
 * src/apps/em/VA13Solver.cpp:34-75).  Here the whole loop lives on the GPU:
 * a persistent work-queue kernel in which a warp claims poses from an atomic
 * cursor (any pair of a batch), lane 0 runs the VA13 state machine in FP64
 * and the warp evaluates each requested point with the fused rigid energy;
 * the minimizer state never leaves the SM.  A pose ends after the evaluation
 * budget (maxFunEval, src/apps/em/VA13Solver.h:66) or when minfor returns;
 * per pose the last evaluated DOF and Result and the evaluation count are
 * written -- what RequestHandler::getResultStates / getResultEnGrads report.
 *
 * Termination is bounded by construction: every path through the machine
 * either requests an evaluation (nfun <= maxFunEval) or finishes; a pose that
 * went past maxFunEval + 1 evaluations would raise GBA_ERR_DEVICE_CHECK.  A
 * wall-time budget (globaltimer, read by lane 0 of each warp from its start:
 * the caller's deadline, else kMinimizeHardCapNs) stops the warp and raises
 * GBA_ERR_TIMEOUT in a device status word.
 */
#include <algorithm>
#include <vector>

#include "gba_context.h"
#include "rigid_pose.cuh"
#include "va13.cuh"

namespace gba {

__device__ __forceinline__ unsigned long long global_ns() {
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

/* Lane 0 reads the clock and the whole warp takes its decision. */
__device__ __forceinline__ bool warp_over_budget(unsigned long long t_start, unsigned long long budget_ns,
		int lane) {
	int over = 0;
	if (lane == 0) over = global_ns() - t_start > budget_ns;
	return __shfl_sync(GBA_FULL_MASK, over, 0) != 0;
}

/* compiled for four resident 256-thread blocks per SM (64 registers, like
 * the scoring kernel's four-block instantiation); the staging areas, one per
 * warp, are dynamic shared memory sized to the block, so that smaller blocks
 * are not held back by shared memory they do not use (128 threads: eight
 * blocks per SM instead of four) */
extern __shared__ __align__(16) unsigned char min_stage_smem[];

__global__ void __launch_bounds__(256, 4) minimize_rigid_kernel(const MinLaunch L) {
	WarpStage* stage = reinterpret_cast<WarpStage*>(min_stage_smem);
	const int lane = threadIdx.x & 31;
	unsigned long long t_start = 0;
	if (lane == 0) t_start = global_ns();
	t_start = __shfl_sync(GBA_FULL_MASK, t_start, 0);
	if (lane == 0 && L.t0) atomicMin(L.t0, t_start);
	/* the caller's wall-time budget, else a hard cap on any warp's run time */
	const unsigned long long budget = L.budget_ns ? L.budget_ns : kMinimizeHardCapNs;
	for (;;) {
		unsigned long long base = 0;
		if (lane == 0) base = atomicAdd(L.counter, (unsigned long long)L.chunk);
		base = __shfl_sync(GBA_FULL_MASK, base, 0);
		if (base >= L.n) break;
		if (warp_over_budget(t_start, budget, lane)) {
			if (lane == 0) atomicExch(L.status, GBA_ERR_TIMEOUT);
			break;
		}
		const size_t end = min((size_t)(base + L.chunk), L.n);
		for (size_t slot = base; slot < end; ++slot) {
			const size_t p = L.order ? (size_t)__ldg(&L.order[slot]) : slot;
			const RigidModel& M = L.models[L.pair_of ? __ldg(&L.pair_of[p]) : 0u];
			VA13<6> va;
			float cur[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
			float res[7];
			int nev = 0;
			if (lane == 0) {
				const gba_dof6d s = L.start[p];
				/* TypesConverter<DOF_6D, Vector>: (ang xyz, pos xyz), src/apps/em/meta.h:66-97 */
				const double x0[6] = {s.ang[0], s.ang[1], s.ang[2], s.pos[0], s.pos[1], s.pos[2]};
				va.start(x0, 6, L.max_evals);
			}
			for (;;) {
				if (lane == 0) {
					const double* pt = va.point();
					cur[0] = (float)pt[3]; cur[1] = (float)pt[4]; cur[2] = (float)pt[5];
					cur[3] = (float)pt[0]; cur[4] = (float)pt[1]; cur[5] = (float)pt[2];
				}
#pragma unroll
				for (int k = 0; k < 6; ++k) cur[k] = __shfl_sync(GBA_FULL_MASK, cur[k], 0);
				eval_pose_rigid<false>(M, cur[0], cur[1], cur[2], cur[3], cur[4], cur[5], lane, stage[threadIdx.x >> 5], res,
						nullptr);
				++nev;
				int done = 0;
				if (lane == 0) {
					/* objective E, gradient -(ang, pos), src/apps/em/meta.h:114-121 */
					const double g[6] = {-(double)res[4], -(double)res[5], -(double)res[6],
							-(double)res[1], -(double)res[2], -(double)res[3]};
					va.provide((double)res[0], g);
					done = va.done();
				}
				if (__shfl_sync(GBA_FULL_MASK, done, 0)) break;
				/* VA13 ends within max_evals + 1 evaluations; anything past that is
				 * a broken machine, reported instead of looping */
				if (nev > L.max_evals + 1) {
					if (lane == 0) atomicExch(L.status, GBA_ERR_DEVICE_CHECK);
					break;
				}
				if ((nev & 15) == 0 && warp_over_budget(t_start, budget, lane)) {
					if (lane == 0) atomicExch(L.status, GBA_ERR_TIMEOUT);
					break;
				}
			}
			store_result7(reinterpret_cast<float*>(L.out_result + p), res, lane);
			if (lane < 6) reinterpret_cast<float*>(L.out_state + p)[lane] = cur[lane];
			if (lane == 0 && L.out_nevals) L.out_nevals[p] = nev;
			if (lane == 0 && L.done_ns) L.done_ns[p] = global_ns();
		}
	}
}

static size_t min_stage_bytes(int threads) { return (size_t)((threads + 31) / 32) * sizeof(WarpStage); }

cudaError_t launch_minimize_rigid(const MinLaunch& L, int blocks, int threads, cudaStream_t s) {
	minimize_rigid_kernel<<<blocks, threads, min_stage_bytes(threads), s>>>(L);
	return cudaGetLastError();
}

int minimize_blocks_per_sm(int threads) {
	int nb = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, minimize_rigid_kernel, threads, min_stage_bytes(threads));
	return nb > 0 ? nb : 1;
}

}  // namespace gba
