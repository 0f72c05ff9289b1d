/*
 * minimize.cu -- device-resident VA13 minimization of rigid poses.
 *
 * The reference minimizes on the host: one coroutine per pose runs
 * minfor/mc11a and every energy evaluation is a round trip through the
 * request server to the GPU service (src/apps/em/RequestHandler.tpp:102-216,
 * src/apps/em/VA13Solver.cpp:34-75).  Here the whole loop lives on the GPU:
 * a persistent work-queue kernel in which a warp claims poses from an atomic
 * cursor (any pair of a batch), the warp steps the VA13 state machine in
 * FP64 (its warp form: element-wise work on lanes, independent divisions
 * together -- va13.cuh) and evaluates each requested point with the fused
 * rigid energy;
 * the minimizer state never leaves the SM.  A pose ends after the evaluation
 * budget (maxFunEval, src/apps/em/VA13Solver.h:66) or when minfor returns;
 * per pose the last evaluated DOF and Result and the evaluation count are
 * written -- what RequestHandler::getResultStates / getResultEnGrads report.
 *
 * Both kernels sum each pose round-wise (rigid_pose.cuh), as the plain
 * per-step form's scoring launches do, so all three give the same bits.
 * With GBA_KOPT_REFERENCE_ORDER both sum in the reference CPU path's order
 * instead (eval_pose_rigid_ref, eval_pose_rigid_team_ref: the same bits).
 *
 * Small jobs (fewer poses than the GPU has warp slots) run the team kernel
 * instead: a team of G warps evaluates one pose, warp t taking the ligand's
 * 64-bead rounds t, t + G, ... and the team's first warp adding the round
 * totals in order (eval_pose_rigid_team) -- the same bits as one warp doing
 * every round -- so a 200-bead ligand (four rounds) evaluates in about the
 * time of one round.  When every pose of the job gets a block of its own
 * (all resident), warp 0 steps the pose's VA13 after each evaluation (the
 * solo kernel); otherwise each block adds a control warp and holds two
 * poses: while the team evaluates one, the control warp runs the other's
 * VA13 step.
 *
 * Termination is bounded by construction: every path through the machine
 * either requests an evaluation (nfun <= maxFunEval) or finishes; a pose that
 * went past maxFunEval + 1 evaluations would raise GBA_ERR_DEVICE_CHECK.  A
 * wall-time budget (globaltimer, read by lane 0 of each warp from its start:
 * the caller's deadline, else kMinimizeHardCapNs) stops the warp and raises
 * GBA_ERR_TIMEOUT in a device status word.
 */
#include <algorithm>
#include <atomic>
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

/* The Result_6D entry behind VA13 gradient element j (1-based, order (ang
 * xyz, pos xyz): src/apps/em/meta.h:114-121); 0 outside 1..6.  Selects with
 * constant indices keep res in registers. */
__device__ __forceinline__ float rigid_grad_entry(const float res[7], int j) {
	float v = 0.f;
#pragma unroll
	for (int k = 1; k <= 6; ++k) v = j == k ? res[k <= 3 ? k + 3 : k - 3] : v;
	return v;
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

/* REF: GBA_KOPT_REFERENCE_ORDER (eval_pose_rigid_ref), compiled for two
 * resident blocks per SM */
template <bool REF>
__global__ void __launch_bounds__(256, REF ? 2 : 4) minimize_rigid_kernel(const MinLaunch L) {
	WarpStage* stage = reinterpret_cast<WarpStage*>(min_stage_smem);
	/* per warp, after the staging areas: the VA13 state of its pose (shared
	 * memory keeps it next to the SM between steps; see TeamShared) */
	VA13<6>* vas = reinterpret_cast<VA13<6>*>(stage + (blockDim.x >> 5));
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
			VA13<6>& va = vas[threadIdx.x >> 5];
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
				if (REF)
					eval_pose_rigid_ref(M, cur[0], cur[1], cur[2], cur[3], cur[4], cur[5], lane, stage[threadIdx.x >> 5],
							res);
				else
					eval_pose_rigid<false, true>(M, cur[0], cur[1], cur[2], cur[3], cur[4], cur[5], lane,
							stage[threadIdx.x >> 5], res, nullptr);
				++nev;
				/* objective E, gradient -(ang, pos), src/apps/em/meta.h:114-121;
				 * the whole warp steps the machine, lane j holding element j */
				const double gl = -(double)rigid_grad_entry(res, lane);
				va.provide_w((double)res[0], [&](int) { return gl; }, VaWarp{lane});
				/* lane 0's reading for all: no lane may see a state that lane 0,
				 * gone on to the next pose, has already restarted */
				if (__shfl_sync(GBA_FULL_MASK, (int)va.done(), 0)) break;
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

/* One pose slot of a pipelined team block. */
struct PipeSlot {
	VA13<6> va;                /* the pose's minimizer state (kept in shared memory: in
	                              thread-local memory the evaluation's traffic evicted it
	                              from L1 between steps) */
	float cur[6];              /* the point to evaluate / last evaluated (DOF_6D order) */
	float res[7];              /* its Result_6D */
	int active;                /* a pose occupies the slot */
	int evaluated;             /* res holds the evaluation of cur, not yet given to VA13 */
	int nev;                   /* evaluations so far */
	int pad;
	unsigned long long p;      /* the pose */
};

struct PipeShared {
	PipeSlot slot[2];
	int more[2];               /* loop continues at half-step h: more[h & 1] */
};

/* Thread 0: the next pose into slot S (VA13 started, first point ready) or
 * the slot closed when the queue is empty or the budget is spent. */
__device__ __forceinline__ void pipe_claim(const MinLaunch& L, PipeSlot& S, unsigned long long t_start,
		unsigned long long budget) {
	unsigned long long slot = atomicAdd(L.counter, 1ull);
	if (slot < L.n && global_ns() - t_start > budget) {
		atomicExch(L.status, GBA_ERR_TIMEOUT);
		slot = ~0ull;
	}
	if (slot >= L.n) {
		S.active = 0;
		return;
	}
	const size_t p = L.order ? (size_t)__ldg(&L.order[slot]) : (size_t)slot;
	const gba_dof6d s0 = L.start[p];
	/* TypesConverter<DOF_6D, Vector>: (ang xyz, pos xyz), src/apps/em/meta.h:66-97 */
	const double x0[6] = {s0.ang[0], s0.ang[1], s0.ang[2], s0.pos[0], s0.pos[1], s0.pos[2]};
	S.va.start(x0, 6, L.max_evals);
	const double* pt = S.va.point();
	S.cur[0] = (float)pt[3]; S.cur[1] = (float)pt[4]; S.cur[2] = (float)pt[5];
	S.cur[3] = (float)pt[0]; S.cur[4] = (float)pt[1]; S.cur[5] = (float)pt[2];
	S.p = p;
	S.nev = 0;
	S.evaluated = 0;
	S.active = 1;
}

/* The control warp, every lane: hands the evaluation of slot S to its VA13
 * (the warp form); then lane 0 alone (t_start is its own) ends the pose --
 * outputs written, slot refilled -- or readies its next point. */
__device__ __forceinline__ void pipe_consume(const MinLaunch& L, PipeSlot& S, unsigned long long t_start,
		unsigned long long budget, int lane) {
	/* objective E, gradient -(ang, pos), src/apps/em/meta.h:114-121 */
	const double gl = -(double)rigid_grad_entry(S.res, lane);
	S.va.provide_w((double)S.res[0], [&](int) { return gl; }, VaWarp{lane});
	if (lane != 0) return;
	S.evaluated = 0;
	++S.nev;
	bool stop = S.va.done();
	/* VA13 ends within max_evals + 1 evaluations; anything past that is a
	 * broken machine, reported instead of looping */
	if (!stop && S.nev > L.max_evals + 1) {
		atomicExch(L.status, GBA_ERR_DEVICE_CHECK);
		stop = true;
	}
	if (!stop && (S.nev & 15) == 0 && global_ns() - t_start > budget) {
		atomicExch(L.status, GBA_ERR_TIMEOUT);
		stop = true;
	}
	if (!stop) {
		const double* pt = S.va.point();
		S.cur[0] = (float)pt[3]; S.cur[1] = (float)pt[4]; S.cur[2] = (float)pt[5];
		S.cur[3] = (float)pt[0]; S.cur[4] = (float)pt[1]; S.cur[5] = (float)pt[2];
		return;
	}
	float* r = reinterpret_cast<float*>(L.out_result + S.p);
	float* x = reinterpret_cast<float*>(L.out_state + S.p);
	for (int k = 0; k < 7; ++k) r[k] = S.res[k];
	for (int k = 0; k < 6; ++k) x[k] = S.cur[k];
	if (L.out_nevals) L.out_nevals[S.p] = S.nev;
	if (L.done_ns) L.done_ns[S.p] = global_ns();
	pipe_claim(L, S, t_start, budget);
}

/* The pipelined team kernel: warp 0 is the control warp (it steps VA13),
 * warps 1..G evaluate.  A block holds two poses; in half-step h the
 * evaluators score slot h & 1 while the control warp gives slot h & 1 ^ 1's
 * fresh evaluation to its VA13 -- the FP64 minimizer step runs beside the
 * evaluation instead of after it.  Each pose still alternates evaluation and
 * VA13 step exactly as in the other forms. */
template <bool REF>
__global__ void __launch_bounds__(256, REF ? 2 : 4) minimize_rigid_team_kernel(const MinLaunch L) {
	const int G = (blockDim.x >> 5) - 1;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpStage* stage = reinterpret_cast<WarpStage*>(min_stage_smem);
	float* slots = reinterpret_cast<float*>(stage + G);
	PipeShared& sh = *reinterpret_cast<PipeShared*>(slots + 16 * G);
	unsigned long long t_start = 0;
	const unsigned long long budget = L.budget_ns ? L.budget_ns : kMinimizeHardCapNs;
	if (threadIdx.x == 0) {
		t_start = global_ns();
		if (L.t0) atomicMin(L.t0, t_start);
		pipe_claim(L, sh.slot[0], t_start, budget);
		pipe_claim(L, sh.slot[1], t_start, budget);
		sh.more[0] = sh.slot[0].active | sh.slot[1].active;
	}
	for (int h = 0;; ++h) {
		__syncthreads();
		if (!sh.more[h & 1]) break;
		const int e = h & 1;
		if (warp == 0) {
			PipeSlot& S = sh.slot[e ^ 1];
			/* lane 0's reading for the warp (lane 0 changes the slot inside) */
			if (__shfl_sync(GBA_FULL_MASK, (int)(S.active && S.evaluated), 0)) pipe_consume(L, S, t_start, budget, lane);
			if (lane == 0) sh.more[(h + 1) & 1] = sh.slot[0].active | sh.slot[1].active;
		} else {
			PipeSlot& S = sh.slot[e];
			if (S.active && !S.evaluated) {
				const RigidModel& M = L.models[L.pair_of ? __ldg(&L.pair_of[S.p]) : 0u];
				float res[7];
				if (REF)
					eval_pose_rigid_team_ref(M, S.cur[0], S.cur[1], S.cur[2], S.cur[3], S.cur[4], S.cur[5], lane,
							warp - 1, G, stage, res, 1);
				else
					eval_pose_rigid_team(M, S.cur[0], S.cur[1], S.cur[2], S.cur[3], S.cur[4], S.cur[5], lane,
							warp - 1, G, stage, slots, res, 1);
				if (warp == 1) {
					if (lane < 7) S.res[lane] = res[lane];
					__syncwarp();
					if (lane == 0) S.evaluated = 1;
				}
			}
		}
	}
}

/* The solo team kernel: a block of G warps holds one pose, evaluates it
 * (eval_pose_rigid_team: the same bits as the other forms) and then steps
 * its VA13 on warp 0 while the other warps wait.  A pose's step costs one
 * evaluation plus one VA13 step; in the pipelined kernel above it costs two
 * evaluations, since the pose waits for the other slot's.  For jobs in
 * which every pose gets its own resident block. */
template <bool REF>
__global__ void __launch_bounds__(256, REF ? 2 : 4) minimize_rigid_solo_kernel(const MinLaunch L) {
	const int G = blockDim.x >> 5;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpStage* stage = reinterpret_cast<WarpStage*>(min_stage_smem);
	float* slots = reinterpret_cast<float*>(stage + G);
	PipeSlot& S = *reinterpret_cast<PipeSlot*>(slots + 16 * G);
	unsigned long long t_start = 0;
	const unsigned long long budget = L.budget_ns ? L.budget_ns : kMinimizeHardCapNs;
	if (threadIdx.x == 0) {
		t_start = global_ns();
		if (L.t0) atomicMin(L.t0, t_start);
		pipe_claim(L, S, t_start, budget);
	}
	for (;;) {
		__syncthreads();   /* the slot as thread 0 left it */
		if (!S.active) break;
		const RigidModel& M = L.models[L.pair_of ? __ldg(&L.pair_of[S.p]) : 0u];
		float res[7];
		/* every warp reads the point before the evaluation's first team
		 * barrier; warp 0 changes the slot only after its last one */
		if (REF)
			eval_pose_rigid_team_ref(M, S.cur[0], S.cur[1], S.cur[2], S.cur[3], S.cur[4], S.cur[5], lane, warp, G,
					stage, res, 1);
		else
			eval_pose_rigid_team(M, S.cur[0], S.cur[1], S.cur[2], S.cur[3], S.cur[4], S.cur[5], lane, warp, G,
					stage, slots, res, 1);
		if (warp == 0) {
			if (lane < 7) S.res[lane] = res[lane];
			__syncwarp();
			pipe_consume(L, S, t_start, budget, lane);
		}
	}
}

static size_t min_stage_bytes(int threads) {
	return (size_t)((threads + 31) / 32) * (sizeof(WarpStage) + sizeof(VA13<6>));
}

/* shared memory of the team kernel with `team` evaluation warps */
static size_t team_smem_bytes(int team) {
	return (size_t)team * (sizeof(WarpStage) + sizeof(float) * 16) + sizeof(PipeShared);
}

/* shared memory of the solo kernel with `team` warps */
static size_t solo_smem_bytes(int team) {
	return (size_t)team * (sizeof(WarpStage) + sizeof(float) * 16) + sizeof(PipeSlot);
}

cudaError_t launch_minimize_rigid(const MinLaunch& L, int blocks, int threads, cudaStream_t s) {
	if (L.ref_order)
		minimize_rigid_kernel<true><<<blocks, threads, min_stage_bytes(threads), s>>>(L);
	else
		minimize_rigid_kernel<false><<<blocks, threads, min_stage_bytes(threads), s>>>(L);
	return cudaGetLastError();
}

cudaError_t launch_minimize_rigid_team(const MinLaunch& L, int blocks, int team, cudaStream_t s) {
	if (team < 1 || team > kMaxTeam) return cudaErrorInvalidValue;
	if (L.ref_order)
		minimize_rigid_team_kernel<true><<<blocks, 32 * (team + 1), team_smem_bytes(team), s>>>(L);
	else
		minimize_rigid_team_kernel<false><<<blocks, 32 * (team + 1), team_smem_bytes(team), s>>>(L);
	return cudaGetLastError();
}

cudaError_t launch_minimize_rigid_solo(const MinLaunch& L, int blocks, int team, cudaStream_t s) {
	if (team < 1 || team > kMaxTeam) return cudaErrorInvalidValue;
	if (L.ref_order)
		minimize_rigid_solo_kernel<true><<<blocks, 32 * team, solo_smem_bytes(team), s>>>(L);
	else
		minimize_rigid_solo_kernel<false><<<blocks, 32 * team, solo_smem_bytes(team), s>>>(L);
	return cudaGetLastError();
}

/* Dynamic shared memory above the 48 KB default (eight one-warp staging
 * areas with their VA13 states need ~53 KB): allowed once per device, before
 * any occupancy query or capture. */
static void allow_minimize_smem() {
	static std::atomic<int> done[64];
	int dev = 0;
	cudaGetDevice(&dev);
	if (dev >= 0 && dev < 64 && done[dev].load()) return;
	cudaFuncSetAttribute(minimize_rigid_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
			(int)min_stage_bytes(256));
	cudaFuncSetAttribute(minimize_rigid_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
			(int)min_stage_bytes(256));
	cudaFuncSetAttribute(minimize_rigid_team_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
			(int)team_smem_bytes(kMaxTeam));
	cudaFuncSetAttribute(minimize_rigid_team_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
			(int)team_smem_bytes(kMaxTeam));
	cudaFuncSetAttribute(minimize_rigid_solo_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
			(int)solo_smem_bytes(kMaxTeam));
	cudaFuncSetAttribute(minimize_rigid_solo_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
			(int)solo_smem_bytes(kMaxTeam));
	cudaGetLastError();
	if (dev >= 0 && dev < 64) done[dev].store(1);
}

int minimize_blocks_per_sm(int threads, bool ref_order) {
	allow_minimize_smem();
	int nb = 0;
	if (ref_order)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, minimize_rigid_kernel<true>, threads,
				min_stage_bytes(threads));
	else
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, minimize_rigid_kernel<false>, threads,
				min_stage_bytes(threads));
	return nb > 0 ? nb : 1;
}

int minimize_team_blocks_per_sm(int team, bool ref_order) {
	allow_minimize_smem();
	int nb = 0;
	if (ref_order)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, minimize_rigid_team_kernel<true>, 32 * (team + 1),
				team_smem_bytes(team));
	else
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, minimize_rigid_team_kernel<false>, 32 * (team + 1),
				team_smem_bytes(team));
	return nb > 0 ? nb : 1;
}

int minimize_solo_blocks_per_sm(int team, bool ref_order) {
	allow_minimize_smem();
	int nb = 0;
	if (ref_order)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, minimize_rigid_solo_kernel<true>, 32 * team,
				solo_smem_bytes(team));
	else
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, minimize_rigid_solo_kernel<false>, 32 * team,
				solo_smem_bytes(team));
	return nb > 0 ? nb : 1;
}

}  // namespace gba
