/*
 * minimize_api.cu -- host side of minimization and multi-pair batches.
 *
 *   gba_minimize_6d        batched form: one persistent work-queue launch,
 *                          VA13 on the device, the whole pipeline (cursor
 *                          reset, copies, kernel) replayed as a cached CUDA
 *                          graph; small jobs give each pose a team of warps
 *   gba_minimize_6d_plain  the reference's execution model on the same GPU:
 *                          VA13 per pose on the host, one energy launch plus
 *                          host<->device copies per evaluation round
 *                          (src/apps/em/RequestHandler.tpp:130-216)
 *   gba_batch_*            many receptor-ligand pairs of uneven sizes in one launch
 */
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "gba_context.h"
#include "va13.cuh"

namespace gba {

namespace {

/* device copies of RigidModel arrays, keyed by the id tuple list */
const RigidModel* models_on_device(Context* ctx, const std::vector<RigidModel>& m,
		const std::vector<gba_id>& key, cudaStream_t s) {
	auto it = ctx->model_cache.find(key);
	if (it == ctx->model_cache.end()) {
		auto buf = std::make_unique<DevBuffer>();
		buf->upload(m.data(), m.size() * sizeof(RigidModel));
		it = ctx->model_cache.emplace(key, std::move(buf)).first;
	}
	(void)s;
	return (const RigidModel*)it->second->ptr;
}

struct Placement {
	bool device;
	size_t off;       /* offset in the staging arrays when not device */
};

}  // namespace

int Context::minimize_team(const TuneParams& tp, size_t n, uint32_t lig_rounds) const {
	int team = team_override;
	if (team == 0 && tp.team > 0 && n <= tp.team_poses) team = tp.team;
	if (team == 0 && (kernel_opts & GBA_KOPT_REFERENCE_ORDER)) {
		/* the reference order's double-precision steps keep the FP64 pipe
		 * busy: teams measured no faster (config 0: 59-73 k poses/s for
		 * teams of 2-4 against 67 k for one warp per pose) */
		team = 1;
	}
	if (team == 0) {
		/* fewer poses than the one-warp kernel has resident warps: give each
		 * pose as many warps as fill them, up to its ligand's rounds */
		const size_t slots = (size_t)num_sms * minimize_blocks_per_sm(tp.threads) * (tp.threads / 32);
		team = n > 0 && n * 2 <= slots ? (int)std::min<size_t>(kMaxTeam, slots / n) : 1;
	}
	team = std::min<int>(team, (int)std::max<uint32_t>(1, lig_rounds));
	return std::max(1, std::min(team, kMaxTeam));
}

namespace {

/* Launch shape of one persistent minimizer launch over n poses. */
struct MinShape {
	int team, threads, chunk;
	size_t blocks;
	bool solo;        /* team > 1: one pose per block (all resident), else two */
};

MinShape min_shape(const Context& ctx, const TuneParams& tp, size_t n, int team) {
	MinShape m{team, tp.threads, 1, 1, false};
	if (team > 1) {
		const bool ref = (ctx.kernel_opts & GBA_KOPT_REFERENCE_ORDER) != 0;
		const size_t solo_cap = (size_t)ctx.num_sms * minimize_solo_blocks_per_sm(team, ref);
		if (n <= solo_cap) {
			/* every pose its own block of team warps, all resident */
			m.solo = true;
			m.threads = 32 * team;
			m.blocks = std::max<size_t>(1, n);
		} else {
			/* team evaluation warps plus a control warp; two poses per block */
			m.threads = 32 * (team + 1);
			m.blocks = std::min<size_t>((n + 1) / 2, (size_t)ctx.num_sms * minimize_team_blocks_per_sm(team, ref));
		}
	} else {
		const int bps = std::min(tp.blocks_per_sm,
				minimize_blocks_per_sm(m.threads, (ctx.kernel_opts & GBA_KOPT_REFERENCE_ORDER) != 0));
		const size_t warps = (size_t)ctx.num_sms * bps * (m.threads / 32);
		m.blocks = (size_t)ctx.num_sms * bps;
		if (warps > n) m.blocks = std::max<size_t>(1, (n * 32 + m.threads - 1) / m.threads);
		m.chunk = tp.chunk;
	}
	return m;
}

cudaError_t launch_shape(const MinLaunch& L, const MinShape& m, cudaStream_t s) {
	if (m.team > 1)
		return m.solo ? launch_minimize_rigid_solo(L, (int)m.blocks, m.team, s)
		              : launch_minimize_rigid_team(L, (int)m.blocks, m.team, s);
	return launch_minimize_rigid(L, (int)m.blocks, m.threads, s);
}

}  // namespace

/* Runs the persistent minimizer over `total` poses whose inputs/outputs live
 * in device memory; captured in a CUDA graph cached by launch signature. */
void Context::run_minimize(MinLaunch& L, cudaStream_t s, int32_t* status_out, uint32_t lig_rounds,
		const TuneParams& tp) {
	L.ref_order = (kernel_opts & GBA_KOPT_REFERENCE_ORDER) ? 1 : 0;
	const MinShape m = min_shape(*this, tp, L.n, minimize_team(tp, L.n, lig_rounds));
	L.chunk = m.chunk;
	if (!aux.ptr) {
		aux.alloc(64);
		note_allocation();
		check_cuda(cudaMallocHost((void**)&pinned_status, sizeof(int32_t)), "cudaMallocHost");
	}
	/* aux: [0,8) cursor, [8,12) status, [16,24) modes cursor, [32,40) earliest warp start */
	L.counter = (unsigned long long*)aux.ptr;
	L.status = (int*)((char*)aux.ptr + 8);
	L.t0 = (unsigned long long*)((char*)aux.ptr + 32);

	GraphKey key{};
	key.kind = 1;
	key.a = (uintptr_t)L.models;
	key.b = (uintptr_t)L.pair_of ^ ((uintptr_t)L.order << 1);
	key.c = (uintptr_t)L.start;
	key.d = (uintptr_t)L.out_state;
	key.e = (uintptr_t)L.out_result;
	key.f = (uintptr_t)L.out_nevals;
	key.g = (uintptr_t)L.done_ns;
	key.n = L.n;
	key.p0 = L.max_evals;
	key.p1 = (int)m.blocks;
	key.p2 = m.threads;
	key.p3 = m.chunk | m.team << 16 | (int)m.solo << 24;
	key.deadline = L.budget_ns;
	cudaGraphExec_t exec = nullptr;
	auto it = graphs.find(key);
	if (it != graphs.end()) {
		exec = it->second;
	} else {
		if (!capture_stream)
			check_cuda(cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking), "stream");
		check_cuda(cudaStreamBeginCapture(capture_stream, cudaStreamCaptureModeThreadLocal), "capture");
		cudaMemsetAsync(aux.ptr, 0, 16, capture_stream);
		cudaMemsetAsync((char*)aux.ptr + 32, 0xff, 8, capture_stream);
		cudaError_t le = launch_shape(L, m, capture_stream);
		cudaMemcpyAsync(pinned_status, L.status, sizeof(int32_t), cudaMemcpyDeviceToHost, capture_stream);
		cudaGraph_t g = nullptr;
		cudaError_t ce = cudaStreamEndCapture(capture_stream, &g);
		if (le != cudaSuccess || ce != cudaSuccess) {
			if (g) cudaGraphDestroy(g);
			cudaGetLastError();      /* leave no stale error for the next call */
		}
		check_cuda(le, "minimize launch (capture)");
		check_cuda(ce, "end capture");
		cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
		cudaGraphDestroy(g);
		check_cuda(ie, "graph instantiate");
		if (graphs.size() > 64) clear_graphs();
		graphs.emplace(key, exec);
	}
	check_cuda(cudaGraphLaunch(exec, s), "graph launch");
	check_cuda(cudaStreamSynchronize(s), "minimize sync");
	if (status_out) *status_out = *pinned_status;
}

/* Concurrent launches, one per group: forked from and joined back into the
 * capture stream, so the whole batch is still one graph launch. */
void Context::run_minimize_groups(MinLaunch& L, const std::vector<MinGroup>& groups, cudaStream_t s,
		int32_t* status_out) {
	const size_t G = groups.size();
	if (G > kMaxGroups) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "batch minimize: too many launch shapes");
	if (!group_aux.ptr) {
		group_aux.alloc(64 * (kMaxGroups + 1));
		note_allocation();
		check_cuda(cudaMallocHost((void**)&pinned_group_status, sizeof(int32_t) * kMaxGroups), "cudaMallocHost");
	}
	while (group_streams.size() < G) {
		cudaStream_t st = nullptr;
		check_cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
		group_streams.push_back(st);
	}
	while (group_events.size() < G + 1) {
		cudaEvent_t ev = nullptr;
		check_cuda(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
		group_events.push_back(ev);
	}
	L.ref_order = (kernel_opts & GBA_KOPT_REFERENCE_ORDER) ? 1 : 0;
	std::vector<MinLaunch> Ls(G, L);
	std::vector<MinShape> shapes(G);
	uint64_t h = 1469598103934665603ull;
	for (size_t g = 0; g < G; ++g) {
		shapes[g] = min_shape(*this, groups[g].tp, groups[g].n, 1);
		MinLaunch& Lg = Ls[g];
		Lg.order = L.order + groups[g].off;
		Lg.n = groups[g].n;
		Lg.chunk = shapes[g].chunk;
		Lg.counter = (unsigned long long*)((char*)group_aux.ptr + 64 * g);
		Lg.status = (int*)((char*)group_aux.ptr + 64 * g + 8);
		Lg.t0 = (unsigned long long*)((char*)group_aux.ptr + 64 * kMaxGroups);
		for (uint64_t v : {(uint64_t)groups[g].off, (uint64_t)groups[g].n, (uint64_t)shapes[g].blocks,
				(uint64_t)shapes[g].threads, (uint64_t)shapes[g].chunk})
			h = (h ^ v) * 1099511628211ull;
	}
	L.t0 = Ls[0].t0;
	GraphKey key{};
	key.kind = 3;
	key.a = (uintptr_t)L.models;
	key.b = (uintptr_t)L.pair_of ^ ((uintptr_t)L.order << 1);
	key.c = (uintptr_t)L.start;
	key.d = (uintptr_t)L.out_state;
	key.e = (uintptr_t)L.out_result;
	key.f = (uintptr_t)L.out_nevals;
	key.g = (uintptr_t)L.done_ns;
	key.n = L.n;
	key.p0 = L.max_evals;
	key.p1 = (int)G;
	key.p2 = (int)(h & 0x7fffffff);
	key.p3 = (int)(h >> 33);
	key.deadline = L.budget_ns;
	cudaGraphExec_t exec = nullptr;
	auto it = graphs.find(key);
	if (it != graphs.end()) {
		exec = it->second;
	} else {
		if (!capture_stream)
			check_cuda(cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking), "stream");
		check_cuda(cudaStreamBeginCapture(capture_stream, cudaStreamCaptureModeThreadLocal), "capture");
		cudaError_t le = cudaSuccess;
		cudaMemsetAsync(group_aux.ptr, 0, 64 * G, capture_stream);
		cudaMemsetAsync((char*)group_aux.ptr + 64 * kMaxGroups, 0xff, 8, capture_stream);
		cudaEventRecord(group_events[G], capture_stream);
		for (size_t g = 0; g < G; ++g) {
			cudaStreamWaitEvent(group_streams[g], group_events[G], 0);
			cudaError_t e = launch_shape(Ls[g], shapes[g], group_streams[g]);
			if (le == cudaSuccess) le = e;
			cudaEventRecord(group_events[g], group_streams[g]);
			cudaStreamWaitEvent(capture_stream, group_events[g], 0);
		}
		for (size_t g = 0; g < G; ++g)
			cudaMemcpyAsync(pinned_group_status + g, Ls[g].status, sizeof(int32_t), cudaMemcpyDeviceToHost,
					capture_stream);
		cudaGraph_t gr = nullptr;
		cudaError_t ce = cudaStreamEndCapture(capture_stream, &gr);
		if (le != cudaSuccess || ce != cudaSuccess) {
			if (gr) cudaGraphDestroy(gr);
			cudaGetLastError();      /* leave no stale error for the next call */
		}
		check_cuda(le, "minimize launch (capture)");
		check_cuda(ce, "end capture");
		cudaError_t ie = cudaGraphInstantiate(&exec, gr, 0);
		cudaGraphDestroy(gr);
		check_cuda(ie, "graph instantiate");
		if (graphs.size() > 64) clear_graphs();
		graphs.emplace(key, exec);
	}
	check_cuda(cudaGraphLaunch(exec, s), "graph launch");
	check_cuda(cudaStreamSynchronize(s), "minimize sync");
	if (status_out) {
		*status_out = GBA_OK;
		for (size_t g = 0; g < G; ++g)
			if (pinned_group_status[g] != GBA_OK) *status_out = pinned_group_status[g];
	}
}

void Context::clear_graphs() {
	for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
	graphs.clear();
}

}  // namespace gba

using namespace gba;

#define GBA_TRY try {
#define GBA_CATCH(ctx)                                  \
	}                                                   \
	catch (const ApiError& e) {                         \
		(ctx)->set_error(e.what());                     \
		return e.code;                                  \
	}                                                   \
	catch (const std::exception& e) {                   \
		(ctx)->set_error(e.what());                     \
		return GBA_ERR_INVALID_ARGUMENT;                \
	}                                                   \
	return GBA_OK;

namespace {

/* Gathers the poses of all jobs into device arrays (staging slots 0..2),
 * returning per-job placements. */
struct Gathered {
	std::vector<RigidModel> models;
	std::vector<gba_id> key;
	std::vector<uint32_t> pair_of;
	std::vector<size_t> offset;
	size_t total = 0;
};

Gathered gather_jobs(Context* ctx, const gba_pair_job* jobs, size_t njobs) {
	Gathered G;
	for (size_t j = 0; j < njobs; ++j) {
		const gba_pair_job& jb = jobs[j];
		RigidLaunch L = ctx->rigid_launch(jb.rec, jb.lig, jb.grid, jb.params);
		G.models.push_back(L.m);
		G.key.insert(G.key.end(), {jb.rec, jb.lig, jb.grid, jb.params});
		G.offset.push_back(G.total);
		G.total += jb.n;
		if (jb.n && (!jb.start || !jb.out_result))
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "batch: job " + std::to_string(j) + " has null pointers");
	}
	if (G.total > 0xffffffffull) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "batch: more than 2^32 poses");
	G.pair_of.resize(G.total);
	for (size_t j = 0; j < njobs; ++j)
		std::fill(G.pair_of.begin() + G.offset[j], G.pair_of.begin() + G.offset[j] + jobs[j].n, (uint32_t)j);
	return G;
}

void copy_in(void* dst, const void* src, size_t bytes, cudaStream_t s) {
	check_cuda(cudaMemcpyAsync(dst, src, bytes, is_device_pointer(src) ? cudaMemcpyDeviceToDevice
			: cudaMemcpyHostToDevice, s), "batch: gather");
}

void copy_out(void* dst, const void* src, size_t bytes, cudaStream_t s) {
	check_cuda(cudaMemcpyAsync(dst, src, bytes, is_device_pointer(dst) ? cudaMemcpyDeviceToDevice
			: cudaMemcpyDeviceToHost, s), "batch: scatter");
}

}  // namespace

extern "C" {

int gba_set_minimize_team(gba_ctx* ctx, int warps_per_pose) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_TRY
	if (warps_per_pose < 0 || warps_per_pose > kMaxTeam)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_set_minimize_team: warps per pose must be 0.." +
				std::to_string(kMaxTeam));
	ctx->bind();
	Lock g(ctx->stage_mu);
	ctx->team_override = warps_per_pose;
	GBA_CATCH(ctx)
}

int gba_minimize_6d(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_dof6d* start, size_t n, int max_evals, gba_dof6d* out_state,
		gba_result6d* out_result, int32_t* out_nevals, void* stream) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	gba_pair_job job{rec, lig, grid, params, start, n, out_state, out_result, out_nevals, nullptr};
	return gba_batch_minimize_6d(ctx, &job, 1, max_evals, stream);
}

int gba_batch_minimize_6d(gba_ctx* ctx, const gba_pair_job* jobs, size_t njobs, int max_evals,
		void* stream) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_TRY
	if (njobs == 0) return GBA_OK;
	if (!jobs) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_batch_minimize_6d: null jobs");
	if (max_evals < 0) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "max_evals < 0");
	for (size_t j = 0; j < njobs; ++j)
		if (jobs[j].n && !jobs[j].out_state)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_batch_minimize_6d: null out_state");
	ctx->bind();
	cudaStream_t s = (cudaStream_t)stream;
	Lock lk(ctx->stage_mu);
	/* rigid_launch takes the items lock itself */
	Gathered G = gather_jobs(ctx, jobs, njobs);
	if (G.total == 0) return GBA_OK;
	const size_t n = G.total;
	const bool single_dev = njobs == 1 && is_device_pointer(jobs[0].start) &&
			is_device_pointer(jobs[0].out_state) && is_device_pointer(jobs[0].out_result) &&
			(!jobs[0].out_nevals || is_device_pointer(jobs[0].out_nevals));
	MinLaunch L{};
	L.n = n;
	L.max_evals = max_evals;
	L.models = models_on_device(ctx, G.models, G.key, s);
	if (njobs > 1) {
		ctx->pair_buf.upload(G.pair_of.data(), n * sizeof(uint32_t));
		L.pair_of = (const uint32_t*)ctx->pair_buf.ptr;
	}
	L.budget_ns = (unsigned long long)ctx->deadline_ms * 1000000ull;
	if (single_dev) {
		L.start = jobs[0].start;
		L.out_state = jobs[0].out_state;
		L.out_result = jobs[0].out_result;
		L.out_nevals = jobs[0].out_nevals;
	} else {
		L.start = (const gba_dof6d*)ctx->staging(0, n * sizeof(gba_dof6d));
		L.out_state = (gba_dof6d*)ctx->staging(1, n * sizeof(gba_dof6d));
		L.out_result = (gba_result6d*)ctx->staging(2, n * sizeof(gba_result6d));
		L.out_nevals = (int32_t*)ctx->staging(3, n * sizeof(int32_t));
	}
	bool want_done = false;
	for (size_t j = 0; j < njobs; ++j) want_done |= jobs[j].out_done_ns != nullptr && jobs[j].n > 0;
	if (want_done) L.done_ns = (unsigned long long*)ctx->staging(4, n * sizeof(unsigned long long));
	if (!single_dev) {
		for (size_t j = 0; j < njobs; ++j)
			if (jobs[j].n) copy_in((void*)(L.start + G.offset[j]), jobs[j].start, jobs[j].n * sizeof(gba_dof6d), s);
	}
	/* launch shapes: the pairs' tuned shapes (gba_autotune), else the
	 * context's; a job small enough for teams runs as one team launch */
	uint32_t lig_rounds = 1;
	for (const RigidModel& m : G.models) lig_rounds = std::max(lig_rounds, (m.lig.n + 63) / 64);
	std::vector<TuneParams> tps(njobs);
	for (size_t j = 0; j < njobs; ++j)
		tps[j] = ctx->pair_tuned("minimize", PairKey{jobs[j].rec, jobs[j].lig, jobs[j].grid, jobs[j].params});
	const TuneParams base_tp = njobs == 1 ? tps[0] : ctx->tuned("minimize", n);
	const bool team_launch = ctx->minimize_team(base_tp, n, lig_rounds) > 1;
	/* group index of each job: one per distinct (threads, chunk) */
	std::vector<uint32_t> group_of(njobs, 0);
	std::vector<TuneParams> group_tp{tps[0]};
	if (!team_launch)
		for (size_t j = 1; j < njobs; ++j) {
			size_t g = 0;
			while (g < group_tp.size() &&
					!(group_tp[g].threads == tps[j].threads && group_tp[g].chunk == tps[j].chunk &&
					  group_tp[g].blocks_per_sm == tps[j].blocks_per_sm))
				++g;
			if (g == group_tp.size()) group_tp.push_back(tps[j]);
			group_of[j] = (uint32_t)g;
		}
	const bool grouped = group_tp.size() > 1;
	if (group_tp.size() > Context::kMaxGroups) throw ApiError(GBA_ERR_INVALID_ARGUMENT,
			"gba_batch_minimize_6d: more than " + std::to_string(Context::kMaxGroups) + " tuned launch shapes");
	/* visit poses grouped by pair, in Morton order of the start translation;
	 * pairs with larger ligands (more work per evaluation) first, so that the
	 * poses still running when the queue empties are cheap ones; with
	 * several launch shapes the pairs of one shape come together */
	const uint32_t* pair_rank = nullptr;
	std::vector<uint32_t> by_cost(njobs), rank(njobs);
	for (size_t j = 0; j < njobs; ++j) by_cost[j] = (uint32_t)j;
	std::stable_sort(by_cost.begin(), by_cost.end(), [&](uint32_t a, uint32_t b) {
		if (group_of[a] != group_of[b]) return group_of[a] < group_of[b];
		return G.models[a].lig.n > G.models[b].lig.n;
	});
	for (size_t r = 0; r < njobs; ++r) rank[by_cost[r]] = (uint32_t)r;
	if (njobs > 1) {
		ctx->rank_buf.upload(rank.data(), njobs * sizeof(uint32_t));
		pair_rank = (const uint32_t*)ctx->rank_buf.ptr;
	}
	L.order = ctx->pose_order_persistent(L.start, 6, n, G.models[0].grid.outer, L.models, L.pair_of,
			pair_rank, njobs, s);
	int32_t status = GBA_OK;
	if (!grouped) {
		ctx->run_minimize(L, s, &status, lig_rounds, base_tp);
	} else {
		if (!L.order) {
			/* no spatial order (small batch or switched off): pairs of one
			 * shape together, each pair's poses in submission order */
			std::vector<uint32_t> ord;
			ord.reserve(n);
			for (uint32_t j : by_cost)
				for (size_t k = 0; k < jobs[j].n; ++k) ord.push_back((uint32_t)(G.offset[j] + k));
			DevBuffer& b = ctx->order_buf;
			if (b.bytes < n * sizeof(uint32_t)) b.alloc(n * sizeof(uint32_t) + 256);
			check_cuda(cudaMemcpyAsync(b.ptr, ord.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, s),
					"batch minimize: order");
			L.order = (const uint32_t*)b.ptr;
		}
		std::vector<Context::MinGroup> groups(group_tp.size());
		size_t off = 0;
		for (size_t g = 0; g < group_tp.size(); ++g) {
			groups[g].off = off;
			groups[g].tp = group_tp[g];
			groups[g].n = 0;
			for (size_t j = 0; j < njobs; ++j)
				if (group_of[j] == g) groups[g].n += jobs[j].n;
			off += groups[g].n;
		}
		ctx->run_minimize_groups(L, groups, s, &status);
	}
	if (!single_dev) {
		for (size_t j = 0; j < njobs; ++j) {
			const size_t o = G.offset[j], m = jobs[j].n;
			if (!m) continue;
			copy_out(jobs[j].out_state, L.out_state + o, m * sizeof(gba_dof6d), s);
			copy_out(jobs[j].out_result, L.out_result + o, m * sizeof(gba_result6d), s);
			if (jobs[j].out_nevals) copy_out(jobs[j].out_nevals, L.out_nevals + o, m * sizeof(int32_t), s);
		}
		check_cuda(cudaStreamSynchronize(s), "batch minimize: scatter");
	}
	if (want_done) {
		std::vector<unsigned long long> d(n);
		unsigned long long t0 = 0;
		check_cuda(cudaMemcpy(d.data(), L.done_ns, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost),
				"batch minimize: completion times");
		check_cuda(cudaMemcpy(&t0, L.t0, sizeof(t0), cudaMemcpyDeviceToHost), "batch minimize: start time");
		for (size_t j = 0; j < njobs; ++j)
			if (jobs[j].out_done_ns)
				for (size_t k = 0; k < jobs[j].n; ++k) {
					const unsigned long long v = d[G.offset[j] + k];
					jobs[j].out_done_ns[k] = v >= t0 ? v - t0 : 0;
				}
	}
	if (status == GBA_ERR_TIMEOUT)
		throw ApiError(GBA_ERR_TIMEOUT, "minimization stopped: device wall-time budget exhausted");
	if (status == GBA_ERR_DEVICE_CHECK)
		throw ApiError(GBA_ERR_DEVICE_CHECK, "minimization stopped: a pose exceeded its evaluation budget");
	GBA_CATCH(ctx)
}

int gba_batch_energy_6d(gba_ctx* ctx, const gba_pair_job* jobs, size_t njobs, void* stream) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_TRY
	if (njobs == 0) return GBA_OK;
	if (!jobs) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_batch_energy_6d: null jobs");
	ctx->bind();
	cudaStream_t s = (cudaStream_t)stream;
	Lock lk(ctx->stage_mu);
	/* rigid_launch takes the items lock itself */
	Gathered G = gather_jobs(ctx, jobs, njobs);
	if (G.total == 0) return GBA_OK;
	const size_t n = G.total;
	BatchEnergyLaunch L{};
	L.n = n;
	L.ref_order = (ctx->kernel_opts & GBA_KOPT_REFERENCE_ORDER) ? 1 : 0;
	L.models = models_on_device(ctx, G.models, G.key, s);
	ctx->pair_buf.upload(G.pair_of.data(), n * sizeof(uint32_t));
	L.pair_of = (const uint32_t*)ctx->pair_buf.ptr;
	L.dofs = (const gba_dof6d*)ctx->staging(0, n * sizeof(gba_dof6d));
	L.out = (gba_result6d*)ctx->staging(2, n * sizeof(gba_result6d));
	for (size_t j = 0; j < njobs; ++j)
		if (jobs[j].n) copy_in((void*)(L.dofs + G.offset[j]), jobs[j].start, jobs[j].n * sizeof(gba_dof6d), s);
	StreamScratch scratch(ctx->scratch_pool);
	L.next = (unsigned long long*)scratch.get(sizeof(unsigned long long), s);
	check_cuda(cudaMemsetAsync(L.next, 0, sizeof(unsigned long long), s), "batch energy: pose counter");
	const int threads = 256;
	size_t blocks = std::max<size_t>(1, std::min<size_t>((n + 7) / 8, (size_t)ctx->num_sms * 3));
	check_cuda(launch_batch_energy(L, (int)blocks, threads, s), "batch energy launch");
	for (size_t j = 0; j < njobs; ++j)
		if (jobs[j].n) copy_out(jobs[j].out_result, L.out + G.offset[j], jobs[j].n * sizeof(gba_result6d), s);
	check_cuda(cudaStreamSynchronize(s), "batch energy");
	GBA_CATCH(ctx)
}

int gba_minimize_6d_plain(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_dof6d* start, size_t n, int max_evals, size_t item_size, gba_dof6d* out_state,
		gba_result6d* out_result, int32_t* out_nevals, void* stream) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_TRY
	if (n == 0) return GBA_OK;
	if (!start || !out_state || !out_result)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_minimize_6d_plain: null pointer");
	if (max_evals < 0) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "max_evals < 0");
	if (is_device_pointer(start) || is_device_pointer(out_state) || is_device_pointer(out_result))
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_minimize_6d_plain: host pointers required");
	ctx->bind();
	cudaStream_t s = (cudaStream_t)stream;
	RigidLaunch L = ctx->rigid_launch(rec, lig, grid, params);
	const TuneParams shape = ctx->pair_tuned("energy", PairKey{rec, lig, grid, params});
	Lock lk(ctx->stage_mu);
	/* pinned request/result buffers, like the server's HostPinnedAllocator
	 * buffers (src/service/GPUEnergyService.tpp:22-23) */
	gba_dof6d* hin = (gba_dof6d*)ctx->pinned(0, n * sizeof(gba_dof6d));
	gba_result6d* hout = (gba_result6d*)ctx->pinned(1, n * sizeof(gba_result6d));
	gba_dof6d* din = (gba_dof6d*)ctx->staging(0, n * sizeof(gba_dof6d));
	gba_result6d* dout = (gba_result6d*)ctx->staging(1, n * sizeof(gba_result6d));
	std::vector<VA13<6>> va(n);
	std::vector<size_t> active(n), next;
	std::vector<int32_t> nev(n, 0);
	for (size_t p = 0; p < n; ++p) {
		const double x0[6] = {start[p].ang[0], start[p].ang[1], start[p].ang[2], start[p].pos[0],
				start[p].pos[1], start[p].pos[2]};
		va[p].start(x0, 6, max_evals);
		active[p] = p;
	}
	/* VA13 ends within max_evals + 1 evaluations per pose: so do the rounds */
	for (int round = 0; !active.empty(); ++round) {
		if (round > max_evals + 1)
			throw ApiError(GBA_ERR_DEVICE_CHECK, "plain minimization: a pose exceeded its evaluation budget");
		const size_t na = active.size();
		for (size_t k = 0; k < na; ++k) {
			const double* pt = va[active[k]].point();
			gba_dof6d& d = hin[k];
			d.ang[0] = (float)pt[0]; d.ang[1] = (float)pt[1]; d.ang[2] = (float)pt[2];
			d.pos[0] = (float)pt[3]; d.pos[1] = (float)pt[4]; d.pos[2] = (float)pt[5];
		}
		/* one round = the active poses cut into work items (src/server/ServerFunctions.h:50),
		 * each copied in, evaluated by one launch and copied out */
		const size_t item = item_size ? item_size : na;
		for (size_t b = 0; b < na; b += item) {
			const size_t m = std::min(item, na - b);
			check_cuda(cudaMemcpyAsync(din + b, hin + b, m * sizeof(gba_dof6d), cudaMemcpyHostToDevice, s),
					"plain: H2D");
			L.dofs = din + b;
			L.out = dout + b;
			L.n = m;
			L.census = nullptr;
			L.roundwise = 1;      /* the device minimizer's summation order */
			ctx->run_rigid(L, s, &shape);
			check_cuda(cudaMemcpyAsync(hout + b, dout + b, m * sizeof(gba_result6d), cudaMemcpyDeviceToHost, s),
					"plain: D2H");
		}
		check_cuda(cudaStreamSynchronize(s), "plain: sync");
		next.clear();
		for (size_t k = 0; k < na; ++k) {
			const size_t p = active[k];
			const gba_result6d& r = hout[k];
			out_state[p] = hin[k];
			out_result[p] = r;
			++nev[p];
			const double g[6] = {-(double)r.ang[0], -(double)r.ang[1], -(double)r.ang[2],
					-(double)r.pos[0], -(double)r.pos[1], -(double)r.pos[2]};
			va[p].provide((double)r.E, g);
			if (!va[p].done()) next.push_back(p);
		}
		active.swap(next);
	}
	if (out_nevals) std::memcpy(out_nevals, nev.data(), n * sizeof(int32_t));
	GBA_CATCH(ctx)
}

int gba_minimize_6d_modes(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid_rec, gba_id grid_lig,
		gba_id params, const gba_dof6d_modes* start, size_t n, int max_evals,
		gba_dof6d_modes* out_state, gba_result6d_modes* out_result, int32_t* out_nevals,
		void* stream) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_TRY
	if (n == 0) return GBA_OK;
	if (!start || !out_state || !out_result)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_minimize_6d_modes: null pointer");
	if (max_evals < 0) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "max_evals < 0");
	ctx->bind();
	cudaStream_t s = (cudaStream_t)stream;
	ModesMinLaunch M{};
	M.m = ctx->modes_launch(rec, lig, grid_rec, grid_lig, params);
	Lock lk(ctx->stage_mu);
	const bool dev = is_device_pointer(start) && is_device_pointer(out_state) &&
			is_device_pointer(out_result) && (!out_nevals || is_device_pointer(out_nevals));
	M.n = n;
	M.max_evals = max_evals;
	if (dev) {
		M.start = start;
		M.out_state = out_state;
		M.out_result = out_result;
		M.out_nevals = out_nevals;
	} else {
		M.start = (const gba_dof6d_modes*)ctx->staging(0, n * sizeof(gba_dof6d_modes));
		M.out_state = (gba_dof6d_modes*)ctx->staging(1, n * sizeof(gba_dof6d_modes));
		M.out_result = (gba_result6d_modes*)ctx->staging(2, n * sizeof(gba_result6d_modes));
		M.out_nevals = (int32_t*)ctx->staging(3, n * sizeof(int32_t));
		copy_in((void*)M.start, start, n * sizeof(gba_dof6d_modes), s);
	}
	if (!ctx->aux.ptr) {
		ctx->aux.alloc(64);
		note_allocation();
		check_cuda(cudaMallocHost((void**)&ctx->pinned_status, sizeof(int32_t)), "cudaMallocHost");
	}
	/* aux [12,16): modes status, [16,24): modes cursor */
	M.status = (int*)((char*)ctx->aux.ptr + 12);
	M.counter = (unsigned long long*)((char*)ctx->aux.ptr + 16);
	check_cuda(cudaMemsetAsync((char*)ctx->aux.ptr + 12, 0, 12, s), "modes minimize: cursor");
	const int threads = 128;
	const int bps = minimize_modes_blocks_per_sm(threads, M.m);
	size_t blocks = std::max<size_t>(1, std::min<size_t>((n * 32 + threads - 1) / threads,
			(size_t)ctx->num_sms * bps));
	StreamScratch scratch(ctx->scratch_pool);
	if (M.m.ref_order)   /* the reference order's receptor arrays, one per warp */
		M.m.ref_rf = (float4*)scratch.get(blocks * (threads / 32) * std::max<uint32_t>(1, M.m.rec.n) *
				sizeof(float4), s);
	check_cuda(launch_minimize_modes(M, (int)blocks, threads, s), "modes minimize launch");
	if (!dev) {
		copy_out(out_state, M.out_state, n * sizeof(gba_dof6d_modes), s);
		copy_out(out_result, M.out_result, n * sizeof(gba_result6d_modes), s);
		if (out_nevals) copy_out(out_nevals, M.out_nevals, n * sizeof(int32_t), s);
	}
	check_cuda(cudaMemcpyAsync(ctx->pinned_status, M.status, sizeof(int32_t), cudaMemcpyDeviceToHost, s),
			"modes minimize: status");
	check_cuda(cudaStreamSynchronize(s), "modes minimize");
	if (*ctx->pinned_status == GBA_ERR_TIMEOUT)
		throw ApiError(GBA_ERR_TIMEOUT, "modes minimization stopped: device wall-time cap reached");
	if (*ctx->pinned_status == GBA_ERR_DEVICE_CHECK)
		throw ApiError(GBA_ERR_DEVICE_CHECK, "modes minimization stopped: a pose exceeded its evaluation budget");
	GBA_CATCH(ctx)
}

int gba_minimize_6d_modes_plain(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid_rec,
		gba_id grid_lig, gba_id params, const gba_dof6d_modes* start, size_t n, int max_evals,
		size_t item_size, gba_dof6d_modes* out_state, gba_result6d_modes* out_result,
		int32_t* out_nevals, void* stream) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_TRY
	if (n == 0) return GBA_OK;
	if (!start || !out_state || !out_result)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_minimize_6d_modes_plain: null pointer");
	if (max_evals < 0) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "max_evals < 0");
	if (is_device_pointer(start) || is_device_pointer(out_state) || is_device_pointer(out_result))
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_minimize_6d_modes_plain: host pointers required");
	ctx->bind();
	cudaStream_t s = (cudaStream_t)stream;
	ModesLaunch L = ctx->modes_launch(rec, lig, grid_rec, grid_lig, params);
	const int Mr = (int)L.rec.n_modes, Ml = (int)L.lig.n_modes, jn = 6 + Mr + Ml;
	Lock lk(ctx->stage_mu);
	auto* hin = (gba_dof6d_modes*)ctx->pinned(0, n * sizeof(gba_dof6d_modes));
	auto* hout = (gba_result6d_modes*)ctx->pinned(1, n * sizeof(gba_result6d_modes));
	auto* din = (gba_dof6d_modes*)ctx->staging(0, n * sizeof(gba_dof6d_modes));
	auto* dout = (gba_result6d_modes*)ctx->staging(1, n * sizeof(gba_result6d_modes));
	std::vector<VA13<6 + 2 * GBA_MODES_MAX>> va(n);
	std::vector<size_t> active(n), next;
	std::vector<int32_t> nev(n, 0);
	for (size_t p = 0; p < n; ++p) {
		double x0[6 + 2 * GBA_MODES_MAX];
		for (int k = 0; k < 3; ++k) { x0[k] = start[p].rigid.ang[k]; x0[3 + k] = start[p].rigid.pos[k]; }
		for (int m = 0; m < Mr; ++m) x0[6 + m] = start[p].modesRec[m];
		for (int m = 0; m < Ml; ++m) x0[6 + Mr + m] = start[p].modesLig[m];
		va[p].start(x0, jn, max_evals);
		active[p] = p;
	}
	/* VA13 ends within max_evals + 1 evaluations per pose: so do the rounds */
	for (int round = 0; !active.empty(); ++round) {
		if (round > max_evals + 1)
			throw ApiError(GBA_ERR_DEVICE_CHECK, "plain minimization: a pose exceeded its evaluation budget");
		const size_t na = active.size();
		for (size_t k = 0; k < na; ++k) {
			const double* pt = va[active[k]].point();
			gba_dof6d_modes& d = hin[k];
			std::memset(&d, 0, sizeof(d));
			for (int a = 0; a < 3; ++a) { d.rigid.ang[a] = (float)pt[a]; d.rigid.pos[a] = (float)pt[3 + a]; }
			for (int m = 0; m < Mr; ++m) d.modesRec[m] = (float)pt[6 + m];
			for (int m = 0; m < Ml; ++m) d.modesLig[m] = (float)pt[6 + Mr + m];
		}
		/* one round = the active poses cut into work items, each copied in,
		 * evaluated by one launch and copied out */
		const size_t item = item_size ? item_size : na;
		for (size_t b = 0; b < na; b += item) {
			const size_t m = std::min(item, na - b);
			check_cuda(cudaMemcpyAsync(din + b, hin + b, m * sizeof(gba_dof6d_modes), cudaMemcpyHostToDevice, s),
					"H2D");
			L.dofs = din + b;
			L.out = dout + b;
			L.n = m;
			ctx->run_modes(L, s);
			check_cuda(cudaMemcpyAsync(hout + b, dout + b, m * sizeof(gba_result6d_modes), cudaMemcpyDeviceToHost,
					s), "D2H");
		}
		check_cuda(cudaStreamSynchronize(s), "plain modes: sync");
		next.clear();
		for (size_t k = 0; k < na; ++k) {
			const size_t p = active[k];
			const gba_result6d_modes& r = hout[k];
			out_state[p] = hin[k];
			out_result[p] = r;
			++nev[p];
			double g[6 + 2 * GBA_MODES_MAX];
			for (int a = 0; a < 3; ++a) { g[a] = -(double)r.rigid.ang[a]; g[3 + a] = -(double)r.rigid.pos[a]; }
			/* mode entries are gradients already (reduceModeForce) */
			for (int m = 0; m < Mr; ++m) g[6 + m] = (double)r.modesRec[m];
			for (int m = 0; m < Ml; ++m) g[6 + Mr + m] = (double)r.modesLig[m];
			va[p].provide((double)r.rigid.E, g);
			if (!va[p].done()) next.push_back(p);
		}
		active.swap(next);
	}
	if (out_nevals) std::memcpy(out_nevals, nev.data(), n * sizeof(int32_t));
	GBA_CATCH(ctx)
}

int gba_set_deadline(gba_ctx* ctx, uint32_t milliseconds) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	ctx->deadline_ms = milliseconds;
	return GBA_OK;
}

}  // extern "C"
