/*
 * autotune.cu -- picks launch shapes for one receptor-ligand pair by timing
 * them on a sample of its poses.
 *
 *   energy    threads per block {128, 256} x resident blocks per SM
 *             {1 .. occupancy limit} of the fused scoring kernel
 *   minimize  one warp per pose: threads per block {64, 128, 256} x poses
 *             claimed per queue grab {1, 2, 4} (resident blocks = the
 *             occupancy limit: the kernel is persistent); and teams of 2 ..
 *             min(ligand rounds, 7) warps per pose -- poses per CTA below
 *             one -- for jobs the size of the sample
 * Each candidate runs on the caller's sample poses, timed with CUDA events
 * (best of three for scoring, two for minimization); the winners are kept
 * in the context for this pair (gba_energy_6d, gba_minimize_6d and batches
 * containing the pair launch with them) and, when a cache path is given, in
 * a text file keyed by device name, SM count and pair size (bead counts
 * rounded to 64; the team also by the sample size), so later processes skip
 * the search.
 */
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "gba_context.h"

namespace gba {

namespace {

struct EventTimer {
	cudaEvent_t a = nullptr, b = nullptr;
	EventTimer() {
		check_cuda(cudaEventCreate(&a), "event");
		check_cuda(cudaEventCreate(&b), "event");
	}
	~EventTimer() {
		cudaEventDestroy(a);
		cudaEventDestroy(b);
	}
	template <typename F>
	float best_ms(F run, cudaStream_t s, int reps = 3) {
		float best = 1e30f;
		for (int r = 0; r < reps; ++r) {
			check_cuda(cudaEventRecord(a, s), "event");
			run();
			check_cuda(cudaEventRecord(b, s), "event");
			check_cuda(cudaEventSynchronize(b), "event sync");
			float ms = 0.f;
			check_cuda(cudaEventElapsedTime(&ms, a, b), "elapsed");
			best = std::min(best, ms);
		}
		return best;
	}
};

std::string cache_key(const Context* ctx, const char* kind, uint32_t nrec, uint32_t nlig) {
	cudaDeviceProp prop;
	cudaGetDeviceProperties(&prop, ctx->device);
	std::ostringstream k;
	std::string name = prop.name;
	std::replace(name.begin(), name.end(), ' ', '_');
	k << kind << ' ' << name << ' ' << prop.multiProcessorCount << ' ' << ((nrec + 63) / 64) * 64
	  << ' ' << ((nlig + 63) / 64) * 64;
	return k.str();
}

bool cache_lookup(const char* path, const std::string& key, TuneParams& tp) {
	if (!path) return false;
	std::ifstream f(path);
	std::string line;
	bool found = false;
	while (std::getline(f, line)) {
		if (line.compare(0, key.size(), key) != 0 || line.size() <= key.size() || line[key.size()] != ' ')
			continue;
		std::istringstream in(line.substr(key.size()));
		TuneParams t;
		if (in >> t.threads >> t.blocks_per_sm >> t.chunk) {
			int team = 0;
			size_t poses = 0;
			if (in >> team >> poses) {
				t.team = team;
				t.team_poses = poses;
			}
			tp = t;
			found = true;
		}
	}
	return found;
}

void cache_store(const char* path, const std::string& key, const TuneParams& tp) {
	if (!path) return;
	std::ofstream f(path, std::ios::app);
	f << key << ' ' << tp.threads << ' ' << tp.blocks_per_sm << ' ' << tp.chunk << ' ' << tp.team << ' '
	  << tp.team_poses << '\n';
}

}  // namespace

}  // namespace gba

using namespace gba;

extern "C" int gba_autotune(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_dof6d* sample, size_t n, int max_evals, const char* cache_path,
		gba_tune_result* out) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	try {
		if (!sample || n == 0) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_autotune: empty sample");
		ctx->bind();
		RigidLaunch base = ctx->rigid_launch(rec, lig, grid, params);
		const PairKey pk{rec, lig, grid, params};
		const uint32_t rounds = (base.m.lig.n + 63) / 64;
		const std::string ek = cache_key(ctx, "energy", base.m.rec.n, base.m.lig.n);
		const std::string mk = cache_key(ctx, "minimize", base.m.rec.n, base.m.lig.n) + " " + std::to_string(n);
		TuneParams te, tm;
		const bool have_e = cache_lookup(cache_path, ek, te);
		const bool have_m = cache_lookup(cache_path, mk, tm);
		float best_e = -1.f, best_m = -1.f;
		if (!have_e || !have_m) {
			Lock lk(ctx->stage_mu);
			cudaStream_t s = 0;
			gba_dof6d* d = (gba_dof6d*)ctx->staging(0, n * sizeof(gba_dof6d));
			check_cuda(cudaMemcpy(d, sample, n * sizeof(gba_dof6d), cudaMemcpyDefault), "sample");
			gba_result6d* r = (gba_result6d*)ctx->staging(1, n * sizeof(gba_result6d));
			EventTimer T;
			StreamScratch scratch(ctx->scratch_pool);
			unsigned long long* next = (unsigned long long*)scratch.get(sizeof(unsigned long long), s);
			if (!have_e) {
				best_e = 1e30f;
				for (int threads : {128, 256}) {
					const int maxb = rigid_blocks_per_sm(threads, false, base.bound4 != 0, false, base.ref_order != 0);
					for (int bps = 1; bps <= maxb; ++bps) {
						RigidLaunch L = base;
						L.dofs = d;
						L.out = r;
						L.n = n;
						L.next = next;
						const size_t blocks = std::max<size_t>(1, std::min<size_t>(
								(n + threads / 32 - 1) / (threads / 32), (size_t)ctx->num_sms * bps));
						const float ms = T.best_ms([&] {
							check_cuda(cudaMemsetAsync(next, 0, sizeof(unsigned long long), s), "tune: pose counter");
							check_cuda(launch_rigid_energy(L, (int)blocks, threads, s), "tune launch");
						}, s);
						if (ms < best_e) {
							best_e = ms;
							te = TuneParams{threads, bps, 1};
						}
					}
				}
				cache_store(cache_path, ek, te);
			}
			if (!have_m) {
				best_m = 1e30f;
				gba_dof6d* st = (gba_dof6d*)ctx->staging(2, n * sizeof(gba_dof6d));
				gba_result6d* rs = (gba_result6d*)ctx->staging(3, n * sizeof(gba_result6d));
				std::vector<RigidModel> models{base.m};
				DevBuffer mb;
				mb.upload(models.data(), sizeof(RigidModel));
				const int evals = std::min(std::max(max_evals, 1), 50);
				std::vector<TuneParams> cand;
				for (int threads : {64, 128, 256})
					for (int chunk : {1, 2, 4}) cand.push_back(TuneParams{threads, 64, chunk, 1, n});
				for (int team = 2; team <= std::min<int>(kMaxTeam, (int)rounds); ++team)
					cand.push_back(TuneParams{128, 64, 1, team, n});
				const int saved_override = ctx->team_override;
				ctx->team_override = 0;
				for (const TuneParams& c : cand) {
					MinLaunch L{};
					L.models = (const RigidModel*)mb.ptr;
					L.start = d;
					L.out_state = st;
					L.out_result = rs;
					L.n = n;
					L.max_evals = evals;
					const float ms = T.best_ms([&] { ctx->run_minimize(L, s, nullptr, rounds, c); }, s, 2);
					if (ms < best_m) {
						best_m = ms;
						tm = c;
					}
				}
				ctx->team_override = saved_override;
				ctx->clear_graphs();
				cache_store(cache_path, mk, tm);
			}
		}
		ctx->set_pair_tuned("energy", pk, te);
		ctx->set_pair_tuned("minimize", pk, tm);
		if (out) {
			out->energy_threads = te.threads;
			out->energy_blocks_per_sm = te.blocks_per_sm;
			out->minimize_threads = tm.team > 1 ? 32 * (tm.team + 1) : tm.threads;
			out->minimize_chunk = tm.chunk;
			out->minimize_team = tm.team > 1 ? tm.team : 1;
			out->energy_ms = best_e;
			out->minimize_ms = best_m;
			out->from_cache = (have_e ? 1 : 0) | (have_m ? 2 : 0);
		}
	} catch (const ApiError& e) {
		ctx->set_error(e.what());
		return e.code;
	} catch (const std::exception& e) {
		ctx->set_error(e.what());
		return GBA_ERR_INVALID_ARGUMENT;
	}
	return GBA_OK;
}

extern "C" int gba_set_pair_shape(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_tune_result* shape) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	try {
		if (!shape) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_set_pair_shape: null shape");
		const gba_tune_result& t = *shape;
		const auto threads_ok = [](int th) { return th >= 32 && th <= 256 && th % 32 == 0; };
		if (!threads_ok(t.energy_threads) || t.energy_blocks_per_sm < 1)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_set_pair_shape: bad energy shape");
		if (t.minimize_team < 1 || t.minimize_team > kMaxTeam)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_set_pair_shape: minimize_team must be 1.." +
					std::to_string(kMaxTeam));
		if (t.minimize_team == 1 && (!threads_ok(t.minimize_threads) || t.minimize_chunk < 1 || t.minimize_chunk > 16))
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_set_pair_shape: bad minimize shape");
		ctx->bind();
		{
			Lock g(ctx->mu);     /* the ids must name a valid pair */
			ctx->find(rec, ItemKind::Protein);
			ctx->find(lig, ItemKind::Protein);
			ctx->find(grid, ItemKind::Grid);
			ctx->find(params, ItemKind::Params);
		}
		const PairKey pk{rec, lig, grid, params};
		ctx->set_pair_tuned("energy", pk, TuneParams{t.energy_threads, t.energy_blocks_per_sm, 1, 0, 0});
		TuneParams m{t.minimize_team == 1 ? t.minimize_threads : 128, 64, t.minimize_team == 1 ? t.minimize_chunk : 1,
				t.minimize_team, (size_t)-1};
		ctx->set_pair_tuned("minimize", pk, m);
	} catch (const ApiError& e) {
		ctx->set_error(e.what());
		return e.code;
	} catch (const std::exception& e) {
		ctx->set_error(e.what());
		return GBA_ERR_INVALID_ARGUMENT;
	}
	return GBA_OK;
}
