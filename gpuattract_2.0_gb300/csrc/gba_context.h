/*
 * gba_context.h -- host-side state behind a gba_ctx handle.
 */
#ifndef GBA_CONTEXT_H_
#define GBA_CONTEXT_H_

#include <array>
#include <map>
#include <memory>
#include <set>
#include <atomic>
#include <mutex>
#include <thread>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>
#include <cstring>

#include "gba_internal.h"

namespace gba {

/* Carries a GBA_ERR_* code through the C++ implementation to the C ABI. */
struct ApiError : std::runtime_error {
	int code;
	ApiError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

/* A mutex that refuses to be taken twice by the same thread: a nested lock
 * becomes an ApiError instead of a silent self-deadlock. */
class CheckedMutex {
public:
	void lock() {
		if (owner_.load(std::memory_order_relaxed) == std::this_thread::get_id())
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "internal error: context lock taken twice by one thread");
		m_.lock();
		owner_.store(std::this_thread::get_id(), std::memory_order_relaxed);
	}
	void unlock() {
		owner_.store(std::thread::id(), std::memory_order_relaxed);
		m_.unlock();
	}

private:
	std::mutex m_;
	std::atomic<std::thread::id> owner_{};
};
using Lock = std::lock_guard<CheckedMutex>;

void check_cuda(cudaError_t e, const char* what);
bool is_device_pointer(const void* p);

/* Counts every device or pinned-host allocation the library makes
 * (gba_allocation_count). */
void note_allocation();

/* One cudaMalloc'd buffer, freed on destruction. */
struct DevBuffer {
	void* ptr = nullptr;
	size_t bytes = 0;
	DevBuffer() = default;
	DevBuffer(const DevBuffer&) = delete;
	DevBuffer& operator=(const DevBuffer&) = delete;
	~DevBuffer() { release(); }
	void alloc(size_t b);
	void release();
	void upload(const void* src, size_t b);
};

/* Stream-ordered scratch: allocated on a stream, freed on it when the
 * holder goes out of scope (after the work that reads it was enqueued).
 * From `pool` when given (the context's pool keeps its memory reserved
 * between calls; the default pool gives it back at every synchronisation and
 * then costs ~90 us of host time per allocation). */
struct StreamScratch {
	std::vector<void*> ptrs;
	cudaStream_t stream = nullptr;
	cudaMemPool_t pool = nullptr;
	void* get(size_t bytes, cudaStream_t s);
	explicit StreamScratch(cudaMemPool_t p = nullptr) : pool(p) {}
	StreamScratch(const StreamScratch&) = delete;
	~StreamScratch();
};

enum class ItemKind { Protein, Grid, Params };
const char* kind_name(ItemKind k);

struct Item {
	ItemKind kind;
	explicit Item(ItemKind k) : kind(k) {}
	virtual ~Item() {}
};

struct ProteinItem : Item {
	ProteinItem() : Item(ItemKind::Protein) {}
	DevBuffer xyzq, tm, modes;
	DevProtein dev{};
	uint32_t max_type = 0, max_mapped = 0;
	std::vector<float> host_xyz;   /* SoA copy for host-side layout work */
};

struct GridItem : Item {
	GridItem() : Item(ItemKind::Grid) {}
	DevBuffer inner, outer, nlgrid, nllist, ratio;
	DevBuffer inner_oct, outer_oct;   /* optional duplicated-octet copies */
	DevGrid dev{};
	gba_intrpl_desc inner_desc{}, outer_desc{};
	gba_nl_desc nl_desc{};
	uint32_t nl_max_index = 0;
	bool nl_has_entries = false;
	/* radius around a voxel centre that its list is known to cover: the
	 * builder's nl_cutoff, or for uploaded grids the least radius the
	 * reference's NL term relies on (plateau + half a voxel diagonal) */
	double nl_list_radius = 0.0;
	/* per receptor id: the list with that receptor's bead types in bits 24..31 */
	std::map<gba_id, DevBuffer> typed_lists;
};

struct ParamsItem : Item {
	ParamsItem() : Item(ItemKind::Params) {}
	DevBuffer lj, ivor;
	DevParams dev{};
	std::vector<gba_ffparam> host_table;
	/* per plateau^2 (bit pattern): the pair-term table with the plateau
	 * terms folded in (plateau_table) */
	std::map<uint32_t, std::unique_ptr<DevBuffer>> pair_tables;
	/* the table for plateau^2 dPlateau2; built on first use when
	 * may_allocate, else an ApiError if it does not exist yet */
	const float4* pair_table(float dPlateau2, bool may_allocate = true);
};

/* Visiting order of n poses (grouped by translation cell) computed in the
 * given device memory (pose_order.cu); throws ApiError if [buf, buf + cap)
 * is too small. */
const uint32_t* pose_order_in(const void* dofs, size_t stride_floats, size_t n, const DevIntrpl& box,
		void* buf, size_t cap, cudaStream_t s);

DevIntrpl intrpl_from_desc(const gba_intrpl_desc& d);
DevNL nl_from_desc(const gba_nl_desc& d);
std::vector<float> nl_ratio_table(float dPlateau2);

/* Launch shape chosen by the autotuner (or the defaults). */
struct TuneParams {
	int threads = 128;
	int blocks_per_sm = 64;   /* capped by occupancy */
	int chunk = 1;
	/* minimizer: warps per pose (1 = one warp per pose, 2..7 = the team
	 * kernel), 0 = chosen from the job size; a tuned team applies to jobs of
	 * at most team_poses poses (the size it was timed on), larger ones
	 * choose their own */
	int team = 0;
	size_t team_poses = 0;
};

/* Ids of one receptor-ligand pair's data: (receptor, ligand, grid, parameter table). */
using PairKey = std::array<gba_id, 4>;

/* Signature of a captured minimizer pipeline. */
struct GraphKey {
	int kind;
	uintptr_t a, b, c, d, e, f, g;
	size_t n;
	int p0, p1, p2, p3;
	unsigned long long deadline;
	bool operator<(const GraphKey& o) const {
		return std::memcmp(this, &o, sizeof(GraphKey)) < 0;
	}
};

struct Context {
	Context() = default;
	~Context();
	int device = 0;
	int num_sms = 0;
	cudaMemPool_t scratch_pool = nullptr;   /* per-call scratch (StreamScratch); may stay null */
	CheckedMutex mu;               /* items map */
	CheckedMutex stage_mu;         /* host-pointer staging buffers */
	std::unordered_map<gba_id, std::unique_ptr<Item>> items;
	gba_id next_id = 1;
	DevBuffer stage[6];

	mutable std::mutex err_mu;
	std::string err;

	void bind() { check_cuda(cudaSetDevice(device), "cudaSetDevice"); }
	void set_error(const std::string& m) { std::lock_guard<std::mutex> g(err_mu); err = m; }
	const char* last_error() const { std::lock_guard<std::mutex> g(err_mu); return err.c_str(); }

	Item* find(gba_id id, ItemKind kind);
	/* registers an item; a grid or parameter table also gets the pair-term
	 * tables it forms with the items already present (one per parameter
	 * table and distinct plateau), so that no scoring call has to build one */
	gba_id add(std::unique_ptr<Item> item);
	std::set<uint32_t> plateau_keys;   /* plateau^2 bit patterns of every grid added */
	void* staging(int slot, size_t bytes);
	void* pinned(int slot, size_t bytes);

	/* minimizer / batch state */
	std::map<std::vector<gba_id>, std::unique_ptr<DevBuffer>> model_cache;
	DevBuffer pair_buf, aux;
	int32_t* pinned_status = nullptr;
	void* pinned_buf[2] = {nullptr, nullptr};
	size_t pinned_bytes[2] = {0, 0};
	std::map<GraphKey, cudaGraphExec_t> graphs;
	cudaStream_t capture_stream = nullptr;
	uint32_t deadline_ms = 0;
	mutable std::mutex tune_mu;    /* guards tune and pair_tune (gba_autotune writes them while calls read them) */
	std::map<std::string, TuneParams> tune;
	/* per pair: the shapes gba_autotune chose for it ("energy", "minimize") */
	std::map<std::pair<std::string, PairKey>, TuneParams> pair_tune;
	void set_tuned(const std::string& key, const TuneParams& p);
	void set_pair_tuned(const std::string& kind, const PairKey& key, const TuneParams& p);
	/* the pair's tuned shape, else the context-wide one */
	TuneParams pair_tuned(const std::string& kind, const PairKey& key) const;

	/* device address of the static scratch of gba_energy_6d_noalloc,
	 * resolved by the first such call on this context */
	void* noalloc_scratch = nullptr;

	/* spatial visiting order of large batches (pose_order.cu) */
	static constexpr size_t kOrderMinPoses = 4096;
	bool order_enabled = true;
	const uint32_t* pose_order(const void* dofs, size_t stride_floats, size_t n, const DevIntrpl& box,
			cudaStream_t s, StreamScratch& scratch);
	DevBuffer order_buf;      /* visiting-order keys, indices and sort scratch */
	DevBuffer rank_buf;       /* per pair of a batch: its place in the visiting order */
	/* pair_rank (optional, device): the rank of each pair's poses in the
	 * visiting order, else the pair index */
	const uint32_t* pose_order_persistent(const void* dofs, size_t stride_floats, size_t n,
			const DevIntrpl& box, const RigidModel* models, const uint32_t* pair_of, const uint32_t* pair_rank,
			size_t npairs, cudaStream_t s);
	TuneParams tuned(const std::string& kind, size_t n) const;
	/* lig_rounds: the largest ligand of the launch in 64-bead rounds (caps
	 * the team size) */
	void run_minimize(MinLaunch& L, cudaStream_t s, int32_t* status_out, uint32_t lig_rounds,
			const TuneParams& tp);
	/* One launch per group of pairs, each with its own shape, concurrently
	 * in one captured graph: group g takes the queue slots
	 * [off[g], off[g] + n[g]) of L.order. */
	struct MinGroup {
		size_t off, n;
		TuneParams tp;
	};
	void run_minimize_groups(MinLaunch& L, const std::vector<MinGroup>& groups, cudaStream_t s,
			int32_t* status_out);
	static constexpr size_t kMaxGroups = 16;
	std::vector<cudaStream_t> group_streams;
	std::vector<cudaEvent_t> group_events;
	DevBuffer group_aux;          /* per group: cursor, status; then the earliest warp start */
	int32_t* pinned_group_status = nullptr;
	/* warps per pose the minimizer uses for n poses */
	int minimize_team(const TuneParams& tp, size_t n, uint32_t lig_rounds) const;
	int team_override = 0;         /* gba_set_minimize_team; 0 = tuned or automatic */
	void clear_graphs();

	/* may_allocate = false: the typed list is used only if it already exists
	 * (gba_energy_6d_noalloc) */
	RigidLaunch rigid_launch(gba_id rec, gba_id lig, gba_id grid, gba_id params, bool may_allocate = true);
	/* the grid's typed list for receptor `rec_id` (built on first use), or
	 * nullptr when the receptor's types or indices do not fit */
	const uint32_t* typed_list(GridItem& g, gba_id rec_id, const ProteinItem& rec, bool may_allocate);
	void validate_pair(const ProteinItem& rec, const ProteinItem& lig, const GridItem& g,
			const ParamsItem& p);
	/* tp: launch shape (nullptr: the context-wide "energy" shape) */
	void run_rigid(RigidLaunch& L, cudaStream_t s, const TuneParams* tp = nullptr);
	ModesLaunch modes_launch(gba_id rec, gba_id lig, gba_id grid_rec, gba_id grid_lig, gba_id params);
	void run_modes(ModesLaunch& L, cudaStream_t s);

	/* the host C library's sin/cos table (gba_set_host_sincos); trig.sc ==
	 * nullptr: off */
	DevBuffer trig_table;
	DevTrig trig{nullptr, 0u, 0u};

	/* GBA_KOPT_* flags (gba_set_kernel_options) and their effect on a grid */
	uint32_t kernel_opts = GBA_KOPT_DEFAULT;
	DevGrid apply_kernel_options(DevGrid g) const;

	/* CUDA-event timing of the fused rigid energy kernel (gba_kernel_timing) */
	static constexpr size_t kTimingPool = 1024;
	bool timing = false;
	std::vector<std::pair<cudaEvent_t, cudaEvent_t>> timing_events;
	size_t timing_used = 0;
	double timing_ms = 0.0;
	uint64_t timing_launches = 0;
	void timing_fold();
};

}  // namespace gba

struct gba_ctx : gba::Context {};

#endif
