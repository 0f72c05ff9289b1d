/*
 * gba_api.cu -- the C ABI of libgbattract (declared in include/gbattract.h).
 *
 * Owns the device copies of proteins, grids and parameter tables (the role of
 * the reference's DataManager/DeviceManager, src/server/DataManager.cpp:23-101,
 * src/server/DeviceManager.cpp:29-59) and dispatches the fused kernels.  No
 * entry point throws or exits: failures come back as a status code with the
 * message in gba_last_error().
 */
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "gba_context.h"

using namespace gba;

namespace {
thread_local std::string t_create_error;
std::atomic<uint64_t> g_allocations{0};
}

/* ------------------------------------------------------------------------ */
/* context helpers                                                          */
/* ------------------------------------------------------------------------ */

namespace gba {

void note_allocation() { g_allocations.fetch_add(1, std::memory_order_relaxed); }

void DevBuffer::alloc(size_t b) {
	release();
	if (b == 0) return;
	note_allocation();
	cudaError_t e = cudaMalloc(&ptr, b);
	if (e != cudaSuccess) {
		ptr = nullptr;
		throw ApiError(e == cudaErrorMemoryAllocation ? GBA_ERR_OUT_OF_MEMORY : GBA_ERR_CUDA,
				std::string("cudaMalloc(") + std::to_string(b) + "): " + cudaGetErrorString(e));
	}
	bytes = b;
}

void DevBuffer::release() {
	if (ptr) cudaFree(ptr);
	ptr = nullptr;
	bytes = 0;
}

void DevBuffer::upload(const void* src, size_t b) {
	alloc(b);
	if (b) check_cuda(cudaMemcpy(ptr, src, b, cudaMemcpyHostToDevice), "upload");
}

void check_cuda(cudaError_t e, const char* what) {
	if (e != cudaSuccess)
		throw ApiError(e == cudaErrorMemoryAllocation ? GBA_ERR_OUT_OF_MEMORY : GBA_ERR_CUDA,
				std::string(what) + ": " + cudaGetErrorString(e));
}

bool is_device_pointer(const void* p) {
	cudaPointerAttributes a;
	cudaError_t e = cudaPointerGetAttributes(&a, p);
	if (e != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

Item* Context::find(gba_id id, ItemKind kind) {
	auto it = items.find(id);
	if (it == items.end() || it->second->kind != kind)
		throw ApiError(GBA_ERR_UNKNOWN_ID, "unknown " + std::string(kind_name(kind)) + " id " +
				std::to_string(id));
	return it->second.get();
}

gba_id Context::add(std::unique_ptr<Item> item) {
	Lock g(mu);
	if (item->kind == ItemKind::Grid) {
		const float p2 = static_cast<GridItem*>(item.get())->dev.nl.dPlateau2;
		uint32_t key;
		std::memcpy(&key, &p2, 4);
		if (!plateau_keys.count(key)) {
			for (auto& kv : items)
				if (kv.second->kind == ItemKind::Params)
					static_cast<ParamsItem*>(kv.second.get())->pair_table(p2);
			plateau_keys.insert(key);
		}
	} else if (item->kind == ItemKind::Params) {
		for (uint32_t key : plateau_keys) {
			float p2;
			std::memcpy(&p2, &key, 4);
			static_cast<ParamsItem*>(item.get())->pair_table(p2);
		}
	}
	gba_id id = next_id++;
	items.emplace(id, std::move(item));
	return id;
}

void* Context::staging(int slot, size_t bytes) {
	DevBuffer& b = stage[slot];
	if (b.bytes < bytes) b.alloc(bytes + bytes / 4);
	return b.ptr;
}

void* Context::pinned(int slot, size_t bytes) {
	if (pinned_bytes[slot] < bytes) {
		if (pinned_buf[slot]) cudaFreeHost(pinned_buf[slot]);
		pinned_buf[slot] = nullptr;
		pinned_bytes[slot] = 0;
		note_allocation();
		check_cuda(cudaMallocHost(&pinned_buf[slot], bytes + bytes / 4), "cudaMallocHost");
		pinned_bytes[slot] = bytes + bytes / 4;
	}
	return pinned_buf[slot];
}

void Context::set_tuned(const std::string& key, const TuneParams& p) {
	std::lock_guard<std::mutex> g(tune_mu);
	tune[key] = p;
}

void Context::set_pair_tuned(const std::string& kind, const PairKey& key, const TuneParams& p) {
	std::lock_guard<std::mutex> g(tune_mu);
	pair_tune[{kind, key}] = p;
}

TuneParams Context::pair_tuned(const std::string& kind, const PairKey& key) const {
	{
		std::lock_guard<std::mutex> g(tune_mu);
		auto it = pair_tune.find({kind, key});
		if (it != pair_tune.end()) return it->second;
	}
	return tuned(kind, 0);
}

TuneParams Context::tuned(const std::string& kind, size_t) const {
	std::lock_guard<std::mutex> g(tune_mu);
	auto it = tune.find(kind);
	if (it != tune.end()) return it->second;
	/* defaults until gba_autotune has run: full occupancy */
	return kind == "energy" ? TuneParams{256, 64, 1} : TuneParams{128, 64, 1};
}

Context::~Context() {
	clear_graphs();
	for (auto& e : timing_events) {
		cudaEventDestroy(e.first);
		cudaEventDestroy(e.second);
	}
	if (capture_stream) cudaStreamDestroy(capture_stream);
	for (cudaStream_t st : group_streams) cudaStreamDestroy(st);
	for (cudaEvent_t ev : group_events) cudaEventDestroy(ev);
	if (pinned_status) cudaFreeHost(pinned_status);
	if (pinned_group_status) cudaFreeHost(pinned_group_status);
	for (void* p : pinned_buf)
		if (p) cudaFreeHost(p);
	/* frees still in flight complete before the pool's memory is released */
	if (scratch_pool) cudaMemPoolDestroy(scratch_pool);
}

const char* kind_name(ItemKind k) {
	switch (k) {
	case ItemKind::Protein: return "protein";
	case ItemKind::Grid: return "grid";
	case ItemKind::Params: return "parameter table";
	}
	return "item";
}

/* Derived members exactly as IntrplGrid's constructor
 * (src/model/IntrplGrid.tpp:29-41); host code is built unfused. */
DevIntrpl intrpl_from_desc(const gba_intrpl_desc& d) {
	DevIntrpl g{};
	for (int a = 0; a < 3; ++a) { g.dimN[a] = d.dimN[a]; g.pos[a] = d.posMin[a]; }
	g.numGrids = d.numGrids;
	g.dVox = d.gridSpacing;
	const float vol = g.dVox * g.dVox * g.dVox;
	g.voxelVol_inv = 1.f / vol;
	g.dVox_inv = 1.f / g.dVox;
	for (int a = 0; a < 3; ++a) g.maxDim[a] = g.pos[a] + (float)(g.dimN[a] - 1) * g.dVox;
	return g;
}

/* NLGrid's constructor, src/model/NLGrid.tpp:29-41 */
DevNL nl_from_desc(const gba_nl_desc& d) {
	DevNL g{};
	for (int a = 0; a < 3; ++a) { g.dimN[a] = d.dimN[a]; g.pos[a] = d.posMin[a]; }
	const float dVox = d.gridSpacing;
	g.dPlateau2 = d.dPlateau * d.dPlateau;
	g.dPlateau2_inv = 1 / g.dPlateau2;
	g.dVox_inv = 1 / dVox;
	for (int a = 0; a < 3; ++a) g.maxDim[a] = g.pos[a] + (float)(g.dimN[a] - 1) * dVox;
	g.ratio_size = (uint32_t)int(10000 * g.dPlateau2) + 1;
	g.ratio_scale = (float)(1.0 / 10000.0 / (double)g.dPlateau2);
	g.approx_inv = g.dPlateau2 < 2500.0f ? 1 : 0;
	return g;
}

/* The sqrt-ratio table of src/model/NLGrid.tpp:45-50, bit-identical. */
std::vector<float> nl_ratio_table(float dPlateau2) {
	const int size = int(10000 * dPlateau2);
	std::vector<float> r(size + 1);
	for (int n = 0; n <= size; n++) {
		double d2 = ((n + 0.5) / 10000);
		r[n] = (float)std::sqrt(d2 / (double)dPlateau2);
	}
	return r;
}

}  // namespace gba

#define GBA_API_BEGIN try {
#define GBA_API_END(ctx)                                                   \
	}                                                                      \
	catch (const ApiError& e) {                                            \
		(ctx)->set_error(e.what());                                        \
		return e.code;                                                     \
	}                                                                      \
	catch (const std::bad_alloc&) {                                        \
		(ctx)->set_error("host allocation failed");                        \
		return GBA_ERR_OUT_OF_MEMORY;                                      \
	}                                                                      \
	catch (const std::exception& e) {                                      \
		(ctx)->set_error(e.what());                                        \
		return GBA_ERR_INVALID_ARGUMENT;                                   \
	}                                                                      \
	return GBA_OK;

extern "C" {

const char* gba_version(void) { return "gbattract 0.1 (sm_103a)"; }

int gba_allocation_count(uint64_t* out) {
	if (!out) return GBA_ERR_INVALID_ARGUMENT;
	*out = g_allocations.load(std::memory_order_relaxed);
	return GBA_OK;
}

int gba_create(int device, gba_ctx** out) {
	if (!out) {
		t_create_error = "gba_create: out is NULL";
		return GBA_ERR_INVALID_ARGUMENT;
	}
	*out = nullptr;
	int n = 0;
	cudaError_t e = cudaGetDeviceCount(&n);
	if (e != cudaSuccess || n == 0) {
		cudaGetLastError();
		t_create_error = std::string("gba_create: no CUDA device (") + cudaGetErrorString(e) + ")";
		return GBA_ERR_NO_DEVICE;
	}
	if (device < 0 || device >= n) {
		t_create_error = "gba_create: device " + std::to_string(device) + " out of range [0," +
				std::to_string(n) + ")";
		return GBA_ERR_INVALID_ARGUMENT;
	}
	e = cudaSetDevice(device);
	if (e == cudaSuccess) e = cudaFree(nullptr);
	if (e != cudaSuccess) {
		t_create_error = std::string("gba_create: ") + cudaGetErrorString(e);
		return GBA_ERR_CUDA;
	}
	auto* c = new (std::nothrow) gba_ctx();
	if (!c) {
		t_create_error = "gba_create: host allocation failed";
		return GBA_ERR_OUT_OF_MEMORY;
	}
	c->device = device;
	cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
	/* a private stream-ordered pool for per-call scratch that keeps its
	 * memory reserved (without it the calls fall back to the default pool) */
	cudaMemPoolProps props{};
	props.allocType = cudaMemAllocationTypePinned;
	props.location.type = cudaMemLocationTypeDevice;
	props.location.id = device;
	if (cudaMemPoolCreate(&c->scratch_pool, &props) == cudaSuccess) {
		uint64_t keep = UINT64_MAX;
		if (cudaMemPoolSetAttribute(c->scratch_pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
			cudaMemPoolDestroy(c->scratch_pool);
			c->scratch_pool = nullptr;
		}
	} else {
		c->scratch_pool = nullptr;
	}
	cudaGetLastError();
	*out = c;
	return GBA_OK;
}

int gba_destroy(gba_ctx* ctx) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	cudaSetDevice(ctx->device);
	delete ctx;
	return GBA_OK;
}

const char* gba_last_error(const gba_ctx* ctx) {
	if (!ctx) return t_create_error.c_str();
	return ctx->last_error();
}

int gba_upload_protein(gba_ctx* ctx, uint32_t n, const float* xyz, const uint32_t* type,
		const uint32_t* mapped, const float* charge, uint32_t n_modes, const float* modes,
		const float* mode_force, gba_id* out) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_API_BEGIN
	if (!out || n == 0 || !xyz || !type || !mapped || !charge)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_upload_protein: null pointer or n == 0");
	if (n_modes > GBA_MODES_MAX)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_upload_protein: n_modes > GBA_MODES_MAX");
	if (n_modes > 0 && (!modes || !mode_force))
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_upload_protein: modes/mode_force NULL");
	ctx->bind();
	auto item = std::make_unique<ProteinItem>();
	std::vector<float4> xq(n);
	std::vector<uint32_t> tm(n);
	uint32_t max_type = 0, max_mapped = 0;
	for (uint32_t i = 0; i < n; ++i) {
		xq[i] = make_float4(xyz[i], xyz[n + i], xyz[2 * (size_t)n + i], charge[i]);
		if (type[i] > 0xffffu || mapped[i] > 0xffffu)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_upload_protein: type/mapped type > 65535");
		tm[i] = type[i] | (mapped[i] << 16);
		max_type = std::max(max_type, type[i]);
		max_mapped = std::max(max_mapped, mapped[i]);
	}
	item->xyzq.upload(xq.data(), xq.size() * sizeof(float4));
	item->tm.upload(tm.data(), tm.size() * sizeof(uint32_t));
	item->max_type = max_type;
	item->max_mapped = max_mapped;
	item->host_xyz.assign(xyz, xyz + 3 * (size_t)n);
	item->dev.n = n;
	item->dev.n_modes = n_modes;
	item->dev.xyzq = (const float4*)item->xyzq.ptr;
	item->dev.tm = (const uint32_t*)item->tm.ptr;
	if (n_modes > 0) {
		/* reference layout x[i*M+m] | y | z  ->  device [i][m][axis], each
		 * bead's record padded to mode_stride floats */
		const size_t ms = mode_stride(n_modes);
		std::vector<float> md(ms * n, 0.0f);
		for (uint32_t a = 0; a < 3; ++a)
			for (uint32_t i = 0; i < n; ++i)
				for (uint32_t m = 0; m < n_modes; ++m)
					md[(size_t)i * ms + (size_t)m * 3 + a] = modes[(size_t)a * n * n_modes + (size_t)i * n_modes + m];
		item->modes.upload(md.data(), md.size() * sizeof(float));
		item->dev.modes = (const float*)item->modes.ptr;
		for (uint32_t m = 0; m < n_modes; ++m) item->dev.mode_force[m] = mode_force[m];
	}
	*out = ctx->add(std::move(item));
	GBA_API_END(ctx)
}

int gba_upload_grid(gba_ctx* ctx, const gba_intrpl_desc* inner, const float* inner_data,
		const gba_intrpl_desc* outer, const float* outer_data, const gba_nl_desc* nl,
		const gba_neighbour_desc* nl_grid, const uint32_t* nl_list, gba_id* out) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_API_BEGIN
	if (!out || !inner || !inner_data || !outer || !outer_data || !nl || !nl_grid ||
			(nl->numEl > 0 && !nl_list))
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_upload_grid: null pointer");
	for (const gba_intrpl_desc* d : {inner, outer}) {
		if (d->numGrids < 1 || d->dimN[0] < 2 || d->dimN[1] < 2 || d->dimN[2] < 2 ||
				!(d->gridSpacing > 0))
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_upload_grid: bad interpolation grid descriptor");
		if ((double)d->numGrids * d->dimN[0] * d->dimN[1] * d->dimN[2] > 4.0e9)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_upload_grid: grid exceeds 2^32 float4");
	}
	if (nl->dimN[0] < 1 || nl->dimN[1] < 1 || nl->dimN[2] < 1 || !(nl->gridSpacing > 0) ||
			!(nl->dPlateau > 0))
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_upload_grid: bad neighbour grid descriptor");
	ctx->bind();
	auto item = std::make_unique<GridItem>();
	item->inner_desc = *inner;
	item->outer_desc = *outer;
	item->nl_desc = *nl;
	const size_t ni = (size_t)inner->numGrids * inner->dimN[0] * inner->dimN[1] * inner->dimN[2];
	const size_t no = (size_t)outer->numGrids * outer->dimN[0] * outer->dimN[1] * outer->dimN[2];
	const size_t nv = (size_t)nl->dimN[0] * nl->dimN[1] * nl->dimN[2];
	for (size_t v = 0; v < nv; ++v)
		if ((uint64_t)nl_grid[v].idx + nl_grid[v].numEl > nl->numEl && nl_grid[v].numEl > 0)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_upload_grid: neighbour descriptor past the list end");
	item->inner.upload(inner_data, ni * sizeof(float4));
	item->outer.upload(outer_data, no * sizeof(float4));
	item->nlgrid.upload(nl_grid, nv * sizeof(uint2));
	item->nllist.upload(nl_list, (size_t)nl->numEl * sizeof(uint32_t));
	item->dev.inner = intrpl_from_desc(*inner);
	item->dev.inner.data = (const float4*)item->inner.ptr;
	item->dev.outer = intrpl_from_desc(*outer);
	item->dev.outer.data = (const float4*)item->outer.ptr;
	item->dev.nl = nl_from_desc(*nl);
	std::vector<float> ratio = nl_ratio_table(item->dev.nl.dPlateau2);
	item->ratio.upload(ratio.data(), ratio.size() * sizeof(float));
	item->dev.nl.grid = (const uint2*)item->nlgrid.ptr;
	item->dev.nl.list = (const uint32_t*)item->nllist.ptr;
	item->dev.nl.ratio = (const float*)item->ratio.ptr;
	/* every receptor index in the list is checked against the receptor at call time */
	uint32_t max_idx = 0;
	for (uint32_t k = 0; k < nl->numEl; ++k) max_idx = std::max(max_idx, nl_list[k]);
	item->nl_max_index = nl->numEl ? max_idx : 0;
	item->nl_has_entries = nl->numEl > 0;
	item->nl_list_radius = (double)nl->dPlateau + 0.5 * std::sqrt(3.0) * (double)nl->gridSpacing;
	*out = ctx->add(std::move(item));
	GBA_API_END(ctx)
}

int gba_upload_params(gba_ctx* ctx, uint32_t num_types, const gba_ffparam* table, int potshape,
		int dielec, float ffelec, gba_id* out) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_API_BEGIN
	if (!out || !table || num_types == 0)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_upload_params: null table or num_types == 0");
	if (potshape != GBA_POTSHAPE_8_6 && potshape != GBA_POTSHAPE_12_6)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_upload_params: unknown potential shape");
	if (dielec != GBA_DIELEC_CONSTANT && dielec != GBA_DIELEC_VARIABLE)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_upload_params: unknown dielectric");
	ctx->bind();
	auto item = std::make_unique<ParamsItem>();
	const size_t T2 = (size_t)num_types * num_types;
	std::vector<float4> lj(T2);
	std::vector<float> iv(T2);
	for (size_t k = 0; k < T2; ++k) {
		lj[k] = make_float4(table[k].rc, table[k].ac, table[k].rmin2, table[k].emin);
		iv[k] = (float)table[k].ipon;
	}
	item->lj.upload(lj.data(), T2 * sizeof(float4));
	item->ivor.upload(iv.data(), T2 * sizeof(float));
	item->host_table.assign(table, table + T2);
	item->dev.num_types = num_types;
	item->dev.potshape = potshape;
	item->dev.dielec = dielec;
	item->dev.ffelec = ffelec;
	item->dev.lj = (const float4*)item->lj.ptr;
	item->dev.ivor = (const float*)item->ivor.ptr;
	*out = ctx->add(std::move(item));
	GBA_API_END(ctx)
}

/* The pair-term table for a grid of plateau^2 dPlateau2: per type pair the
 * parameters and LJPotForce (src/model/forcefield.h:30-83) evaluated at the
 * plateau distance -- the force factor and energy the NL term subtracts
 * (src/model/neighborlist.h:122-130) -- in the rounding of the device's
 * lj_pot_force (unfused FP32, one fused multiply-add), so folding them in
 * changes no bit of the result.  Stored transposed against the host table
 * (which is indexed receptor type major): the pairs of one ligand bead then
 * read one contiguous row. */
const float4* ParamsItem::pair_table(float dPlateau2, bool may_allocate) {
	uint32_t key;
	std::memcpy(&key, &dPlateau2, 4);
	auto it = pair_tables.find(key);
	if (it != pair_tables.end()) return (const float4*)it->second->ptr;
	if (!may_allocate)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "no pair-term table for this grid's plateau and parameter table");
	const size_t T2 = host_table.size();
	std::vector<float4> t(2 * T2);
	const float p2inv = 1.0f / dPlateau2;
	const bool shape86 = dev.potshape == GBA_POTSHAPE_8_6;
	for (size_t k = 0; k < T2; ++k) {
		const gba_ffparam& p = host_table[k];
		const float ivor = (float)p.ipon;
		const float rr23 = (p2inv * p2inv) * p2inv;
		const float rrd = shape86 ? p2inv : rr23;
		const float sd = shape86 ? 2.0f : 6.0f;
		const float rep = p.rc * rrd;
		const float vlj = (rep - p.ac) * rr23;
		float fb = std::fmaf(6.0f, vlj, sd * (rep * rr23));
		float e;
		if (dPlateau2 < p.rmin2) {
			e = std::fmaf(ivor - 1.0f, p.emin, vlj);
		} else {
			e = ivor * vlj;
			fb = ivor * fb;
		}
		const size_t nt = (size_t)dev.num_types;
		const size_t kt = (k % nt) * nt + k / nt;
		t[2 * kt] = make_float4(p.rc, p.ac, p.rmin2, p.emin);
		t[2 * kt + 1] = make_float4(ivor, fb, e, 0.0f);
	}
	auto buf = std::make_unique<DevBuffer>();
	buf->upload(t.data(), t.size() * sizeof(float4));
	const float4* ptr = (const float4*)buf->ptr;
	pair_tables.emplace(key, std::move(buf));
	return ptr;
}

/* Adds the elapsed time of every recorded event pair to the running total. */
void Context::timing_fold() {
	for (size_t k = 0; k < timing_used; ++k) {
		check_cuda(cudaEventSynchronize(timing_events[k].second), "kernel timing: event sync");
		float ms = 0.f;
		check_cuda(cudaEventElapsedTime(&ms, timing_events[k].first, timing_events[k].second),
				"kernel timing: elapsed");
		timing_ms += ms;
		++timing_launches;
	}
	timing_used = 0;
}

int gba_kernel_timing(gba_ctx* ctx, int32_t enable) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_API_BEGIN
	ctx->bind();
	ctx->timing = enable != 0;
	GBA_API_END(ctx)
}

int gba_kernel_time(gba_ctx* ctx, double* ms_total, uint64_t* launches, int32_t reset) {
	if (!ctx || !ms_total || !launches) return GBA_ERR_INVALID_ARGUMENT;
	GBA_API_BEGIN
	ctx->bind();
	ctx->timing_fold();
	*ms_total = ctx->timing_ms;
	*launches = ctx->timing_launches;
	if (reset) {
		ctx->timing_ms = 0.0;
		ctx->timing_launches = 0;
	}
	GBA_API_END(ctx)
}

int gba_set_kernel_options(gba_ctx* ctx, uint32_t flags) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_API_BEGIN
	if (flags & ~(uint32_t)(GBA_KOPT_RATIO_COMPUTED | GBA_KOPT_COOP_LOOKUP | GBA_KOPT_FOUR_BLOCKS |
			GBA_KOPT_TYPED_LIST | GBA_KOPT_REFERENCE_ORDER))
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_set_kernel_options: unknown flag");
	ctx->bind();
	Lock g(ctx->stage_mu);
	ctx->kernel_opts = flags;
	/* cached device models and minimizer graphs hold the old options */
	ctx->model_cache.clear();
	ctx->clear_graphs();
	GBA_API_END(ctx)
}

int gba_set_pose_order(gba_ctx* ctx, int enable) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	ctx->order_enabled = enable != 0;
	return GBA_OK;
}

int gba_release(gba_ctx* ctx, gba_id id) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_API_BEGIN
	ctx->bind();
	Lock g(ctx->mu);
	auto it = ctx->items.find(id);
	if (it == ctx->items.end())
		throw ApiError(GBA_ERR_UNKNOWN_ID, "gba_release: unknown id " + std::to_string(id));
	if (it->second->kind == ItemKind::Protein)
		for (auto& kv : ctx->items)
			if (kv.second->kind == ItemKind::Grid)
				static_cast<GridItem*>(kv.second.get())->typed_lists.erase(id);
	ctx->items.erase(it);
	ctx->model_cache.clear();
	ctx->clear_graphs();
	GBA_API_END(ctx)
}

int gba_energy_6d(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_dof6d* dofs, size_t n, gba_result6d* out, void* stream) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_API_BEGIN
	if (n == 0) return GBA_OK;
	if (!dofs || !out) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_energy_6d: null dofs/out");
	ctx->bind();
	RigidLaunch L = ctx->rigid_launch(rec, lig, grid, params);
	cudaStream_t s = (cudaStream_t)stream;
	const bool din = is_device_pointer(dofs), dout = is_device_pointer(out);
	std::unique_lock<CheckedMutex> stage_lock(ctx->stage_mu, std::defer_lock);
	if (!din || !dout) stage_lock.lock();
	L.n = n;
	L.dofs = din ? dofs : (const gba_dof6d*)ctx->staging(0, n * sizeof(gba_dof6d));
	L.out = dout ? out : (gba_result6d*)ctx->staging(1, n * sizeof(gba_result6d));
	L.census = nullptr;
	if (!din)
		check_cuda(cudaMemcpyAsync((void*)L.dofs, dofs, n * sizeof(gba_dof6d), cudaMemcpyHostToDevice, s),
				"gba_energy_6d: H2D");
	const TuneParams shape = ctx->pair_tuned("energy", PairKey{rec, lig, grid, params});
	ctx->run_rigid(L, s, &shape);
	if (!dout)
		check_cuda(cudaMemcpyAsync(out, L.out, n * sizeof(gba_result6d), cudaMemcpyDeviceToHost, s),
				"gba_energy_6d: D2H");
	if (!din || !dout) check_cuda(cudaStreamSynchronize(s), "gba_energy_6d: sync");
	GBA_API_END(ctx)
}

int gba_energy_6d_modes(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid_rec, gba_id grid_lig,
		gba_id params, const gba_dof6d_modes* dofs, size_t n, gba_result6d_modes* out,
		void* stream) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_API_BEGIN
	if (n == 0) return GBA_OK;
	if (!dofs || !out) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_energy_6d_modes: null dofs/out");
	ctx->bind();
	ModesLaunch L = ctx->modes_launch(rec, lig, grid_rec, grid_lig, params);
	cudaStream_t s = (cudaStream_t)stream;
	const bool din = is_device_pointer(dofs), dout = is_device_pointer(out);
	std::unique_lock<CheckedMutex> stage_lock(ctx->stage_mu, std::defer_lock);
	if (!din || !dout) stage_lock.lock();
	L.n = n;
	L.dofs = din ? dofs : (const gba_dof6d_modes*)ctx->staging(0, n * sizeof(gba_dof6d_modes));
	L.out = dout ? out : (gba_result6d_modes*)ctx->staging(1, n * sizeof(gba_result6d_modes));
	if (!din)
		check_cuda(cudaMemcpyAsync((void*)L.dofs, dofs, n * sizeof(gba_dof6d_modes),
				cudaMemcpyHostToDevice, s), "gba_energy_6d_modes: H2D");
	ctx->run_modes(L, s);
	if (!dout)
		check_cuda(cudaMemcpyAsync(out, L.out, n * sizeof(gba_result6d_modes), cudaMemcpyDeviceToHost, s),
				"gba_energy_6d_modes: D2H");
	if (!din || !dout) check_cuda(cudaStreamSynchronize(s), "gba_energy_6d_modes: sync");
	GBA_API_END(ctx)
}

int gba_census_6d(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_dof6d* dofs, size_t n, gba_result6d* out, uint32_t* census) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	GBA_API_BEGIN
	if (n == 0) return GBA_OK;
	if (!dofs || !out || !census) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_census_6d: null pointer");
	ctx->bind();
	RigidLaunch L = ctx->rigid_launch(rec, lig, grid, params);
	Lock stage_lock(ctx->stage_mu);
	const bool din = is_device_pointer(dofs), dout = is_device_pointer(out), dc = is_device_pointer(census);
	L.n = n;
	L.dofs = din ? dofs : (const gba_dof6d*)ctx->staging(0, n * sizeof(gba_dof6d));
	L.out = dout ? out : (gba_result6d*)ctx->staging(1, n * sizeof(gba_result6d));
	L.census = dc ? (PoseCensus*)census : (PoseCensus*)ctx->staging(2, n * sizeof(PoseCensus));
	if (!din)
		check_cuda(cudaMemcpy((void*)L.dofs, dofs, n * sizeof(gba_dof6d), cudaMemcpyHostToDevice), "H2D");
	ctx->run_rigid(L, 0);
	if (!dout) check_cuda(cudaMemcpy(out, L.out, n * sizeof(gba_result6d), cudaMemcpyDeviceToHost), "D2H");
	if (!dc) check_cuda(cudaMemcpy(census, L.census, n * sizeof(PoseCensus), cudaMemcpyDeviceToHost), "D2H");
	check_cuda(cudaDeviceSynchronize(), "gba_census_6d");
	GBA_API_END(ctx)
}

}  // extern "C"

/* ------------------------------------------------------------------------ */
/* launch assembly                                                          */
/* ------------------------------------------------------------------------ */

namespace gba {

RigidLaunch Context::rigid_launch(gba_id rec, gba_id lig, gba_id grid, gba_id params, bool may_allocate) {
	Lock g(mu);
	auto* R = static_cast<ProteinItem*>(find(rec, ItemKind::Protein));
	auto* Lg = static_cast<ProteinItem*>(find(lig, ItemKind::Protein));
	auto* G = static_cast<GridItem*>(find(grid, ItemKind::Grid));
	auto* P = static_cast<ParamsItem*>(find(params, ItemKind::Params));
	validate_pair(*R, *Lg, *G, *P);
	RigidLaunch L{};
	L.m.rec = R->dev;
	L.m.lig = Lg->dev;
	L.m.grid = apply_kernel_options(G->dev);
	L.m.par = P->dev;
	L.m.par.pair = P->pair_table(G->dev.nl.dPlateau2, may_allocate);
	L.m.trig = trig;
	L.bound4 = (kernel_opts & GBA_KOPT_FOUR_BLOCKS) ? 1 : 0;
	L.ref_order = (kernel_opts & GBA_KOPT_REFERENCE_ORDER) ? 1 : 0;
	if (kernel_opts & GBA_KOPT_TYPED_LIST)
		L.m.grid.nl.typed_list = typed_list(*G, rec, *R, may_allocate);
	return L;
}

namespace {

/* out[k] = list[k] | type(list[k]) << 24 */
__global__ void typed_list_kernel(const uint32_t* __restrict__ list, size_t n, const uint32_t* __restrict__ tm,
		uint32_t* __restrict__ out) {
	for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
		const uint32_t j = list[k];
		out[k] = j | (tm[j] & 0xffu) << 24;
	}
}

}  // namespace

const uint32_t* Context::typed_list(GridItem& G, gba_id rec_id, const ProteinItem& R, bool may_allocate) {
	const size_t n = G.nl_desc.numEl;
	if (n == 0 || R.max_type > 255 || R.dev.n > (1u << 24)) return nullptr;
	auto it = G.typed_lists.find(rec_id);
	if (it != G.typed_lists.end()) return (const uint32_t*)it->second.ptr;
	if (!may_allocate) return nullptr;
	it = G.typed_lists.try_emplace(rec_id).first;
	try {
		it->second.alloc(n * sizeof(uint32_t));
		/* list indices were checked against the receptor size (validate_pair) */
		const int threads = 256;
		const size_t blocks = std::min<size_t>((n + threads - 1) / threads, (size_t)num_sms * 32);
		typed_list_kernel<<<(unsigned)blocks, threads>>>(G.dev.nl.list, n, R.dev.tm, (uint32_t*)it->second.ptr);
		check_cuda(cudaGetLastError(), "typed list launch");
		check_cuda(cudaDeviceSynchronize(), "typed list");
	} catch (...) {
		G.typed_lists.erase(it);
		throw;
	}
	return (const uint32_t*)it->second.ptr;
}

DevGrid Context::apply_kernel_options(DevGrid g) const {
	g.nl.ratio_computed = (kernel_opts & GBA_KOPT_RATIO_COMPUTED) ? 1 : 0;
	g.coop_lookup = ((kernel_opts & GBA_KOPT_COOP_LOOKUP) && g.inner.oct && g.outer.oct) ? 1 : 0;
	return g;
}

/* The index checks that keep every device access in bounds (the reference
 * asserts them in debug builds only: src/model/neighborlist.h:94-97,
 * src/model/IntrplGrid.h:132-146). */
void Context::validate_pair(const ProteinItem& rec, const ProteinItem& lig, const GridItem& g,
		const ParamsItem& p) {
	if (lig.max_type > p.dev.num_types || rec.max_type > p.dev.num_types)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "bead type exceeds the parameter table (" +
				std::to_string(std::max(lig.max_type, rec.max_type)) + " > " +
				std::to_string(p.dev.num_types) + ")");
	if (lig.max_mapped >= g.inner_desc.numGrids || lig.max_mapped >= g.outer_desc.numGrids)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "ligand mapped type exceeds the grid's channels");
	if (g.nl_has_entries && g.nl_max_index >= rec.dev.n)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "neighbour list indexes beyond the receptor");
}

ModesLaunch Context::modes_launch(gba_id rec, gba_id lig, gba_id grid_rec, gba_id grid_lig,
		gba_id params) {
	Lock g(mu);
	auto* R = static_cast<ProteinItem*>(find(rec, ItemKind::Protein));
	auto* Lg = static_cast<ProteinItem*>(find(lig, ItemKind::Protein));
	auto* GR = static_cast<GridItem*>(find(grid_rec, ItemKind::Grid));
	auto* GL = static_cast<GridItem*>(find(grid_lig, ItemKind::Grid));
	auto* P = static_cast<ParamsItem*>(find(params, ItemKind::Params));
	validate_pair(*R, *Lg, *GR, *P);
	/* receptor beads are interpolated in the ligand grid */
	if (R->max_mapped >= GL->inner_desc.numGrids || R->max_mapped >= GL->outer_desc.numGrids)
		throw ApiError(GBA_ERR_INVALID_ARGUMENT, "receptor mapped type exceeds the ligand grid's channels");
	ModesLaunch L{};
	L.rec = R->dev;
	L.lig = Lg->dev;
	L.grid_rec = apply_kernel_options(GR->dev);
	L.grid_lig = apply_kernel_options(GL->dev);
	L.par = P->dev;
	L.par.pair = P->pair_table(GR->dev.nl.dPlateau2);
	L.trig = trig;
	L.ref_order = (kernel_opts & GBA_KOPT_REFERENCE_ORDER) ? 1 : 0;
	L.rec_modes = R->dev.modes;
	L.rec_ms = mode_stride(R->dev.n_modes);
	L.lig_modes = Lg->dev.modes;
	L.lig_ms = mode_stride(Lg->dev.n_modes);
	return L;
}

void Context::run_modes(ModesLaunch& L, cudaStream_t s) {
	StreamScratch scratch(scratch_pool);
	L.next = (unsigned long long*)scratch.get(2 * sizeof(unsigned long long), s);
	L.next2 = L.next + 1;
	if (L.ref_order)
		L.ref_rf = (float4*)scratch.get(modes_ref_warps(L, num_sms) * std::max<uint32_t>(1, L.rec.n) * sizeof(float4), s);
	check_cuda(cudaMemsetAsync(L.next, 0, 2 * sizeof(unsigned long long), s), "modes energy: pose counters");
	check_cuda(launch_modes_energy(L, num_sms, s), "modes energy launch");
}

void Context::run_rigid(RigidLaunch& L, cudaStream_t s, const TuneParams* shape) {
	StreamScratch scratch(scratch_pool);
	L.order = pose_order(L.dofs, 6, L.n, L.m.grid.outer, s, scratch);
	L.next = (unsigned long long*)scratch.get(sizeof(unsigned long long), s);
	check_cuda(cudaMemsetAsync(L.next, 0, sizeof(unsigned long long), s), "rigid energy: pose counter");
	const TuneParams tp = shape ? *shape : tuned("energy", L.n);
	const int threads = tp.threads;
	const int warps_per_block = threads / 32;
	const int bps = std::min(tp.blocks_per_sm, rigid_blocks_per_sm(threads, L.census != nullptr, L.bound4 && !L.census,
			L.roundwise && !L.census, L.ref_order && !L.census));
	size_t want = (L.n + warps_per_block - 1) / warps_per_block;
	size_t blocks = std::min<size_t>(want, (size_t)num_sms * bps);
	if (blocks == 0) blocks = 1;
	if (!timing) {
		check_cuda(launch_rigid_energy(L, (int)blocks, threads, s), "rigid energy launch");
		return;
	}
	if (timing_used == kTimingPool) timing_fold();
	if (timing_used == timing_events.size()) {
		std::pair<cudaEvent_t, cudaEvent_t> e{};
		check_cuda(cudaEventCreate(&e.first), "kernel timing: event");
		check_cuda(cudaEventCreate(&e.second), "kernel timing: event");
		timing_events.push_back(e);
	}
	auto& e = timing_events[timing_used];
	check_cuda(cudaEventRecord(e.first, s), "kernel timing: record");
	check_cuda(launch_rigid_energy(L, (int)blocks, threads, s), "rigid energy launch");
	check_cuda(cudaEventRecord(e.second, s), "kernel timing: record");
	++timing_used;
}

}  // namespace gba
