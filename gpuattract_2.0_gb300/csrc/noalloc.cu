/*
 * noalloc.cu -- gba_energy_6d_noalloc: the fused rigid energy launch of
 * gba_energy_6d for device-resident poses, with the visiting-order scratch
 * (the pose counter, translation-cell counts, each pose's cell and rank, the
 * order) taken from a fixed, statically allocated device array instead of the
 * stream-ordered allocator.  The call performs no device or host memory
 * allocation: no cudaMalloc / cudaMallocAsync / cudaFree, no allocating
 * library routine; the pose counter and the cell counts are cleared with
 * cudaMemsetAsync on every call.  Everything else it reads was made when the
 * data was uploaded: the pair-term table of a (parameter table, plateau)
 * combination is built when the second of the two is added to the context.
 * The receptor-typed copy of a neighbour list is the one exception: it is
 * built by the first allocating scoring call of a (grid, receptor)
 * combination; until then this call walks the plain list and gathers each
 * neighbour's type (the same results bit for bit, a little slower).
 *
 * Scratch: one file-scope __device__ array of kNoAllocScratchBytes per device
 * (2 MiB), addressed through cudaGetSymbolAddress by the first call made on
 * each context (with the context's device current) and kept with the
 * context; that first call may load the module, so make it before any stream
 * capture.  Batches of more than kNoAllocMaxPoses poses are rejected with
 * GBA_ERR_INVALID_ARGUMENT.  The first 256 bytes hold the pose counter,
 * cleared by every call like the cell counts after it; nothing else in the
 * scratch has to start at zero: the order kernels write every key and index
 * they read back.  The array is shared by every
 * call on a device: overlapping calls (other streams, threads or contexts on
 * the same device) race on it and must be serialized by the caller.
 */
#include <algorithm>
#include <string>

#include "gba_context.h"

namespace gba {

constexpr size_t kNoAllocScratchBytes = (size_t)2 << 20;
constexpr size_t kNoAllocMaxPoses = 65536;
constexpr size_t kCounterBytes = 256;   /* the pose counter, keeping the order scratch 256-byte aligned */

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

/* Device address of the scratch array, resolved once per context (with the
 * context's device current, before the first launch that uses it). */
void* noalloc_scratch(Context& ctx) {
	if (!ctx.noalloc_scratch) {
		void* p = nullptr;
		check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), "gba_energy_6d_noalloc: cudaGetSymbolAddress");
		ctx.noalloc_scratch = p;
	}
	return ctx.noalloc_scratch;
}

}  // namespace gba

using namespace gba;

extern "C" int gba_energy_6d_noalloc(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_dof6d* dofs, size_t n, gba_result6d* out, void* stream) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	try {
		if (n == 0) return GBA_OK;
		if (!dofs || !out) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_energy_6d_noalloc: null dofs/out");
		if (n > kNoAllocMaxPoses)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_energy_6d_noalloc: " + std::to_string(n) +
					" poses exceed the static scratch limit of " + std::to_string(kNoAllocMaxPoses));
		ctx->bind();
		if (!is_device_pointer(dofs) || !is_device_pointer(out))
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_energy_6d_noalloc: device pointers required");
		void* scratch = noalloc_scratch(*ctx);
		RigidLaunch L = ctx->rigid_launch(rec, lig, grid, params, false);
		cudaStream_t s = (cudaStream_t)stream;
		L.n = n;
		L.dofs = dofs;
		L.out = out;
		L.census = nullptr;
		L.next = (unsigned long long*)scratch;
		check_cuda(cudaMemsetAsync(L.next, 0, sizeof(unsigned long long), s), "gba_energy_6d_noalloc: pose counter");
		L.order = (ctx->order_enabled && n >= Context::kOrderMinPoses)
				? pose_order_in(dofs, 6, n, L.m.grid.outer, (char*)scratch + kCounterBytes,
						kNoAllocScratchBytes - kCounterBytes, s)
				: nullptr;
		/* launch shape as gba_energy_6d chooses it */
		const TuneParams tp = ctx->pair_tuned("energy", PairKey{rec, lig, grid, params});
		const int threads = tp.threads;
		const int bps = std::min(tp.blocks_per_sm, rigid_blocks_per_sm(threads, false, L.bound4 != 0, false,
				L.ref_order != 0));
		size_t blocks = std::min<size_t>((n + threads / 32 - 1) / (threads / 32), (size_t)ctx->num_sms * bps);
		if (blocks == 0) blocks = 1;
		check_cuda(launch_rigid_energy(L, (int)blocks, threads, s), "gba_energy_6d_noalloc: launch");
	} catch (const ApiError& e) {
		ctx->set_error(e.what());
		return e.code;
	} catch (const std::exception& e) {
		ctx->set_error(e.what());
		return GBA_ERR_INVALID_ARGUMENT;
	}
	return GBA_OK;
}
