/*
 * gb300_service.h -- the GB300 energy services behind the request interface.
 *
 *   GB300EnergyService6D       Types_6D      (rigid), stands in for
 *                              CPUEnergyService6D / GPUEnergyService6D
 *                              (src/service/CPUEnergyService6D.tpp:63-200,
 *                              src/service/GPUEnergyService6D.tpp:470-510)
 *   GB300EnergyService6DModes  Types_6D_Modes (normal modes), stands in for
 *                              src/service/CPUEnergyService6DModes.tpp:76-336
 * Each item processor hands its whole work item to libgbattract through the
 * C ABI (one fused launch per item, the copies in and out of the
 * server's pinned buffers on a per-processor stream) and marks it processed.
 * Data items are addressed by ids inside one gba_ctx: Common carries the
 * protein / grid / table ids exactly as the reference's Common does
 * (src/model/Types_6D.h:39-45); paramsId (SimParam) is folded into the
 * parameter table upload and is ignored here.
 */
#ifndef GBA_GB300_SERVICE_H_
#define GBA_GB300_SERVICE_H_

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "gbattract.h"
#include "gba_server.h"

namespace gba {
namespace host {

/* Common, src/model/Types_6D.h:39-45 */
struct Common {
	gba_id gridId, ligId, recId, tableId, paramsId;
};

/* Common_Modes, src/model/Types_6D_Modes.h:43-52 */
struct Common_Modes {
	gba_id gridIdRec, gridIdLig, ligId, recId, tableId, paramsId;
};

using Types_6D = GenericTypes<gba_dof6d, Common, gba_result6d>;
using Types_6D_Modes = GenericTypes<gba_dof6d_modes, Common_Modes, gba_result6d_modes>;

/* HostPinnedAllocator, src/allocator/HostPinnedAllocator.tpp: page-locked
 * server buffers so the service's copies run asynchronously. */
template <typename T>
class HostPinnedAllocator : public Allocator<T> {
public:
	T* allocate(size_t size) override {
		void* p = nullptr;
		if (cudaMallocHost(&p, sizeof(T) * (size ? size : 1)) != cudaSuccess)
			throw std::runtime_error("HostPinnedAllocator: cudaMallocHost failed");
		return static_cast<T*>(p);
	}
	void deallocate(T* buffer, size_t) override { cudaFreeHost(buffer); }
};

inline void gba_throw(gba_ctx* ctx, int rc) {
	if (rc != GBA_OK) throw std::runtime_error(std::string("libgbattract: ") + gba_last_error(ctx));
}

class GB300EnergyService6D : public Service<Types_6D> {
public:
	explicit GB300EnergyService6D(gba_ctx* ctx)
		: Service<Types_6D>(std::make_shared<HostPinnedAllocator<gba_dof6d>>(),
		                     std::make_shared<HostPinnedAllocator<gba_result6d>>()),
		  _ctx(ctx) {}

	itemProcessor_t createItemProcessor() override {
		gba_ctx* ctx = _ctx;
		auto stream = std::make_shared<StreamHolder>();
		return [ctx, stream](workItem_t* item) -> bool {
			if (item == nullptr) return false;
			const Common* c = item->common();
			gba_throw(ctx, gba_energy_6d(ctx, c->recId, c->ligId, c->gridId, c->tableId,
					item->inputBuffer(), item->size(), item->resultBuffer(), stream->get()));
			item->setProcessed();
			return false;
		};
	}

private:
	struct StreamHolder {
		cudaStream_t s = nullptr;
		void* get() {
			if (!s && cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
				throw std::runtime_error("cudaStreamCreate failed");
			return (void*)s;
		}
		~StreamHolder() {
			if (s) cudaStreamDestroy(s);
		}
	};
	gba_ctx* _ctx;
};

class GB300EnergyService6DModes : public Service<Types_6D_Modes> {
public:
	explicit GB300EnergyService6DModes(gba_ctx* ctx)
		: Service<Types_6D_Modes>(std::make_shared<HostPinnedAllocator<gba_dof6d_modes>>(),
		                           std::make_shared<HostPinnedAllocator<gba_result6d_modes>>()),
		  _ctx(ctx) {}

	itemProcessor_t createItemProcessor() override {
		gba_ctx* ctx = _ctx;
		return [ctx](workItem_t* item) -> bool {
			if (item == nullptr) return false;
			const Common_Modes* c = item->common();
			gba_throw(ctx, gba_energy_6d_modes(ctx, c->recId, c->ligId, c->gridIdRec, c->gridIdLig,
					c->tableId, item->inputBuffer(), item->size(), item->resultBuffer(), nullptr));
			item->setProcessed();
			return false;
		};
	}

private:
	gba_ctx* _ctx;
};

}  // namespace host
}  // namespace gba

#endif
