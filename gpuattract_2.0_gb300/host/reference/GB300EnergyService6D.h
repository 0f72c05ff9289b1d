/*
 * GB300EnergyService6D.h -- the reference-side binding of libgbattract.
 *
 * Drop-in energy service for gpuATTRACT 2.0's request server: it derives from
 * the reference's own EnergyService<Types_6D<float>> (src/service/EnergyService.h)
 * and is created where ServiceFactory::create builds its CPU/GPU services
 * (src/service/ServiceFactory.tpp:30-46).  It is compiled inside the
 * reference tree (it includes the reference's headers) and links
 * libgbattract; nothing else in the reference changes.
 *
 * Item processor: resolves the Common ids through the DataManager exactly as
 * CPUEnergyService6D does (src/service/CPUEnergyService6D.tpp:76-89), uploads
 * each data item to the device once (cached by item address), then hands the
 * whole work item -- the server's pinned DOF_6D<float> / Result_6D<float>
 * slices, bit-compatible with gba_dof6d / gba_result6d -- to gba_energy_6d.
 * Errors come back as std::runtime_error, the reference's CUDA_CHECK
 * behaviour (src/commons/macros.h:62-72).
 */
#ifndef AS_GB300ENERGYSERVICE6D_H_
#define AS_GB300ENERGYSERVICE6D_H_

#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "EnergyService.h"
#include "Allocator.h"
#include "DataManager.h"
#include "GridUnion.h"
#include "IntrplGrid.h"
#include "NLGrid.h"
#include "ParamTable.h"
#include "Protein.h"
#include "SimParam.h"
#include "Types_6D.h"
#include "WorkItem.h"

#include "gbattract.h"

namespace as {

static_assert(sizeof(DOF_6D<float>) == sizeof(gba_dof6d), "DOF_6D<float> layout");
static_assert(sizeof(Result_6D<float>) == sizeof(gba_result6d), "Result_6D<float> layout");
static_assert(sizeof(ParamTable<float>::type_t) == sizeof(gba_ffparam), "attractFFParams_t layout");

/* Page-locked server buffers (the role of the reference's HostPinnedAllocator). */
template <typename T>
class GB300PinnedAllocator : public Allocator<T> {
public:
	T* allocate(size_t n) override {
		void* p = nullptr;
		if (cudaMallocHost(&p, sizeof(T) * (n ? n : 1)) != cudaSuccess)
			throw std::runtime_error("GB300PinnedAllocator: cudaMallocHost failed");
		return static_cast<T*>(p);
	}
	void deallocate(T* p, size_t) override { cudaFreeHost(p); }
};

class GB300EnergyService6D : public EnergyService<Types_6D<float>> {
public:
	using base_t = EnergyService<Types_6D<float>>;
	using typename base_t::itemProcessor_t;
	using typename base_t::distributor_t;
	using workItem_t = typename Service<Types_6D<float>>::workItem_t;
	using common_t = Common;

	GB300EnergyService6D(std::shared_ptr<DataManager> dataMng, int device = 0)
		: base_t(std::make_shared<GB300PinnedAllocator<DOF_6D<float>>>(),
		         std::make_shared<GB300PinnedAllocator<Result_6D<float>>>(), dataMng) {
		if (gba_create(device, &_ctx) != GBA_OK)
			throw std::runtime_error(std::string("gba_create: ") + gba_last_error(nullptr));
	}

	~GB300EnergyService6D() override { gba_destroy(_ctx); }

	itemProcessor_t createItemProcessor() override {
		return [this](workItem_t* item) -> bool {
			if (item == nullptr) return false;
			const Common* c = item->common();
			gba_id rec, lig, grid, params;
			resolve(*c, rec, lig, grid, params);
			check(gba_energy_6d(_ctx, rec, lig, grid, params,
					reinterpret_cast<const gba_dof6d*>(item->inputBuffer()), item->size(),
					reinterpret_cast<gba_result6d*>(item->resultBuffer()), nullptr));
			item->setProcessed();
			return false;
		};
	}

	/* every worker may take any item: one device context serves them all */
	distributor_t createDistributor() override {
		return [](common_t const*, size_t numWorkers) {
			std::vector<workerId_t> ids(numWorkers);
			std::iota(ids.begin(), ids.end(), 0u);
			return ids;
		};
	}

private:
	void check(int rc) {
		if (rc != GBA_OK) throw std::runtime_error(std::string("libgbattract: ") + gba_last_error(_ctx));
	}

	void resolve(const Common& c, gba_id& rec, gba_id& lig, gba_id& grid, gba_id& params) {
		std::lock_guard<std::mutex> g(_mu);
		auto p_rec = std::dynamic_pointer_cast<Protein<float>>(_dataMng->get(c.recId));
		auto p_lig = std::dynamic_pointer_cast<Protein<float>>(_dataMng->get(c.ligId));
		auto p_grid = std::dynamic_pointer_cast<GridUnion<float>>(_dataMng->get(c.gridId));
		auto p_tab = std::dynamic_pointer_cast<ParamTable<float>>(_dataMng->get(c.tableId));
		auto p_sim = std::dynamic_pointer_cast<SimParam<float>>(_dataMng->get(c.paramsId));
		if (!p_rec || !p_lig || !p_grid || !p_tab || !p_sim)
			throw std::invalid_argument("GB300EnergyService6D: data item of the wrong type");
		rec = cached(p_rec.get(), [&] { return upload(*p_rec); });
		lig = cached(p_lig.get(), [&] { return upload(*p_lig); });
		grid = cached(p_grid.get(), [&] { return upload(*p_grid); });
		params = cached(p_tab.get(), [&] { return upload(*p_tab, *p_sim); });
	}

	template <typename F>
	gba_id cached(const void* key, F make) {
		auto it = _ids.find(key);
		if (it != _ids.end()) return it->second;
		const gba_id id = make();
		_ids.emplace(key, id);
		return id;
	}

	gba_id upload(Protein<float>& p) {
		gba_id id;
		const unsigned n = p.numAtoms();
		check(gba_upload_protein(_ctx, n, p.xPos(), p.type(), p.mappedType(), p.charge(), p.numModes(),
				p.numModes() ? p.xModes() : nullptr, p.numModes() ? p.modeForce() : nullptr, &id));
		return id;
	}

	static gba_intrpl_desc desc(const IntrplGrid<float>& g) {
		gba_intrpl_desc d;
		d.numGrids = g.numTypes();
		d.dimN[0] = g.dimN().x; d.dimN[1] = g.dimN().y; d.dimN[2] = g.dimN().z;
		d.gridSpacing = g.dVox();
		d.posMin[0] = g.pos().x; d.posMin[1] = g.pos().y; d.posMin[2] = g.pos().z;
		return d;
	}

	gba_id upload(GridUnion<float>& gu) {
		const gba_intrpl_desc in = desc(*gu.inner), out = desc(*gu.outer);
		const NLGrid<float>& nl = *gu.NL;
		gba_nl_desc nd;
		nd.dimN[0] = nl.dimN().x; nd.dimN[1] = nl.dimN().y; nd.dimN[2] = nl.dimN().z;
		nd.gridSpacing = nl.dVox();
		nd.dPlateau = std::sqrt(nl.dPlateau2());
		nd.posMin[0] = nl.pos().x; nd.posMin[1] = nl.pos().y; nd.posMin[2] = nl.pos().z;
		nd.numEl = nl.neighborListSize();
		gba_id id;
		check(gba_upload_grid(_ctx, &in, reinterpret_cast<const float*>(gu.inner->getHostGridPtr(0)),
				&out, reinterpret_cast<const float*>(gu.outer->getHostGridPtr(0)), &nd,
				reinterpret_cast<const gba_neighbour_desc*>(nl.grid()), nl.neighborList(), &id));
		return id;
	}

	gba_id upload(ParamTable<float>& t, SimParam<float>& s) {
		gba_id id;
		check(gba_upload_params(_ctx, t.numTypes(), reinterpret_cast<const gba_ffparam*>(t.table()),
				t.potShape() == PotShape::_8_6 ? GBA_POTSHAPE_8_6 : GBA_POTSHAPE_12_6,
				s.dielec == Dielec::constant ? GBA_DIELEC_CONSTANT : GBA_DIELEC_VARIABLE, s.ffelec, &id));
		return id;
	}

	gba_ctx* _ctx = nullptr;
	std::mutex _mu;
	std::map<const void*, gba_id> _ids;
};

}  // namespace as

#endif
