/*
 * ref_driver.cpp -- runs the reference's own CPU energy service.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled together with the unmodified
 * gpuATTRACT 2.0 sources (see build_ref.sh) into oracle/_ref/libattract_ref.so.
 * It builds the reference's Protein / GridUnion / ParamTable / SimParam data
 * items from plain arrays, registers them in its DataManager and pushes the
 * poses through its Server<Types_6D<float>> with CPUEnergyService6D<float>
 * (or the modes variant) exactly as Configurator_6D::init + scATTRACT::run do
 * (src/service/Configurator_6D.tpp:31-142, src/apps/sc/scATTRACT.tpp:33-48).
 * Used to pin the C++ restatement in attract_oracle.cpp and to write the
 * golden fixtures under tests/golden/.
 */
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "Protein.h"
#include "GridUnion.h"
#include "IntrplGrid.h"
#include "NLGrid.h"
#include "ParamTable.h"
#include "SimParam.h"
#include "DataManager.h"
#include "CPUEnergyService6D.h"
#include "CPUEnergyService6DModes.h"
#include "Server.h"
#include "Request.h"
#include "Types_6D.h"
#include "Types_6D_Modes.h"
#include "WorkItem.h"
#include "readFile.h"
#include <algorithm>

#include "oracle.h"

using namespace as;

namespace {

std::string g_err;

std::shared_ptr<Protein<float>> make_protein(const orc_protein* p) {
	auto prot = std::make_shared<Protein<float>>();
	prot->setNumAtoms(p->n);
	float* pos = prot->getOrCreatePosPtr();
	std::memcpy(pos, p->xyz, sizeof(float) * 3 * p->n);
	unsigned* type = prot->getOrCreateTypePtr();
	std::memcpy(type, p->type, sizeof(unsigned) * p->n);
	prot->setNumMappedTypes(1);
	unsigned* mapped = prot->getOrCreateMappedPtr();
	std::memcpy(mapped, p->mapped, sizeof(unsigned) * p->n);
	float* charge = prot->getOrCreateChargePtr();
	std::memcpy(charge, p->charge, sizeof(float) * p->n);
	if (p->n_modes > 0) {
		prot->setNumModes(p->n_modes);
		float* modes = prot->getOrCreateModePtr();
		std::memcpy(modes, p->modes, sizeof(float) * 3 * p->n * p->n_modes);
		float* mf = prot->getOrCreateModeForcePtr();
		std::memcpy(mf, p->mode_force, sizeof(float) * p->n_modes);
	}
	return prot;
}

std::shared_ptr<IntrplGrid<float>> make_intrpl(const gba_intrpl_desc& d, const float* data) {
	IntrplGrid<float>::Desc desc;
	std::memset(desc.typemask, 0, sizeof(desc.typemask));
	desc.numGrids = d.numGrids;
	desc.dimN.x = d.dimN[0]; desc.dimN.y = d.dimN[1]; desc.dimN.z = d.dimN[2];
	desc.gridSpacing = d.gridSpacing;
	desc.posMin.x = d.posMin[0]; desc.posMin.y = d.posMin[1]; desc.posMin.z = d.posMin[2];
	size_t n = (size_t)d.numGrids * d.dimN[0] * d.dimN[1] * d.dimN[2];
	desc.grid = new float4[n];
	std::memcpy(desc.grid, data, n * sizeof(float4));
	return std::make_shared<IntrplGrid<float>>(desc);
}

std::shared_ptr<GridUnion<float>> make_grid(const orc_grid* g) {
	auto inner = make_intrpl(g->inner, g->inner_data);
	auto outer = make_intrpl(g->outer, g->outer_data);
	NLGrid<float>::Desc nd;
	nd.dimN.x = g->nl.dimN[0]; nd.dimN.y = g->nl.dimN[1]; nd.dimN.z = g->nl.dimN[2];
	nd.gridSpacing = g->nl.gridSpacing;
	nd.dPlateau = g->nl.dPlateau;
	nd.posMin.x = g->nl.posMin[0]; nd.posMin.y = g->nl.posMin[1]; nd.posMin.z = g->nl.posMin[2];
	size_t nv = (size_t)nd.dimN.x * nd.dimN.y * nd.dimN.z;
	nd.grid = new NeighbourDesc[nv];
	for (size_t i = 0; i < nv; ++i) { nd.grid[i].numEl = g->nl_grid[i].numEl; nd.grid[i].idx = g->nl_grid[i].idx; }
	nd.numEl = g->nl.numEl;
	nd.neighborArray = new unsigned[nd.numEl > 0 ? nd.numEl : 1];
	std::memcpy(nd.neighborArray, g->nl_list, sizeof(unsigned) * nd.numEl);
	auto nl = std::make_shared<NLGrid<float>>(nd);
	return std::make_shared<GridUnion<float>>(inner, outer, nl);
}

std::shared_ptr<ParamTable<float>> make_table(const orc_params* p) {
	auto t = std::make_shared<ParamTable<float>>();
	t->setNumTypes(p->num_types);
	t->setPotShape(p->potshape == GBA_POTSHAPE_8_6 ? PotShape::_8_6 : PotShape::_12_6);
	auto* tab = t->getOrCreateTable();
	for (size_t i = 0; i < (size_t)p->num_types * p->num_types; ++i) {
		tab[i].rc = p->table[i].rc;
		tab[i].ac = p->table[i].ac;
		tab[i].ipon = p->table[i].ipon;
		tab[i].rmin2 = p->table[i].rmin2;
		tab[i].emin = p->table[i].emin;
	}
	return t;
}

std::shared_ptr<SimParam<float>> make_sim(const orc_params* p) {
	auto s = std::make_shared<SimParam<float>>();
	s->dielec = p->dielec == GBA_DIELEC_CONSTANT ? Dielec::constant : Dielec::variable;
	s->ffelec = p->ffelec;
	s->epsilon = 0;
	return s;
}

}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

/* Rigid scoring through Server<Types_6D<float>> + CPUEnergyService6D<float>. */
int ref_energy_6d(const orc_protein* rec, const orc_protein* lig, const orc_grid* grid,
		const orc_params* par, const gba_dof6d* dofs, size_t n, gba_result6d* out,
		int nworkers, int item_size) {
	try {
		auto dm = std::make_shared<DataManager>();
		Common common;
		common.recId = dm->add(make_protein(rec));
		common.ligId = dm->add(make_protein(lig));
		common.gridId = dm->add(make_grid(grid));
		common.tableId = dm->add(make_table(par));
		common.paramsId = dm->add(make_sim(par));
		auto service = std::make_shared<CPUEnergyService6D<float>>(dm);
		Server<Types_6D<float>> server(service);
		server.createWorkers(nworkers > 0 ? nworkers : 1);
		if (item_size > 0) server.setItemSize(item_size);
		server.setWaitTime(3600 * 1000);
		std::vector<DOF_6D<float>> in(n);
		for (size_t i = 0; i < n; ++i) {
			in[i].pos.x = dofs[i].pos[0]; in[i].pos.y = dofs[i].pos[1]; in[i].pos.z = dofs[i].pos[2];
			in[i].ang.x = dofs[i].ang[0]; in[i].ang.y = dofs[i].ang[1]; in[i].ang.z = dofs[i].ang[2];
		}
		std::vector<Result_6D<float>> res(n);
		Server<Types_6D<float>>::request_t req(in.data(), n, common);
		server.submit(req);
		server.wait(req, res.data());
		for (size_t i = 0; i < n; ++i) {
			out[i].E = res[i].E;
			out[i].pos[0] = res[i].pos.x; out[i].pos[1] = res[i].pos.y; out[i].pos[2] = res[i].pos.z;
			out[i].ang[0] = res[i].ang.x; out[i].ang[1] = res[i].ang.y; out[i].ang[2] = res[i].ang.z;
		}
	} catch (std::exception& e) {
		g_err = e.what();
		return GBA_ERR_INVALID_ARGUMENT;
	}
	return GBA_OK;
}

/* Flexible scoring with CPUEnergyService6DModes<float>'s own item processor.
 *
 * That processor sizes its scratch buffers with the receptor/ligand roles
 * swapped (allocateBufferRec fills the ligand buffers and allocateBufferLig the
 * receptor ones, src/service/CPUEnergyService6DModes.tpp:47-57), so any real
 * pair overruns a buffer or dereferences an unallocated one.  The driver
 * therefore calls the processor directly -- the same function a Server worker
 * calls (src/server/Worker.tpp:14-35) -- and first hands it one zero-pose item
 * on a placeholder pair of sizes (A, A+1), A = max(nRec, nLig): that sizes
 * both buffer sets large enough and evaluates nothing.  Every real item then
 * runs the reference's code unchanged. */
int ref_energy_6d_modes(const orc_protein* rec, const orc_protein* lig, const orc_grid* grid_rec,
		const orc_grid* grid_lig, const orc_params* par, const gba_dof6d_modes* dofs, size_t n,
		gba_result6d_modes* out, int nworkers, int item_size) {
	(void)nworkers;
	try {
		auto dm = std::make_shared<DataManager>();
		Common_Modes common;
		common.recId = dm->add(make_protein(rec));
		common.ligId = dm->add(make_protein(lig));
		common.gridIdRec = dm->add(make_grid(grid_rec));
		common.gridIdLig = dm->add(make_grid(grid_lig));
		common.tableId = dm->add(make_table(par));
		common.paramsId = dm->add(make_sim(par));
		Common_Modes::numModesRec = rec->n_modes;
		Common_Modes::numModesLig = lig->n_modes;
		auto service = std::make_shared<CPUEnergyService6DModes<float>>(dm);
		auto process = service->createItemProcessor();

		const uint32_t A = std::max(rec->n, lig->n);
		std::vector<float> zx(3 * (size_t)(A + 1), 0.f), zq(A + 1, 0.f);
		std::vector<uint32_t> zt(A + 1, 0u);
		orc_protein pa = {A, zx.data(), zt.data(), zt.data(), zq.data(), 0, nullptr, nullptr};
		orc_protein pb = {A + 1, zx.data(), zt.data(), zt.data(), zq.data(), 0, nullptr, nullptr};
		Common_Modes warm = common;
		warm.recId = dm->add(make_protein(&pa));
		warm.ligId = dm->add(make_protein(&pb));
		DOF_6D_Modes<float> dummy_in;
		Result_6D_Modes<float> dummy_out;
		WorkItem<DOF_6D_Modes<float>, Common_Modes, Result_6D_Modes<float>> w0(&dummy_in, 0, &warm, &dummy_out);
		process(&w0);

		std::vector<DOF_6D_Modes<float>> in(n);
		for (size_t i = 0; i < n; ++i) {
			auto& d = in[i];
			d._6D.pos.x = dofs[i].rigid.pos[0]; d._6D.pos.y = dofs[i].rigid.pos[1]; d._6D.pos.z = dofs[i].rigid.pos[2];
			d._6D.ang.x = dofs[i].rigid.ang[0]; d._6D.ang.y = dofs[i].rigid.ang[1]; d._6D.ang.z = dofs[i].rigid.ang[2];
			for (int m = 0; m < GBA_MODES_MAX; ++m) { d.modesRec[m] = dofs[i].modesRec[m]; d.modesLig[m] = dofs[i].modesLig[m]; }
		}
		std::vector<Result_6D_Modes<float>> res(n);
		std::memset((void*)res.data(), 0, sizeof(Result_6D_Modes<float>) * n);
		const size_t step = item_size > 0 ? (size_t)item_size : 100;
		for (size_t b = 0; b < n; b += step) {
			const unsigned sz = (unsigned)std::min(step, n - b);
			WorkItem<DOF_6D_Modes<float>, Common_Modes, Result_6D_Modes<float>> item(in.data() + b, sz, &common, res.data() + b);
			process(&item);
			if (!item.isProcessed()) throw std::runtime_error("modes item not processed");
		}
		for (size_t i = 0; i < n; ++i) {
			auto& r = res[i];
			std::memset(&out[i], 0, sizeof(out[i]));
			out[i].rigid.E = r._6D.E;
			out[i].rigid.pos[0] = r._6D.pos.x; out[i].rigid.pos[1] = r._6D.pos.y; out[i].rigid.pos[2] = r._6D.pos.z;
			out[i].rigid.ang[0] = r._6D.ang.x; out[i].rigid.ang[1] = r._6D.ang.y; out[i].rigid.ang[2] = r._6D.ang.z;
			for (unsigned m = 0; m < rec->n_modes; ++m) out[i].modesRec[m] = r.modesRec[m];
			for (unsigned m = 0; m < lig->n_modes; ++m) out[i].modesLig[m] = r.modesLig[m];
		}
	} catch (std::exception& e) {
		g_err = e.what();
		return GBA_ERR_INVALID_ARGUMENT;
	}
	return GBA_OK;
}

/* Reads a reduced PDB with the reference's reader (src/fileIO/readFile.cpp:107-178),
 * applies the default type map (99 -> 0) when asked.  Returns the bead count;
 * copies up to cap beads into the SoA buffers. */
int ref_read_pdb(const char* path, int default_map, float* xyz, uint32_t* type, float* charge, int cap) {
	try {
		auto p = createProteinFromPDB<float>(path);
		int n = (int)p->numAtoms();
		if (default_map) applyDefaultMapping(p->numAtoms(), p->type(), p->type());
		if (n <= cap) {
			for (int i = 0; i < n; ++i) {
				xyz[i] = p->xPos()[i]; xyz[cap + i] = p->yPos()[i]; xyz[2 * cap + i] = p->zPos()[i];
				type[i] = p->type()[i];
				charge[i] = p->charge()[i];
			}
		}
		return n;
	} catch (std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

/* Reads attract.par with the reference's reader (src/fileIO/readFile.cpp:440-527).
 * Returns numTypes and fills up to cap*cap entries; *potshape gets GBA_POTSHAPE_*. */
int ref_read_params(const char* path, gba_ffparam* table, int cap, int* potshape) {
	try {
		auto t = createParamTableFromFile<float>(path);
		int T = (int)t->numTypes();
		*potshape = t->potShape() == PotShape::_8_6 ? GBA_POTSHAPE_8_6 : GBA_POTSHAPE_12_6;
		if (T <= cap) {
			for (int i = 0; i < T * T; ++i) {
				table[i].rc = t->table()[i].rc;
				table[i].ac = t->table()[i].ac;
				table[i].ipon = t->table()[i].ipon;
				table[i].rmin2 = t->table()[i].rmin2;
				table[i].emin = t->table()[i].emin;
			}
		}
		return T;
	} catch (std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

}  // extern "C"
