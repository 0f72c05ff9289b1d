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
#include "grid_orig.h"
#include "DOFTransform.h"
#include "TypeMap.h"
#include <algorithm>
#include <cstdlib>
#include <fstream>

#include "oracle.h"
#include "../include/gbattract_io.h"

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

/* ---- file formats, through the reference's own readers and writers ---- */

extern "C" {

/* readDOF + readDOFHeader<float> (src/fileIO/readFile.cpp:579-651,747-871).
 * values[(s*M + m)*16 + k] as gba_read_dof lays them out (DOFConverter's
 * double -> float); returns the structure count, *molecules the molecule
 * count, header fields into hdr[0..3] = auto_pivot, centered rec, centered
 * lig, num_pivots and pivots[16*3]. */
int ref_read_dof(const char* path, float* values, int32_t* counts, long cap, int32_t* molecules, int32_t* hdr,
		float* pivots) {
	try {
		auto h = readDOFHeader<float>(path);
		auto D = readDOF(path);
		const long M = (long)D.size(), S = M ? (long)D[0].size() : 0;
		*molecules = (int32_t)M;
		hdr[0] = h.auto_pivot;
		hdr[1] = h.centered_receptor;
		hdr[2] = h.centered_ligands;
		hdr[3] = (int32_t)h.pivots.size();
		for (size_t k = 0; k < h.pivots.size() && k < 16; ++k) {
			pivots[3 * k] = h.pivots[k].x;
			pivots[3 * k + 1] = h.pivots[k].y;
			pivots[3 * k + 2] = h.pivots[k].z;
		}
		if (S * M <= cap) {
			for (long s = 0; s < S; ++s)
				for (long m = 0; m < M; ++m) {
					const DOF& d = D[m][s];
					float* o = values + (s * M + m) * 16;
					o[0] = (float)d._6D.ang.x; o[1] = (float)d._6D.ang.y; o[2] = (float)d._6D.ang.z;
					o[3] = (float)d._6D.pos.x; o[4] = (float)d._6D.pos.y; o[5] = (float)d._6D.pos.z;
					for (unsigned k = 6; k < d.numDofs && k < 16; ++k) o[k] = (float)d.dofs[k - 6];
					counts[s * M + m] = (int32_t)d.numDofs;
				}
		}
		return (int)S;
	} catch (std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

/* readResult (src/fileIO/readFile.cpp:653-745), flattened like
 * gba_read_results: E, then per gradient block its _6D and modes values. */
long ref_read_results(const char* path, double* out, int32_t* counts, long cap, int stride) {
	try {
		auto R = readResult(path);
		for (size_t i = 0; i < R.size() && (long)i < cap; ++i) {
			std::vector<double> v{R[i].E};
			for (auto& g : R[i].gradients) {
				v.insert(v.end(), g._6D.begin(), g._6D.end());
				v.insert(v.end(), g.modes.begin(), g.modes.end());
			}
			counts[i] = (int32_t)v.size();
			for (int k = 0; k < stride; ++k) out[i * stride + k] = k < (int)v.size() ? v[k] : 0.0;
		}
		return (long)R.size();
	} catch (std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

/* operator<<(Result_6D<float>) / operator<<(Result_6D_Modes<float>), each
 * followed by std::endl as the reference's apps print (emATTRACT.tpp:55-57). */
int ref_write_results(const char* path, const float* results, long n, int n_modes_rec, int n_modes_lig) {
	try {
		std::ofstream f(path);
		const bool modes = n_modes_rec + n_modes_lig > 0;
		Common_Modes::numModesRec = n_modes_rec;
		Common_Modes::numModesLig = n_modes_lig;
		for (long i = 0; i < n; ++i) {
			if (!modes) {
				const float* r = results + 7 * i;
				Result_6D<float> e;
				e.E = r[0];
				e.pos.x = r[1]; e.pos.y = r[2]; e.pos.z = r[3];
				e.ang.x = r[4]; e.ang.y = r[5]; e.ang.z = r[6];
				f << e << std::endl;
			} else {
				const float* r = results + 27 * i;
				Result_6D_Modes<float> e;
				e._6D.E = r[0];
				e._6D.pos.x = r[1]; e._6D.pos.y = r[2]; e._6D.pos.z = r[3];
				e._6D.ang.x = r[4]; e._6D.ang.y = r[5]; e._6D.ang.z = r[6];
				for (int m = 0; m < 10; ++m) { e.modesRec[m] = r[7 + m]; e.modesLig[m] = r[17 + m]; }
				f << e << std::endl;
			}
		}
		return 0;
	} catch (std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

/* transformDOF_glob2rec<float> (src/model/DOFTransform.cpp:35-90) on n pairs
 * of {pos xyz, ang xyz} records, in place. */
int ref_glob2rec(float* rec, float* lig, long n, const float* pr, const float* pl, int crec, int clig) {
	std::vector<DOF_6D<float>> R(n), L(n);
	for (long i = 0; i < n; ++i) {
		R[i].pos = Vec3<float>(rec[6 * i], rec[6 * i + 1], rec[6 * i + 2]);
		R[i].ang = Vec3<float>(rec[6 * i + 3], rec[6 * i + 4], rec[6 * i + 5]);
		L[i].pos = Vec3<float>(lig[6 * i], lig[6 * i + 1], lig[6 * i + 2]);
		L[i].ang = Vec3<float>(lig[6 * i + 3], lig[6 * i + 4], lig[6 * i + 5]);
	}
	transformDOF_glob2rec(R, L, Vec3<float>(pr[0], pr[1], pr[2]), Vec3<float>(pl[0], pl[1], pl[2]), crec != 0,
			clig != 0);
	for (long i = 0; i < n; ++i) {
		rec[6 * i] = R[i].pos.x; rec[6 * i + 1] = R[i].pos.y; rec[6 * i + 2] = R[i].pos.z;
		rec[6 * i + 3] = R[i].ang.x; rec[6 * i + 4] = R[i].ang.y; rec[6 * i + 5] = R[i].ang.z;
		lig[6 * i] = L[i].pos.x; lig[6 * i + 1] = L[i].pos.y; lig[6 * i + 2] = L[i].pos.z;
		lig[6 * i + 3] = L[i].ang.x; lig[6 * i + 4] = L[i].ang.y; lig[6 * i + 5] = L[i].ang.z;
	}
	return 0;
}

/* Protein<float>::auto_pivotize (src/model/Protein.tpp:145-157). */
int ref_auto_pivot(const float* xyz, long n, float* pivot) {
	Protein<float> p;
	p.setNumAtoms((unsigned)n);
	std::memcpy(p.getOrCreatePosPtr(), xyz, sizeof(float) * 3 * n);
	p.auto_pivotize();
	pivot[0] = p.pivot().x;
	pivot[1] = p.pivot().y;
	pivot[2] = p.pivot().z;
	return 0;
}

/* readGridAlphabetFromFile + the ligand mapping of Configurator_6D::init
 * (src/service/Configurator_6D.tpp:49-54).  Returns the alphabet length. */
int ref_map_types(const char* alphabet_path, const uint32_t* types, long n, uint32_t* types_out,
		uint32_t* mapped_out, uint32_t* alphabet_out, int cap) {
	try {
		auto vec = readGridAlphabetFromFile(alphabet_path);
		for (size_t i = 0; i < vec.size() && (int)i < cap; ++i) alphabet_out[i] = vec[i];
		TypeMap map = createTypeMapFromVector(vec);
		std::vector<unsigned> t(types, types + n), m(n);
		applyDefaultMapping((unsigned)n, t.data(), t.data());
		applyMapping(map, (unsigned)n, t.data(), m.data());
		std::copy(t.begin(), t.end(), types_out);
		std::copy(m.begin(), m.end(), mapped_out);
		return (int)vec.size();
	} catch (std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

/* readGridFromGridFile<float> (src/fileIO/readFile.cpp:261-422): copies the
 * GridUnion's descriptors and arrays out.  caps in floats / entries. */
int ref_read_grid_file(const char* path, gba_intrpl_desc* inner, float* inner_data, long cap_inner,
		gba_intrpl_desc* outer, float* outer_data, long cap_outer, gba_nl_desc* nl, gba_neighbour_desc* nl_grid,
		long cap_nlgrid, uint32_t* nl_list, long cap_list, float* dplateau2) {
	try {
		auto G = createGridFromGridFile<float>(path);
		auto copy_intrpl = [](const IntrplGrid<float>& g, gba_intrpl_desc* d, float* data, long cap) {
			d->numGrids = g.numTypes();
			d->dimN[0] = g.dimN().x; d->dimN[1] = g.dimN().y; d->dimN[2] = g.dimN().z;
			d->gridSpacing = g.dVox();
			d->posMin[0] = g.pos().x; d->posMin[1] = g.pos().y; d->posMin[2] = g.pos().z;
			const long nv = (long)g.dimN().x * g.dimN().y * g.dimN().z;
			if (nv * 4 * (long)g.numTypes() <= cap)
				std::memcpy(data, g.getHostGridPtr(0), sizeof(float) * 4 * nv * g.numTypes());
		};
		copy_intrpl(*G->inner, inner, inner_data, cap_inner);
		copy_intrpl(*G->outer, outer, outer_data, cap_outer);
		const NLGrid<float>& L = *G->NL;
		nl->dimN[0] = L.dimN().x; nl->dimN[1] = L.dimN().y; nl->dimN[2] = L.dimN().z;
		nl->gridSpacing = L.dVox();
		nl->posMin[0] = L.pos().x; nl->posMin[1] = L.pos().y; nl->posMin[2] = L.pos().z;
		nl->numEl = L.neighborListSize();
		nl->dPlateau = 0.f;
		*dplateau2 = L.dPlateau2();
		const long nv = (long)L.dimN().x * L.dimN().y * L.dimN().z;
		if (nv <= cap_nlgrid)
			for (long v = 0; v < nv; ++v) {
				nl_grid[v].numEl = L.grid()[v].numEl;
				nl_grid[v].idx = L.grid()[v].idx;
			}
		if ((long)L.neighborListSize() <= cap_list)
			std::memcpy(nl_list, L.neighborList(), sizeof(uint32_t) * L.neighborListSize());
		return 0;
	} catch (std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

/* Fills an attract::Grid with every voxel populated (the in-memory form
 * ATTRACT's builder leaves: 1-based indices into the energy records and the
 * neighbour array) and writes it with the reference's Grid::write_std
 * (src/fileIO/grid_orig.cpp:303-484).  Inverse of readGridFromGridFile for
 * the channel order: channel c >= 1 holds type alphabet[c-1], channel 0 the
 * charge grid.  rec_xyz (SoA) sets the neighbour plateau flags as
 * gba_write_grid_file does. */
int ref_write_grid_file(const char* path, const gba_grid_file_info* info, const uint32_t* alphabet,
		const gba_intrpl_desc* in, const float* in_data, const gba_intrpl_desc* out, const float* out_data,
		const gba_nl_desc* nl, const gba_neighbour_desc* nl_grid, const uint32_t* nl_list, const float* rec_xyz) {
	try {
		const int K = MAXATOMTYPES;
		bool alpha[MAXATOMTYPES] = {false};
		std::vector<int> slot_channel(K, -1);
		for (unsigned c = 1; c < in->numGrids; ++c) {
			alpha[alphabet[c - 1] - 1] = true;
			slot_channel[alphabet[c - 1] - 1] = (int)c;
		}
		attract::Grid g;
		g.init(info->gridspacing, info->gridextension, info->plateaudis, info->neighbourdis, alpha);
		g.torquegrid = false;
		g.architecture = info->architecture;
		for (int a = 0; a < 3; ++a) {
			g.ori[a] = info->ori[a];
			g.pivot[a] = info->pivot[a];
		}
		g.gridx = info->inner_dim[0]; g.gridy = info->inner_dim[1]; g.gridz = info->inner_dim[2];
		g.gridx2 = info->outer_dim[0]; g.gridy2 = info->outer_dim[1]; g.gridz2 = info->outer_dim[2];
		g.natoms = info->natoms;
		const long C = in->numGrids;
		const long Ni = (long)g.gridx * g.gridy * g.gridz, No = (long)g.gridx2 * g.gridy2 * g.gridz2;
		g.nr_energrads = (int)((Ni + No) * C);
		g.shm_energrads = -1;
		g.shm_neighbours = -1;
		/* write_std reallocs and frees the records: malloc them */
		g.energrads_std = (attract::EnerGradStd*)std::calloc((size_t)g.nr_energrads, sizeof(attract::EnerGradStd));
		g.innergrid = new attract::Voxel[Ni];
		std::memset(g.innergrid, 0, sizeof(attract::Voxel) * Ni);
		g.biggrid = new attract::Potential[No];
		std::memset(g.biggrid, 0, sizeof(attract::Potential) * No);
		long rec_idx = 0;
		auto fill = [&](unsigned* pot, const float* data, long nvox, long v) {
			for (int slot = 0; slot <= K; ++slot) {
				if (slot < K && !alpha[slot]) continue;
				const int ch = slot == K ? 0 : slot_channel[slot];
				const float* d = data + ((size_t)ch * nvox + v) * 4;
				attract::EnerGradStd& e = g.energrads_std[rec_idx];
				e.energy = d[3];
				e.grad[0] = d[0]; e.grad[1] = d[1]; e.grad[2] = d[2];
				pot[slot] = (unsigned)(++rec_idx);
			}
		};
		for (long v = 0; v < Ni; ++v) fill(g.innergrid[v].potential, in_data, Ni, v);
		for (long v = 0; v < No; ++v) fill(g.biggrid[v], out_data, No, v);
		g.nr_neighbours = (int)nl->numEl;
		g.neighbours = new attract::Neighbour[nl->numEl > 0 ? nl->numEl : 1];
		std::memset(g.neighbours, 0, sizeof(attract::Neighbour) * (nl->numEl > 0 ? nl->numEl : 1));
		for (long v = 0; v < Ni; ++v) {
			const unsigned ne = nl_grid[v].numEl;
			g.innergrid[v].nr_neighbours = (short)ne;
			g.innergrid[v].neighbourlist = ne ? (int)nl_grid[v].idx + 1 : 0;
			const long x = v % g.gridx, y = (v / g.gridx) % g.gridy, z = v / ((long)g.gridx * g.gridy);
			const double cx = (double)nl->posMin[0] + x * (double)nl->gridSpacing;
			const double cy = (double)nl->posMin[1] + y * (double)nl->gridSpacing;
			const double cz = (double)nl->posMin[2] + z * (double)nl->gridSpacing;
			for (unsigned k = 0; k < ne; ++k) {
				attract::Neighbour& nb = g.neighbours[nl_grid[v].idx + k];
				const unsigned j = nl_list[nl_grid[v].idx + k];
				nb.index = j;
				nb.type = 2;
				if (rec_xyz) {
					const double dx = rec_xyz[j] - cx, dy = rec_xyz[info->natoms + j] - cy,
							dz = rec_xyz[2 * (size_t)info->natoms + j] - cz;
					nb.type = dx * dx + dy * dy + dz * dz < info->plateaudis * info->plateaudis ? 1 : 2;
				}
			}
		}
		g.write_std(path);
		return 0;
	} catch (std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

}  // extern "C"
