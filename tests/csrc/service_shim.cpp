/* Runs the GB300 energy services through the request interface (Server,
 * work items, pinned server buffers) for the GPU tests; plain C entry points
 * for ctypes. */
#include <cstring>
#include <memory>
#include <string>

#include "../../gpuattract_2.0_gb300/host/gb300_service.h"

using namespace gba::host;

static void put_error(const std::string& e, char* err, int cap) {
	if (err && cap > 0) {
		std::strncpy(err, e.c_str(), cap - 1);
		err[cap - 1] = 0;
	}
}

extern "C" int run_service_6d(void* ctx, uint32_t rec, uint32_t lig, uint32_t grid, uint32_t params,
		const void* dofs, size_t n, int workers, int item_size, void* out, char* err, int cap) {
	try {
		auto svc = std::make_shared<GB300EnergyService6D>((gba_ctx*)ctx);
		Server<Types_6D> server(svc);
		server.createWorkers(workers);
		server.setItemSize(item_size);
		server.setWaitTime(600000);
		Common c{grid, lig, rec, params, params};
		Server<Types_6D>::request_t req((gba_dof6d*)dofs, n, c);
		server.submit(req);
		server.wait(req, (gba_result6d*)out);
	} catch (std::exception& e) {
		put_error(e.what(), err, cap);
		return 1;
	}
	return 0;
}

extern "C" int run_service_6d_modes(void* ctx, uint32_t rec, uint32_t lig, uint32_t grid_rec,
		uint32_t grid_lig, uint32_t params, const void* dofs, size_t n, int workers, int item_size,
		void* out, char* err, int cap) {
	try {
		auto svc = std::make_shared<GB300EnergyService6DModes>((gba_ctx*)ctx);
		Server<Types_6D_Modes> server(svc);
		server.createWorkers(workers);
		server.setItemSize(item_size);
		server.setWaitTime(600000);
		Common_Modes c{grid_rec, grid_lig, lig, rec, params, params};
		Server<Types_6D_Modes>::request_t req((gba_dof6d_modes*)dofs, n, c);
		server.submit(req);
		server.wait(req, (gba_result6d_modes*)out);
	} catch (std::exception& e) {
		put_error(e.what(), err, cap);
		return 1;
	}
	return 0;
}
