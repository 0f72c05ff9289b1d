/*
 * host_sincos.cu -- gba_set_host_sincos: the host C library's sinf/cosf as a
 * device table.
 *
 * The reference takes each Euler angle's sine and cosine from the C library
 * (euler2rotmat, euler2torquemat: src/model/matrixFunctions.h:40-127, with
 * float angles, i.e. sinf/cosf).  The last bit of those values is the
 * library's choice: glibc's misround about 1 % of arguments by one ulp,
 * while the kernels compute the correctly rounded value.  In a deep clash or
 * along a minimization trajectory one ulp of the rotation shows in the
 * result, so a bit-for-bit reproduction of the reference on a given host
 * needs that host's own values.  This call evaluates the library's sinf and
 * cosf for every float angle whose magnitude lies in [2^-12, max_abs) --
 * both signs, on all host threads -- and keeps them on the device, 8 bytes
 * per angle (2.4 GB for max_abs = 64); the kernels read an angle's pair from
 * it instead of computing one.  Below 2^-12 the correctly rounded values are
 * sin a = a and cos a = 1, which a faithful library returns too; angles at
 * or beyond max_abs keep the computed value.
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "gba_context.h"

namespace gba {

namespace {

uint32_t float_bits(float f) {
	uint32_t b;
	std::memcpy(&b, &f, 4);
	return b;
}

float bits_float(uint32_t b) {
	float f;
	std::memcpy(&f, &b, 4);
	return f;
}

/* Called through pointers so that the compiler neither folds nor merges the
 * two calls: the values are the library's, as the reference receives them. */
float (*volatile g_sinf)(float) = ::sinf;
float (*volatile g_cosf)(float) = ::cosf;

}  // namespace

}  // namespace gba

using namespace gba;

extern "C" int gba_set_host_sincos(gba_ctx* ctx, float max_abs) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	try {
		if (!(max_abs == 0.0f || (max_abs > 0.0f && max_abs <= 4096.0f)))
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_set_host_sincos: max_abs must be 0 or in (0, 4096]");
		ctx->bind();
		Lock g(ctx->stage_mu);
		/* cached device models and minimizer graphs hold the old table */
		ctx->model_cache.clear();
		ctx->clear_graphs();
		ctx->trig = DevTrig{nullptr, 0u, 0u};
		ctx->trig_table.release();
		const uint32_t lo = float_bits(0x1p-12f), hi = float_bits(max_abs);
		if (max_abs == 0.0f || hi <= lo) return GBA_OK;
		const size_t half = hi - lo, n = 2 * half;
		ctx->trig_table.alloc(n * sizeof(float2));
		try {
			const unsigned nthreads = std::max(1u, std::thread::hardware_concurrency());
			const size_t chunk = (size_t)1 << 24;   /* entries per host pass: 128 MB */
			std::vector<float2> buf(std::min(chunk, n));
			for (size_t c0 = 0; c0 < n; c0 += chunk) {
				const size_t m = std::min(chunk, n - c0);
				const auto fill = [&](unsigned t) {
					for (size_t k = m * t / nthreads; k < m * (t + 1) / nthreads; ++k) {
						const size_t e = c0 + k;
						const uint32_t b = (e >= half ? 0x80000000u : 0u) | (uint32_t)(lo + e % half);
						const float a = bits_float(b);
						buf[k] = make_float2(g_sinf(a), g_cosf(a));
					}
				};
				/* slices 1.. on threads (as many as start), slice 0 and any
				 * slice whose thread could not start on this one */
				std::vector<std::thread> pool;
				std::vector<unsigned> here{0u};
				/* reserved before the first thread starts: a vector that grew
				 * (and failed to) under running threads would end the process */
				pool.reserve(nthreads);
				here.reserve(nthreads);
				for (unsigned t = 1; t < nthreads; ++t) {
					try {
						pool.emplace_back(fill, t);
					} catch (const std::system_error&) {
						here.push_back(t);
					}
				}
				for (unsigned t : here) fill(t);
				for (auto& th : pool) th.join();
				check_cuda(cudaMemcpy((float2*)ctx->trig_table.ptr + c0, buf.data(), m * sizeof(float2),
						cudaMemcpyHostToDevice), "gba_set_host_sincos: upload");
			}
		} catch (...) {
			ctx->trig_table.release();
			throw;
		}
		ctx->trig = DevTrig{(const float2*)ctx->trig_table.ptr, lo, hi};
	} catch (const ApiError& e) {
		ctx->set_error(e.what());
		return e.code;
	} catch (const std::bad_alloc&) {
		ctx->set_error("gba_set_host_sincos: host allocation failed");
		return GBA_ERR_OUT_OF_MEMORY;
	} catch (const std::exception& e) {
		ctx->set_error(e.what());
		return GBA_ERR_INVALID_ARGUMENT;
	}
	return GBA_OK;
}
