/*
 * gridbuild.cu -- builds a receptor's inner/outer potential grids and its
 * neighbour-list grid on the device.
 *
 * The reference only reads ATTRACT grid files (src/fileIO/readFile.cpp:261-422;
 * the builder attract::Grid::calculate_std is declared at
 * src/fileIO/grid_orig.h:143 and defined nowhere).  This builder produces the
 * same in-memory layout with these semantics:
 *   channel c >= 1 (ligand type alphabet[c-1]) and the charge channel 0 hold,
 *   at each voxel centre p, the sum over receptor beads j (type != 0) of the
 *   ATTRACT pair force/energy evaluated at max(|p - x_j|, plateau) along the
 *   direction p - x_j (LJPotForce / ChargePotForce, src/model/forcefield.h),
 *   so that grid + NL(r) - NL(plateau) is the exact pair term inside the
 *   plateau (src/model/neighborlist.h:104-157);
 *   voxel v's neighbour list holds, in increasing index, every receptor bead
 *   (type != 0) with |p_v - x_j|^2 <= nl_cutoff^2, tested in double with
 *   unfused operations so the lists are bit-identical to the CPU builder.
 * Arithmetic of the potentials (the CPU builder performs the same operations
 * in the same order, so both produce the same bits): the voxel centre in
 * double, unfused, rounded to float; per bead the separation, its square,
 * the plateau rescaling (plateau / sqrt(r^2)) and 1/r^2 in IEEE-rounded FP32
 * (no approximate reciprocal or square root, nothing contracted); the pair
 * terms of energy_dev.cuh; FP32 partial sums over each block of 256
 * consecutive receptor beads, in bead order; those partials added in double,
 * block after block; the total rounded to float.
 * Layout: inner box = bead bounding box + margin, spacing d; outer grid
 * spacing 2d, extended by outer_ext inner voxels per side; NL grid = inner.
 */
#include <algorithm>
#include <cmath>
#include <vector>

#include "energy_dev.cuh"
#include "gba_context.h"

namespace gba {

namespace {

constexpr int kTile = 256;
constexpr int kGroup = 4;   /* channels per thread */

struct BuildArgs {
	const float4* xyzq;      /* receptor beads */
	const uint32_t* tm;      /* type | mapped << 16 */
	uint32_t n;
	DevParams par;
	const uint32_t* alphabet;  /* device copy, n_alphabet entries */
	uint32_t n_alphabet;
	float plateau, plat2;
	double cut2;
};

__global__ void __launch_bounds__(kTile) grid_potential_kernel(BuildArgs a, gba_intrpl_desc d,
		float4* __restrict__ out) {
	__shared__ float4 sb[kTile];
	__shared__ uint32_t stype[kTile];
	const uint32_t Nx = d.dimN[0], Ny = d.dimN[1], Nz = d.dimN[2];
	const uint32_t N = Nx * Ny * Nz;
	const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
	const bool valid = v < N;
	const uint32_t x = valid ? v % Nx : 0, y = valid ? (v / Nx) % Ny : 0, z = valid ? v / (Nx * Ny) : 0;
	const double sp = (double)d.gridSpacing;
	const float px = (float)__dadd_rn((double)d.posMin[0], __dmul_rn((double)x, sp));
	const float py = (float)__dadd_rn((double)d.posMin[1], __dmul_rn((double)y, sp));
	const float pz = (float)__dadd_rn((double)d.posMin[2], __dmul_rn((double)z, sp));
	const uint32_t c0 = blockIdx.y * kGroup;
	const uint32_t C = a.n_alphabet + 1;
	const bool shape86 = a.par.potshape == GBA_POTSHAPE_8_6;
	const bool cdiel = a.par.dielec == GBA_DIELEC_CONSTANT;
	double acc[kGroup][4];
#pragma unroll
	for (int g = 0; g < kGroup; ++g) acc[g][0] = acc[g][1] = acc[g][2] = acc[g][3] = 0.0;
	uint32_t tl[kGroup];
#pragma unroll
	for (int g = 0; g < kGroup; ++g) {
		const uint32_t c = c0 + g;
		tl[g] = (c >= 1 && c < C) ? __ldg(&a.alphabet[c - 1]) : 0u;
	}
	for (uint32_t t0 = 0; t0 < a.n; t0 += kTile) {
		const uint32_t j = t0 + threadIdx.x;
		if (j < a.n) {
			sb[threadIdx.x] = __ldg(&a.xyzq[j]);
			stype[threadIdx.x] = __ldg(&a.tm[j]) & 0xffffu;
		}
		__syncthreads();
		const uint32_t tn = min((uint32_t)kTile, a.n - t0);
		float tacc[kGroup][4];
#pragma unroll
		for (int g = 0; g < kGroup; ++g) tacc[g][0] = tacc[g][1] = tacc[g][2] = tacc[g][3] = 0.f;
		for (uint32_t b = 0; b < tn; ++b) {
			const uint32_t tr = stype[b];
			if (tr == 0) continue;
			const float4 r = sb[b];
			float ex = fsub(px, r.x), ey = fsub(py, r.y), ez = fsub(pz, r.z);
			float e2 = fadd(fadd(fmul(ex, ex), fmul(ey, ey)), fmul(ez, ez));
			bool dirless = false;
			if (e2 < a.plat2) {
				if (e2 > 0.f) {
					const float sc = __fdiv_rn(a.plateau, __fsqrt_rn(e2));
					ex = fmul(ex, sc); ey = fmul(ey, sc); ez = fmul(ez, sc);
				} else {
					dirless = true;
				}
				e2 = a.plat2;
			}
			const float rr2 = __fdiv_rn(1.0f, e2);
			const float ux = dirless ? 0.f : fmul(ex, rr2), uy = dirless ? 0.f : fmul(ey, rr2),
					uz = dirless ? 0.f : fmul(ez, rr2);
#pragma unroll
			for (int g = 0; g < kGroup; ++g) {
				const uint32_t c = c0 + g;
				float fx, fy, fz, e;
				if (c == 0) {
					const float qf = fmul(r.w, a.par.ffelec);
					if (!(fabsf(qf) > 0.001f)) continue;
					charge_pot_force(rr2, ux, uy, uz, qf, cdiel, fx, fy, fz, e);
				} else {
					if (tl[g] == 0 || tl[g] > a.par.num_types || tr > a.par.num_types) continue;
					const size_t k = (size_t)a.par.num_types * (tr - 1) + (tl[g] - 1);
					lj_pot_force(e2, rr2, ux, uy, uz, __ldg(&a.par.lj[k]), __ldg(&a.par.ivor[k]),
							shape86, fx, fy, fz, e);
				}
				tacc[g][0] = fadd(tacc[g][0], fx);
				tacc[g][1] = fadd(tacc[g][1], fy);
				tacc[g][2] = fadd(tacc[g][2], fz);
				tacc[g][3] = fadd(tacc[g][3], e);
			}
		}
#pragma unroll
		for (int g = 0; g < kGroup; ++g)
#pragma unroll
			for (int k = 0; k < 4; ++k) acc[g][k] = __dadd_rn(acc[g][k], (double)tacc[g][k]);
		__syncthreads();
	}
	if (!valid) return;
#pragma unroll
	for (int g = 0; g < kGroup; ++g) {
		const uint32_t c = c0 + g;
		if (c < C)
			out[(size_t)c * N + v] = make_float4((float)acc[g][0], (float)acc[g][1],
					(float)acc[g][2], (float)acc[g][3]);
	}
}

/* Neighbour membership, unfused double arithmetic (bit-identical to the CPU builder). */
__device__ __forceinline__ bool nl_member(double px, double py, double pz, float4 r, double cut2) {
	const double dx = __dsub_rn(px, (double)r.x);
	const double dy = __dsub_rn(py, (double)r.y);
	const double dz = __dsub_rn(pz, (double)r.z);
	const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
	return d2 <= cut2;
}

template <bool FILL>
__global__ void __launch_bounds__(kTile) nl_kernel(BuildArgs a, gba_nl_desc d,
		uint32_t* __restrict__ count, const uint32_t* __restrict__ offset,
		uint32_t* __restrict__ list) {
	__shared__ float4 sb[kTile];
	__shared__ uint32_t stype[kTile];
	const uint32_t Nx = d.dimN[0], Ny = d.dimN[1], Nz = d.dimN[2];
	const uint32_t N = Nx * Ny * Nz;
	const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
	const bool valid = v < N;
	const uint32_t x = valid ? v % Nx : 0, y = valid ? (v / Nx) % Ny : 0, z = valid ? v / (Nx * Ny) : 0;
	const double px = __dadd_rn((double)d.posMin[0], __dmul_rn((double)x, (double)d.gridSpacing));
	const double py = __dadd_rn((double)d.posMin[1], __dmul_rn((double)y, (double)d.gridSpacing));
	const double pz = __dadd_rn((double)d.posMin[2], __dmul_rn((double)z, (double)d.gridSpacing));
	uint32_t cnt = 0;
	const uint32_t base = (FILL && valid) ? offset[v] : 0;
	for (uint32_t t0 = 0; t0 < a.n; t0 += kTile) {
		const uint32_t j = t0 + threadIdx.x;
		if (j < a.n) {
			sb[threadIdx.x] = __ldg(&a.xyzq[j]);
			stype[threadIdx.x] = __ldg(&a.tm[j]) & 0xffffu;
		}
		__syncthreads();
		const uint32_t tn = min((uint32_t)kTile, a.n - t0);
		if (valid)
			for (uint32_t b = 0; b < tn; ++b) {
				if (stype[b] == 0) continue;
				if (nl_member(px, py, pz, sb[b], a.cut2)) {
					if (FILL) list[base + cnt] = t0 + b;
					++cnt;
				}
			}
		__syncthreads();
	}
	if (valid && !FILL) count[v] = cnt;
}

/* Layout as the CPU builder (double arithmetic, same formulas). */
void grid_layout(const std::vector<float>& xyz, uint32_t n, const gba_grid_build_opts& o,
		gba_intrpl_desc& inner, gba_intrpl_desc& outer, gba_nl_desc& nl) {
	const double s = o.spacing;
	inner.numGrids = outer.numGrids = o.n_alphabet + 1;
	for (int a = 0; a < 3; ++a) {
		const float* P = xyz.data() + (size_t)a * n;
		double lo = P[0], hi = P[0];
		for (uint32_t i = 1; i < n; ++i) { lo = std::min(lo, (double)P[i]); hi = std::max(hi, (double)P[i]); }
		lo -= o.margin;
		hi += o.margin;
		unsigned N = (unsigned)std::ceil((hi - lo) / s) + 1;
		inner.dimN[a] = N;
		inner.posMin[a] = (float)lo;
		/* ATTRACT stores the float inner origin and derives the outer one from
		 * it (readGridFromGridFile, src/fileIO/readFile.cpp:322-324) */
		outer.posMin[a] = (float)((double)inner.posMin[a] - o.outer_ext * s);
		outer.dimN[a] = (unsigned)std::ceil(((N - 1) * s + 2.0 * o.outer_ext * s) / (2 * s)) + 1;
		nl.dimN[a] = N;
		nl.posMin[a] = inner.posMin[a];
	}
	inner.gridSpacing = o.spacing;
	outer.gridSpacing = 2 * o.spacing;
	nl.gridSpacing = o.spacing;
	nl.dPlateau = o.plateau;
	nl.numEl = 0;
}

/* Exclusive prefix sum on the host side of a device array (setup path). */
uint64_t exclusive_scan(const DevBuffer& counts, DevBuffer& offsets, size_t nv, cudaStream_t s) {
	std::vector<uint32_t> h(nv);
	check_cuda(cudaMemcpyAsync(h.data(), counts.ptr, nv * sizeof(uint32_t), cudaMemcpyDeviceToHost, s),
			"grid build: counts D2H");
	check_cuda(cudaStreamSynchronize(s), "grid build: sync");
	uint64_t run = 0;
	for (size_t v = 0; v < nv; ++v) {
		const uint32_t c = h[v];
		if (run > 0xffffffffull) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "neighbour list exceeds 2^32 entries");
		h[v] = (uint32_t)run;
		run += c;
	}
	offsets.upload(h.data(), nv * sizeof(uint32_t));
	return run;
}

}  // namespace

}  // namespace gba

using namespace gba;

extern "C" int gba_build_grid(gba_ctx* ctx, gba_id rec, gba_id params,
		const gba_grid_build_opts* opt, gba_id* out) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	try {
		if (!opt || !out) throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_build_grid: null argument");
		if (!(opt->spacing > 0) || !(opt->plateau > 0) || !(opt->nl_cutoff > 0) || opt->n_alphabet > 98 ||
				opt->margin < 0)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_build_grid: bad options");
		ctx->bind();
		ProteinItem* R;
		ParamsItem* P;
		{
			Lock g(ctx->mu);
			R = static_cast<ProteinItem*>(ctx->find(rec, ItemKind::Protein));
			P = static_cast<ParamsItem*>(ctx->find(params, ItemKind::Params));
		}
		if (R->max_type > P->dev.num_types)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_build_grid: receptor type exceeds the table");
		for (uint32_t c = 0; c < opt->n_alphabet; ++c)
			if (opt->alphabet[c] > P->dev.num_types)
				throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_build_grid: alphabet type exceeds the table");
		auto item = std::make_unique<GridItem>();
		grid_layout(R->host_xyz, R->dev.n, *opt, item->inner_desc, item->outer_desc, item->nl_desc);
		const size_t Ni = (size_t)item->inner_desc.dimN[0] * item->inner_desc.dimN[1] * item->inner_desc.dimN[2];
		const size_t No = (size_t)item->outer_desc.dimN[0] * item->outer_desc.dimN[1] * item->outer_desc.dimN[2];
		const uint32_t C = opt->n_alphabet + 1;
		if ((double)C * std::max(Ni, No) > 4.0e9)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_build_grid: grid exceeds 2^32 float4");
		item->inner.alloc(Ni * C * sizeof(float4));
		item->outer.alloc(No * C * sizeof(float4));
		DevBuffer alpha;
		alpha.upload(opt->alphabet, std::max<size_t>(1, opt->n_alphabet) * sizeof(uint32_t));
		BuildArgs a{};
		a.xyzq = R->dev.xyzq;
		a.tm = R->dev.tm;
		a.n = R->dev.n;
		a.par = P->dev;
		a.alphabet = (const uint32_t*)alpha.ptr;
		a.n_alphabet = opt->n_alphabet;
		a.plateau = opt->plateau;
		a.plat2 = opt->plateau * opt->plateau;
		a.cut2 = (double)opt->nl_cutoff * opt->nl_cutoff;
		cudaStream_t s = 0;
		const unsigned groups = (C + kGroup - 1) / kGroup;
		grid_potential_kernel<<<dim3((unsigned)((Ni + kTile - 1) / kTile), groups), kTile, 0, s>>>(
				a, item->inner_desc, (float4*)item->inner.ptr);
		check_cuda(cudaGetLastError(), "grid build: inner launch");
		grid_potential_kernel<<<dim3((unsigned)((No + kTile - 1) / kTile), groups), kTile, 0, s>>>(
				a, item->outer_desc, (float4*)item->outer.ptr);
		check_cuda(cudaGetLastError(), "grid build: outer launch");
		DevBuffer counts, offsets;
		counts.alloc(Ni * sizeof(uint32_t));
		const unsigned nb = (unsigned)((Ni + kTile - 1) / kTile);
		nl_kernel<false><<<nb, kTile, 0, s>>>(a, item->nl_desc, (uint32_t*)counts.ptr, nullptr, nullptr);
		check_cuda(cudaGetLastError(), "grid build: NL count launch");
		const uint64_t total = exclusive_scan(counts, offsets, Ni, s);
		item->nllist.alloc(std::max<uint64_t>(1, total) * sizeof(uint32_t));
		nl_kernel<true><<<nb, kTile, 0, s>>>(a, item->nl_desc, (uint32_t*)counts.ptr,
				(const uint32_t*)offsets.ptr, (uint32_t*)item->nllist.ptr);
		check_cuda(cudaGetLastError(), "grid build: NL fill launch");
		/* descriptors {numEl, idx} */
		std::vector<uint32_t> hc(Ni), ho(Ni);
		check_cuda(cudaMemcpy(hc.data(), counts.ptr, Ni * 4, cudaMemcpyDeviceToHost), "grid build: D2H");
		check_cuda(cudaMemcpy(ho.data(), offsets.ptr, Ni * 4, cudaMemcpyDeviceToHost), "grid build: D2H");
		std::vector<uint2> desc(Ni);
		for (size_t v = 0; v < Ni; ++v) desc[v] = make_uint2(hc[v], ho[v]);
		item->nlgrid.upload(desc.data(), Ni * sizeof(uint2));
		item->nl_desc.numEl = (uint32_t)total;
		item->dev.inner = intrpl_from_desc(item->inner_desc);
		item->dev.inner.data = (const float4*)item->inner.ptr;
		item->dev.outer = intrpl_from_desc(item->outer_desc);
		item->dev.outer.data = (const float4*)item->outer.ptr;
		item->dev.nl = nl_from_desc(item->nl_desc);
		std::vector<float> ratio = nl_ratio_table(item->dev.nl.dPlateau2);
		item->ratio.upload(ratio.data(), ratio.size() * sizeof(float));
		item->dev.nl.grid = (const uint2*)item->nlgrid.ptr;
		item->dev.nl.list = (const uint32_t*)item->nllist.ptr;
		item->dev.nl.ratio = (const float*)item->ratio.ptr;
		item->nl_max_index = R->dev.n - 1;
		item->nl_has_entries = total > 0;
		item->nl_list_radius = opt->nl_cutoff;
		check_cuda(cudaDeviceSynchronize(), "grid build");
		*out = ctx->add(std::move(item));
	} catch (const ApiError& e) {
		ctx->set_error(e.what());
		return e.code;
	} catch (const std::exception& e) {
		ctx->set_error(e.what());
		return GBA_ERR_INVALID_ARGUMENT;
	}
	return GBA_OK;
}

extern "C" int gba_grid_info(gba_ctx* ctx, gba_id grid, gba_intrpl_desc* inner,
		gba_intrpl_desc* outer, gba_nl_desc* nl) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	try {
		Lock g(ctx->mu);
		auto* G = static_cast<GridItem*>(ctx->find(grid, ItemKind::Grid));
		if (inner) *inner = G->inner_desc;
		if (outer) *outer = G->outer_desc;
		if (nl) *nl = G->nl_desc;
	} catch (const ApiError& e) {
		ctx->set_error(e.what());
		return e.code;
	}
	return GBA_OK;
}

extern "C" int gba_download_grid(gba_ctx* ctx, gba_id grid, float* inner, float* outer,
		gba_neighbour_desc* nl_grid, uint32_t* nl_list) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	try {
		ctx->bind();
		GridItem* G;
		{
			Lock g(ctx->mu);
			G = static_cast<GridItem*>(ctx->find(grid, ItemKind::Grid));
		}
		if (inner) check_cuda(cudaMemcpy(inner, G->inner.ptr, G->inner.bytes, cudaMemcpyDeviceToHost), "D2H");
		if (outer) check_cuda(cudaMemcpy(outer, G->outer.ptr, G->outer.bytes, cudaMemcpyDeviceToHost), "D2H");
		if (nl_grid) check_cuda(cudaMemcpy(nl_grid, G->nlgrid.ptr, G->nlgrid.bytes, cudaMemcpyDeviceToHost), "D2H");
		if (nl_list && G->nl_desc.numEl)
			check_cuda(cudaMemcpy(nl_list, G->nllist.ptr, (size_t)G->nl_desc.numEl * 4, cudaMemcpyDeviceToHost), "D2H");
	} catch (const ApiError& e) {
		ctx->set_error(e.what());
		return e.code;
	}
	return GBA_OK;
}

/* ---- duplicated-octet layout ---------------------------------------------- */

namespace gba {
namespace {

__global__ void build_octets_kernel(const float4* __restrict__ src, uint32_t Nx, uint32_t Ny,
		uint32_t Nz, uint32_t C, float4* __restrict__ dst) {
	const size_t nocts = (size_t)(Nx - 1) * (Ny - 1) * (Nz - 1);
	const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= nocts * C) return;
	const size_t c = t / nocts, o = t % nocts;
	const uint32_t x = (uint32_t)(o % (Nx - 1));
	const uint32_t y = (uint32_t)((o / (Nx - 1)) % (Ny - 1));
	const uint32_t z = (uint32_t)(o / ((size_t)(Nx - 1) * (Ny - 1)));
	const size_t sxy = (size_t)Nx * Ny;
	const float4* b = src + c * sxy * Nz + (size_t)Nx * ((size_t)z * Ny + y) + x;
	float4* d = dst + 8 * t;
	d[0] = b[0];
	d[1] = b[1];
	d[2] = b[Nx];
	d[3] = b[Nx + 1];
	d[4] = b[sxy];
	d[5] = b[sxy + 1];
	d[6] = b[sxy + Nx];
	d[7] = b[sxy + Nx + 1];
}

void make_octets(const gba_intrpl_desc& d, const DevBuffer& src, DevBuffer& dst) {
	const size_t nocts = (size_t)(d.dimN[0] - 1) * (d.dimN[1] - 1) * (d.dimN[2] - 1);
	const size_t total = nocts * d.numGrids;
	dst.alloc(total * 8 * sizeof(float4));
	build_octets_kernel<<<(unsigned)((total + 255) / 256), 256>>>((const float4*)src.ptr, d.dimN[0],
			d.dimN[1], d.dimN[2], d.numGrids, (float4*)dst.ptr);
	check_cuda(cudaGetLastError(), "octet layout");
}

}  // namespace
}  // namespace gba

extern "C" int gba_grid_octets(gba_ctx* ctx, gba_id grid, int enable) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	try {
		ctx->bind();
		Lock lk(ctx->stage_mu);
		Lock g(ctx->mu);
		auto* G = static_cast<GridItem*>(ctx->find(grid, ItemKind::Grid));
		if (enable) {
			if (!G->inner_oct.ptr) make_octets(G->inner_desc, G->inner, G->inner_oct);
			if (!G->outer_oct.ptr) make_octets(G->outer_desc, G->outer, G->outer_oct);
			check_cuda(cudaDeviceSynchronize(), "octet layout");
		} else {
			G->inner_oct.release();
			G->outer_oct.release();
		}
		G->dev.inner.oct = (const float4*)G->inner_oct.ptr;
		G->dev.outer.oct = (const float4*)G->outer_oct.ptr;
		/* cached device copies of the pair descriptors hold the old pointers */
		ctx->model_cache.clear();
		ctx->clear_graphs();
	} catch (const ApiError& e) {
		ctx->set_error(e.what());
		return e.code;
	} catch (const std::exception& e) {
		ctx->set_error(e.what());
		return GBA_ERR_INVALID_ARGUMENT;
	}
	return GBA_OK;
}
