/*
 * adjoint.cu -- pairwise (grid-free) docking energy and its adjoint.
 *
 * The pairwise path scores a pose with the exact ATTRACT pair terms over
 * every receptor-ligand pair closer than `cutoff`:
 *   8-6 Lennard-Jones of LJPotForce (src/model/forcefield.h:30-83) with
 *   rc = eps r0^8, ac = eps r0^6, emin = -27 ac^4 / (256 rc^3),
 *   rmin2 = 4 rc / (3 ac) as readParamTableFromFile derives them
 *   (src/fileIO/readFile.cpp:484-497), and the distance-dependent Coulomb
 *   term of ChargePotForce (src/model/forcefield.h:87-146),
 * with per-bead charges and per-type-pair (r0, eps) as free parameters.
 * Candidate receptor beads come from the receptor's neighbour-list grid
 * (voxel lists cover every bead within cutoff of a ligand bead).
 *
 * The backward kernel recomputes the transformed coordinates and pair terms
 * (nothing is stored by the forward) and produces, scaled by the upstream
 * gradient of each pose's energy:
 *   dE/dDOF   (pos xyz, ang xyz): -(force sum), -(TorqueMat . torque), the
 *             reference's gradient convention (src/apps/em/meta.h:114-121)
 *   dE/dq     per ligand and per receptor bead
 *   dE/dr0, dE/deps per type pair [rec type - 1][lig type - 1]
 * Parameter gradients accumulate in FP64 shared-memory partials per block and
 * are flushed with FP64 global atomics.
 */
#include "energy_dev.cuh"
#include "gba_context.h"

namespace gba {

struct PairwiseLaunch {
	DevProtein rec, lig;
	DevNL nl;
	uint32_t T;
	const float* r0;       /* T*T */
	const float* eps;      /* T*T */
	const int32_t* ipon;   /* T*T */
	const float* q_lig;
	const float* q_rec;
	int dielec;
	float ffelec;
	float cut2;
	const gba_dof6d* dofs;
	size_t n;
	float* E;              /* forward output (n) */
	const float* gE;       /* backward input (n) */
	float* g_dofs;         /* n*6 (pos, ang) */
	double* g_qlig;        /* lig.n */
	double* g_qrec;        /* rec.n */
	double* g_r0;          /* T*T */
	double* g_eps;         /* T*T */
};

namespace {

/* LJ energy, radial force factor and d/d(r0, eps) of one 8-6 pair. */
__device__ __forceinline__ void lj86(float r2, float ir2, float r0, float eps, int ipon, float& e,
		float& fb, float& de_dr0, float& de_deps) {
	const float r0_2 = r0 * r0, r0_6 = r0_2 * r0_2 * r0_2, r0_8 = r0_6 * r0_2;
	const float rc = eps * r0_8, ac = eps * r0_6;
	const float ir6 = ir2 * ir2 * ir2, ir8 = ir6 * ir2;
	const float vlj = rc * ir8 - ac * ir6;
	const float emin = (ac > 0.f && rc > 0.f) ? -27.f * (ac * ac) * (ac * ac) / (256.f * rc * rc * rc) : 0.f;
	const float rmin2 = (ac > 0.f && rc > 0.f) ? 4.f * rc / (3.f * ac) : 0.f;
	const float iv = (float)ipon;
	float de_drc, de_dac;
	fb = 6.f * vlj + 2.f * rc * ir8;     /* force factor: f = fb * d / r^2 */
	if (r2 < rmin2) {
		e = vlj + (iv - 1.f) * emin;
		de_drc = ir8 + (iv - 1.f) * (-3.f * emin / rc);
		de_dac = -ir6 + (iv - 1.f) * (4.f * emin / ac);
	} else {
		e = iv * vlj;
		fb *= iv;
		de_drc = iv * ir8;
		de_dac = -iv * ir6;
	}
	/* rc = eps r0^8, ac = eps r0^6 */
	de_dr0 = eps * (8.f * (r0_6 * r0) * de_drc + 6.f * (r0_2 * r0_2 * r0) * de_dac);
	de_deps = r0_8 * de_drc + r0_6 * de_dac;
}

template <bool BACKWARD>
__global__ void __launch_bounds__(256) pairwise_kernel(const PairwiseLaunch L) {
	extern __shared__ double sm[];
	const uint32_t T2 = L.T * L.T;
	double* s_r0 = sm;
	double* s_eps = sm + T2;
	double* s_ql = sm + 2 * T2;
	double* s_qr = sm + 2 * T2 + L.lig.n;
	if (BACKWARD) {
		const uint32_t tot = 2 * T2 + L.lig.n + L.rec.n;
		for (uint32_t k = threadIdx.x; k < tot; k += blockDim.x) sm[k] = 0.0;
		__syncthreads();
	}
	const int lane = threadIdx.x & 31;
	const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
	const bool cdiel = L.dielec == GBA_DIELEC_CONSTANT;
	for (size_t p = warp; p < L.n; p += nwarps) {
		const float* dofp = reinterpret_cast<const float*>(L.dofs + p);
		const float dv = lane < 6 ? __ldg(dofp + lane) : 0.f;
		float c[6];
#pragma unroll
		for (int k = 0; k < 6; ++k) c[k] = __shfl_sync(GBA_FULL_MASK, dv, k);
		const PoseRot R = pose_rotation(c[3], c[4], c[5], lane);
		const float w = BACKWARD ? __ldg(&L.gE[p]) : 0.f;
		float sE = 0.f, sFx = 0.f, sFy = 0.f, sFz = 0.f;
		float Tq[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
		for (uint32_t i = lane; i < L.lig.n; i += 32) {
			const float4 b = __ldg(&L.lig.xyzq[i]);
			const uint32_t tl = __ldg(&L.lig.tm[i]) & 0xffffu;
			if (tl == 0) continue;
			float px, py, pz;
			rot_apply(R.m, b.x, b.y, b.z, px, py, pz);
			px = fadd(px, c[0]); py = fadd(py, c[1]); pz = fadd(pz, c[2]);
			if (nl_out(L.nl, px, py, pz)) continue;
			const int ix = min(max((int)roundf(fmul(fsub(px, L.nl.pos[0]), L.nl.dVox_inv)), 0), (int)L.nl.dimN[0] - 1);
			const int iy = min(max((int)roundf(fmul(fsub(py, L.nl.pos[1]), L.nl.dVox_inv)), 0), (int)L.nl.dimN[1] - 1);
			const int iz = min(max((int)roundf(fmul(fsub(pz, L.nl.pos[2]), L.nl.dVox_inv)), 0), (int)L.nl.dimN[2] - 1);
			const uint2 d = __ldg(&L.nl.grid[L.nl.dimN[0] * (iz * L.nl.dimN[1] + iy) + ix]);
			const float qi = __ldg(&L.q_lig[i]);
			float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f, gqi = 0.f;
			for (uint32_t k = 0; k < d.x; ++k) {
				const uint32_t j = __ldg(&L.nl.list[d.y + k]);
				const uint32_t tr = __ldg(&L.rec.tm[j]) & 0xffffu;
				if (tr == 0) continue;
				const float4 r = __ldg(&L.rec.xyzq[j]);
				const float dx = px - r.x, dy = py - r.y, dz = pz - r.z;
				const float r2 = dx * dx + dy * dy + dz * dz;
				if (!(r2 < L.cut2)) continue;
				const float ir2 = 1.0f / r2;
				const uint32_t tp = L.T * (tr - 1) + (tl - 1);
				float el, fb, dr0, deps;
				lj86(r2, ir2, __ldg(&L.r0[tp]), __ldg(&L.eps[tp]), __ldg(&L.ipon[tp]), el, fb, dr0, deps);
				/* Coulomb, no |q q| switch: smooth in the charges */
				const float qj = __ldg(&L.q_rec[j]);
				float dd, fcf;
				if (cdiel) {
					const float ir = sqrtf(ir2);
					dd = ir - 0.02f;
					fcf = dd > 0.f ? ir : 0.f;      /* f = ffelec qq (1/r) d / r^2 */
				} else {
					dd = ir2 - 4.0e-4f;
					fcf = dd > 0.f ? 2.f * ir2 : 0.f;  /* f = ffelec qq 2/r^2 d / r^2 */
				}
				dd = fmaxf(dd, 0.f);
				const float qq = L.ffelec * qi * qj;
				e += el + qq * dd;
				const float ff = (fb + qq * fcf) * ir2;
				fx += ff * dx; fy += ff * dy; fz += ff * dz;
				if (BACKWARD) {
					gqi += L.ffelec * qj * dd;
					atomicAdd(&s_qr[j], (double)(w * (L.ffelec * qi * dd)));
					atomicAdd(&s_r0[tp], (double)(w * dr0));
					atomicAdd(&s_eps[tp], (double)(w * deps));
				}
			}
			if (BACKWARD && gqi != 0.f) atomicAdd(&s_ql[i], (double)(w * gqi));
			sE += e; sFx += fx; sFy += fy; sFz += fz;
			Tq[0] += b.x * fx; Tq[1] += b.y * fx; Tq[2] += b.z * fx;
			Tq[3] += b.x * fy; Tq[4] += b.y * fy; Tq[5] += b.z * fy;
			Tq[6] += b.x * fz; Tq[7] += b.y * fz; Tq[8] += b.z * fz;
		}
		if (!BACKWARD) {
			sE = warp_sum(sE);
			if (lane == 0) L.E[p] = sE;
		} else {
			sFx = warp_sum(sFx); sFy = warp_sum(sFy); sFz = warp_sum(sFz);
#pragma unroll
			for (int k = 0; k < 9; ++k) Tq[k] = warp_sum(Tq[k]);
			float ang[3];
			torque_reduce(R, Tq, ang);
			/* dE/dDOF = -(force, Euler torque), DOF_6D order (pos, ang) */
			const float g[6] = {-w * sFx, -w * sFy, -w * sFz, -w * ang[0], -w * ang[1], -w * ang[2]};
			float v = 0.f;
#pragma unroll
			for (int k = 0; k < 6; ++k) v = lane == k ? g[k] : v;
			if (lane < 6) L.g_dofs[6 * p + lane] = v;
		}
	}
	if (BACKWARD) {
		__syncthreads();
		for (uint32_t k = threadIdx.x; k < T2; k += blockDim.x) {
			if (s_r0[k] != 0.0) atomicAdd(&L.g_r0[k], s_r0[k]);
			if (s_eps[k] != 0.0) atomicAdd(&L.g_eps[k], s_eps[k]);
		}
		for (uint32_t k = threadIdx.x; k < L.lig.n; k += blockDim.x)
			if (s_ql[k] != 0.0) atomicAdd(&L.g_qlig[k], s_ql[k]);
		for (uint32_t k = threadIdx.x; k < L.rec.n; k += blockDim.x)
			if (s_qr[k] != 0.0) atomicAdd(&L.g_qrec[k], s_qr[k]);
	}
}

}  // namespace

}  // namespace gba

using namespace gba;

extern "C" int gba_pairwise_6d(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid,
		const gba_pairwise_params* pp, const gba_dof6d* dofs, size_t n, float* E_out,
		const float* gE, float* g_dofs, double* g_qlig, double* g_qrec, double* g_r0,
		double* g_eps, void* stream) {
	if (!ctx) return GBA_ERR_INVALID_ARGUMENT;
	try {
		if (!pp || !pp->r0 || !pp->eps || !pp->ipon || !pp->q_lig || !pp->q_rec)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_pairwise_6d: null parameter array");
		if (n == 0) return GBA_OK;
		const bool backward = gE != nullptr;
		if (!dofs || (!backward && !E_out) ||
				(backward && (!g_dofs || !g_qlig || !g_qrec || !g_r0 || !g_eps)))
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_pairwise_6d: null pose/output pointer");
		for (const void* ptr : {(const void*)dofs, (const void*)pp->r0, (const void*)pp->eps,
					(const void*)pp->ipon, (const void*)pp->q_lig, (const void*)pp->q_rec})
			if (!is_device_pointer(ptr))
				throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_pairwise_6d: device pointers required");
		if (pp->potshape != GBA_POTSHAPE_8_6)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_pairwise_6d: only the 8-6 shape is differentiable here");
		ctx->bind();
		PairwiseLaunch L{};
		{
			Lock g(ctx->mu);
			auto* R = static_cast<ProteinItem*>(ctx->find(rec, ItemKind::Protein));
			auto* Lg = static_cast<ProteinItem*>(ctx->find(lig, ItemKind::Protein));
			auto* G = static_cast<GridItem*>(ctx->find(grid, ItemKind::Grid));
			if (R->max_type > pp->num_types || Lg->max_type > pp->num_types)
				throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_pairwise_6d: bead type exceeds num_types");
			if (G->nl_has_entries && G->nl_max_index >= R->dev.n)
				throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_pairwise_6d: neighbour list indexes beyond the receptor");
			/* the voxel lists must cover every pair within the cutoff */
			const double reach = (double)pp->cutoff + 0.5 * std::sqrt(3.0) * G->nl_desc.gridSpacing;
			if (!(pp->cutoff > 0) || reach > G->nl_list_radius + 1e-6)
				throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_pairwise_6d: cutoff exceeds what the neighbour grid covers");
			L.rec = R->dev;
			L.lig = Lg->dev;
			L.nl = G->dev.nl;
		}
		L.T = pp->num_types;
		L.r0 = pp->r0;
		L.eps = pp->eps;
		L.ipon = pp->ipon;
		L.q_lig = pp->q_lig;
		L.q_rec = pp->q_rec;
		L.dielec = pp->dielec;
		L.ffelec = pp->ffelec;
		L.cut2 = pp->cutoff * pp->cutoff;
		L.dofs = dofs;
		L.n = n;
		L.E = E_out;
		L.gE = gE;
		L.g_dofs = g_dofs;
		L.g_qlig = g_qlig;
		L.g_qrec = g_qrec;
		L.g_r0 = g_r0;
		L.g_eps = g_eps;
		cudaStream_t s = (cudaStream_t)stream;
		const int threads = 256;
		const size_t smem = backward ? sizeof(double) * (2 * (size_t)L.T * L.T + L.lig.n + L.rec.n) : 0;
		if (smem > 200 * 1024)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "gba_pairwise_6d: proteins/types too large for the adjoint's shared partials");
		size_t blocks;
		if (backward) {
			check_cuda(cudaFuncSetAttribute(pairwise_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
					(int)smem), "adjoint smem");
			int nb = 0;
			cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pairwise_kernel<true>, threads, smem);
			blocks = std::max<size_t>(1, std::min<size_t>((n + 7) / 8, (size_t)ctx->num_sms * std::max(nb, 1)));
			pairwise_kernel<true><<<(unsigned)blocks, threads, smem, s>>>(L);
		} else {
			int nb = 0;
			cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pairwise_kernel<false>, threads, 0);
			blocks = std::max<size_t>(1, std::min<size_t>((n + 7) / 8, (size_t)ctx->num_sms * std::max(nb, 1)));
			pairwise_kernel<false><<<(unsigned)blocks, threads, 0, s>>>(L);
		}
		check_cuda(cudaGetLastError(), "pairwise launch");
	} catch (const ApiError& e) {
		ctx->set_error(e.what());
		return e.code;
	} catch (const std::exception& e) {
		ctx->set_error(e.what());
		return GBA_ERR_INVALID_ARGUMENT;
	}
	return GBA_OK;
}
