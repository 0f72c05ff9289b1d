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
 * (voxel lists cover every bead within cutoff of a ligand bead).  Like the
 * rigid kernel, a warp takes one pose and walks the flattened
 * (bead, neighbour) pairs of 64 staged ligand beads at a time.
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
#include <cub/cub.cuh>

#include "gba_context.h"
#include "rigid_pose.cuh"

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
	const float4* tab;     /* 3*T*T: per type pair the constants of lj86 (lj_table_kernel) */
	const float4* rq;      /* rec.n: receptor x, y, z and this call's charge (pack_receptor_kernel) */
	const uint32_t* tlist; /* the neighbour list with receptor types in bits 24..31, or nullptr */
	unsigned long long* next;   /* pose counter, zero at launch (PoseFeed) */
	const uint32_t* order;      /* visiting order (nearest ligands first), or nullptr */
};

namespace {

/* Per type pair (r0, eps, ipon), the constants of the 8-6 term and of its
 * derivatives, computed once per call: {rc, ac, emin, rmin2},
 * {-3 emin / rc, 4 emin / ac, 8 r0^7, 6 r0^5}, {r0^8, r0^6, eps, ipon}, with
 * rc = eps r0^8, ac = eps r0^6, emin = -27 ac^4 / (256 rc^3),
 * rmin2 = 4 rc / (3 ac) as readParamTableFromFile derives them
 * (src/fileIO/readFile.cpp:484-497).  The pair loop then divides nothing but
 * 1/r^2. */
__global__ void lj_table_kernel(uint32_t T2, const float* __restrict__ r0v, const float* __restrict__ epsv,
		const int32_t* __restrict__ ipon, float4* __restrict__ tab) {
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= T2) return;
	const float r0 = r0v[k], eps = epsv[k];
	const float r0_2 = r0 * r0, r0_6 = r0_2 * r0_2 * r0_2, r0_8 = r0_6 * r0_2;
	const float rc = eps * r0_8, ac = eps * r0_6;
	const bool ok = ac > 0.f && rc > 0.f;
	const float emin = ok ? -27.f * (ac * ac) * (ac * ac) / (256.f * rc * rc * rc) : 0.f;
	const float rmin2 = ok ? 4.f * rc / (3.f * ac) : 0.f;
	tab[3 * k] = make_float4(rc, ac, emin, rmin2);
	tab[3 * k + 1] = make_float4(ok ? -3.f * emin / rc : 0.f, ok ? 4.f * emin / ac : 0.f, 8.f * (r0_6 * r0),
			6.f * (r0_2 * r0_2 * r0));
	tab[3 * k + 2] = make_float4(r0_8, r0_6, eps, (float)ipon[k]);
}

/* Sort keys of the visiting order: the bits of |t|^2 for the pose's
 * translation t (non-negative floats order like their bit patterns; NaN
 * sorts last).  Ligands near the receptor's centre meet the most neighbour
 * pairs, so taking them first leaves cheap poses for the end of the launch. */
__global__ void near_first_keys_kernel(const gba_dof6d* __restrict__ dofs, uint32_t n, uint32_t* __restrict__ keys,
		uint32_t* __restrict__ idx) {
	const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= n) return;
	const float* d = reinterpret_cast<const float*>(dofs + p);
	const float x = __ldg(d), y = __ldg(d + 1), z = __ldg(d + 2);
	keys[p] = __float_as_uint(x * x + y * y + z * z);
	idx[p] = p;
}

/* Poses ordered nearest first (sorted on the top 16 bits of the key: the
 * exponent and 7 mantissa bits of |t|^2, about 0.4 % bins), scratch from S. */
const uint32_t* near_first_order(const gba_dof6d* dofs, size_t n, StreamScratch& S, cudaStream_t s) {
	cub::DoubleBuffer<uint32_t> kb(nullptr, nullptr), ib(nullptr, nullptr);
	size_t tmp = 0;
	check_cuda(cub::DeviceRadixSort::SortPairs(nullptr, tmp, kb, ib, (int)n, 16, 32, s), "pairwise order: size");
	const size_t a = (n * sizeof(uint32_t) + 255) & ~(size_t)255;
	char* base = (char*)S.get(4 * a + tmp, s);
	uint32_t* k0 = (uint32_t*)base;
	uint32_t* k1 = (uint32_t*)(base + a);
	uint32_t* i0 = (uint32_t*)(base + 2 * a);
	uint32_t* i1 = (uint32_t*)(base + 3 * a);
	near_first_keys_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dofs, (uint32_t)n, k0, i0);
	check_cuda(cudaGetLastError(), "pairwise order: keys");
	kb = cub::DoubleBuffer<uint32_t>(k0, k1);
	ib = cub::DoubleBuffer<uint32_t>(i0, i1);
	check_cuda(cub::DeviceRadixSort::SortPairs(base + 4 * a, tmp, kb, ib, (int)n, 16, 32, s),
			"pairwise order: sort");
	return ib.Current();
}

/* rq[j] = (x, y, z, q_rec[j]): a neighbour's position and charge in one
 * 16-byte gather (the receptor records are read in random order, so every
 * separate load is its own L1 wavefront). */
__global__ void pack_receptor_kernel(uint32_t n, const float4* __restrict__ xyzq, const float* __restrict__ q,
		float4* __restrict__ rq) {
	for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
		const float4 r = xyzq[j];
		rq[j] = make_float4(r.x, r.y, r.z, q[j]);
	}
}

/* LJ energy, radial force factor and d/d(r0, eps) of one 8-6 pair from the
 * type pair's table entry t. */
template <bool DERIV>
__device__ __forceinline__ void lj86(float r2, float ir2, const float4* __restrict__ t, float& e, float& fb,
		float& de_dr0, float& de_deps) {
	const float4 c = __ldg(t);
	const float4 k = DERIV ? __ldg(t + 1) : make_float4(0.f, 0.f, 0.f, 0.f);
	const float4 m = __ldg(t + 2);
	const float rc = c.x, ac = c.y, emin = c.z, rmin2 = c.w, iv = m.w;
	const float ir6 = ir2 * ir2 * ir2, ir8 = ir6 * ir2;
	const float vlj = rc * ir8 - ac * ir6;
	float de_drc = 0.f, de_dac = 0.f;
	fb = 6.f * vlj + 2.f * rc * ir8;     /* force factor: f = fb * d / r^2 */
	if (r2 < rmin2) {
		e = vlj + (iv - 1.f) * emin;
		if (DERIV) {
			de_drc = ir8 + (iv - 1.f) * k.x;
			de_dac = -ir6 + (iv - 1.f) * k.y;
		}
	} else {
		e = iv * vlj;
		fb *= iv;
		if (DERIV) {
			de_drc = iv * ir8;
			de_dac = -iv * ir6;
		}
	}
	/* rc = eps r0^8, ac = eps r0^6 */
	de_dr0 = DERIV ? m.z * (k.z * de_drc + k.w * de_dac) : 0.f;
	de_deps = DERIV ? m.x * de_drc + m.y * de_dac : 0.f;
}

/* Per-warp staging of the pairwise kernels: one round of 64 ligand beads. */
struct PairStage {
	float4 pq[kBeadsPerRound];       /* transformed x, y, z; charge */
	float4 ut[kBeadsPerRound];       /* unrotated x, y, z (torque lever); type (bits) */
	uint32_t lbase[kBeadsPerRound];  /* list start - first flattened pair of the slot */
	float gq[kBeadsPerRound];        /* backward: dE/dq of the slot's bead over this round */
	uint8_t own[64];                 /* PairWindow: slot of the bead starting at window position b */
};
constexpr int kPairwiseThreads = 256;
constexpr size_t kNearFirstMinPoses = 2048;

/* One warp per pose, the ligand in rounds of 64 beads like the rigid kernel:
 * lane-per-bead staging (transform, neighbour-list voxel), then the round's
 * flattened (bead, neighbour) pairs in windows of 64, two per lane, so that
 * uneven list lengths do not idle lanes.  A warp takes its next pose from a
 * global counter when it finishes one (PoseFeed). */
template <bool BACKWARD>
__global__ void __launch_bounds__(kPairwiseThreads) pairwise_kernel(const PairwiseLaunch L) {
	extern __shared__ double sm[];
	__shared__ PairStage stage[kPairwiseThreads / 32];
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
	PairStage& W = stage[threadIdx.x >> 5];
	const bool cdiel = L.dielec == GBA_DIELEC_CONSTANT;
	PoseFeed feed(L.next);
	for (size_t slot = feed.take(lane); slot < L.n; slot = feed.take(lane)) {
		const size_t p = L.order ? (size_t)__ldg(&L.order[slot]) : slot;
		const float* dofp = reinterpret_cast<const float*>(L.dofs + p);
		const float dv = lane < 6 ? __ldg(dofp + lane) : 0.f;
		float c[6];
#pragma unroll
		for (int k = 0; k < 6; ++k) c[k] = __shfl_sync(GBA_FULL_MASK, dv, k);
		const PoseRot R = pose_rotation(c[3], c[4], c[5], lane, DevTrig{nullptr, 0u, 0u});
		const float w = BACKWARD ? __ldg(&L.gE[p]) : 0.f;
		float sE = 0.f, sFx = 0.f, sFy = 0.f, sFz = 0.f;
		float Tq[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
		for (uint32_t i0 = 0; i0 < L.lig.n; i0 += kBeadsPerRound) {
			uint32_t nln[2];
#pragma unroll
			for (int h = 0; h < 2; ++h) {
				const int s = lane + 32 * h;
				const uint32_t i = i0 + s;
				nln[h] = 0;
				if (i < L.lig.n) {
					const float4 b = __ldg(&L.lig.xyzq[i]);
					const uint32_t tl = __ldg(&L.lig.tm[i]) & 0xffffu;
					if (tl != 0) {
						float px, py, pz;
						rot_apply(R.m, b.x, b.y, b.z, px, py, pz);
						px = fadd(px, c[0]); py = fadd(py, c[1]); pz = fadd(pz, c[2]);
						W.pq[s] = make_float4(px, py, pz, __ldg(&L.q_lig[i]));
						W.ut[s] = make_float4(b.x, b.y, b.z, __uint_as_float(tl));
						if (BACKWARD) W.gq[s] = 0.f;
						bool in_nl;
						nln[h] = stage_nl(L.nl, px, py, pz, s, W, in_nl);
					}
				}
			}
			uint32_t start[2];
			const uint32_t n_pair = queue_pairs(W, nln, lane, start);
			__syncwarp();
			PairWindow win;
			for (uint32_t w0 = 0; w0 < n_pair; w0 += 64) {
				uint32_t so[2];
				win.owners(W, w0, start, nln, lane, so[0], so[1]);
#pragma unroll
				for (int h = 0; h < 2; ++h) {
					const uint32_t q = w0 + 32 * h + lane;
					if (q >= n_pair) continue;
					const uint32_t s = so[h];
					const uint32_t ent = __ldg(&(L.tlist ? L.tlist : L.nl.list)[W.lbase[s] + q]);
					const uint32_t j = L.tlist ? ent & 0xffffffu : ent;
					const uint32_t tr = L.tlist ? ent >> 24 : __ldg(&L.rec.tm[j]) & 0xffffu;
					if (tr == 0) continue;
					const float4 r = __ldg(&L.rq[j]);
					const float4 b = W.pq[s];
					const float dx = b.x - r.x, dy = b.y - r.y, dz = b.z - r.z;
					const float r2 = dx * dx + dy * dy + dz * dz;
					if (!(r2 < L.cut2)) continue;
					const float4 u = W.ut[s];
					const uint32_t tl = __float_as_uint(u.w);
					const float ir2 = __frcp_rn(r2);      /* = 1.0f / r2, correctly rounded */
					const uint32_t tp = L.T * (tr - 1) + (tl - 1);
					float el, fb, dr0, deps;
					lj86<BACKWARD>(r2, ir2, L.tab + 3 * (size_t)tp, el, fb, dr0, deps);
					/* Coulomb, no |q q| switch: smooth in the charges */
					const float qi = b.w, qj = r.w;
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
					sE += el + qq * dd;
					if (BACKWARD) {
						const float ff = (fb + qq * fcf) * ir2;
						const float fx = ff * dx, fy = ff * dy, fz = ff * dz;
						sFx += fx; sFy += fy; sFz += fz;
						Tq[0] += u.x * fx; Tq[1] += u.y * fx; Tq[2] += u.z * fx;
						Tq[3] += u.x * fy; Tq[4] += u.y * fy; Tq[5] += u.z * fy;
						Tq[6] += u.x * fz; Tq[7] += u.y * fz; Tq[8] += u.z * fz;
						atomicAdd(&W.gq[s], L.ffelec * qj * dd);
						atomicAdd(&s_qr[j], (double)(w * (L.ffelec * qi * dd)));
						atomicAdd(&s_r0[tp], (double)(w * dr0));
						atomicAdd(&s_eps[tp], (double)(w * deps));
					}
				}
			}
			if (BACKWARD) {
				__syncwarp();
#pragma unroll
				for (int h = 0; h < 2; ++h) {
					const int s = lane + 32 * h;
					if (nln[h] && W.gq[s] != 0.f) atomicAdd(&s_ql[i0 + s], (double)(w * W.gq[s]));
				}
			}
			__syncwarp();
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
			L.tlist = ctx->typed_list(*G, rec, *R, true);
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
		/* per-call constants of the 8-6 term per type pair (r0, eps change per call) */
		const uint32_t T2 = L.T * L.T;
		StreamScratch scratch(ctx->scratch_pool);
		float4* tab = (float4*)scratch.get(3 * (size_t)std::max<uint32_t>(T2, 1) * sizeof(float4), s);
		L.next = (unsigned long long*)scratch.get(sizeof(unsigned long long), s);
		check_cuda(cudaMemsetAsync(L.next, 0, sizeof(unsigned long long), s), "pairwise: pose counter");
		/* a few poses per warp: the launch's end is set by its slowest poses */
		/* the sort takes an int item count: larger batches keep submission order */
		L.order = (n >= kNearFirstMinPoses && n <= 0x7fffffffu) ? near_first_order(dofs, n, scratch, s) : nullptr;
		if (T2 > 0) {
			lj_table_kernel<<<(T2 + 255) / 256, 256, 0, s>>>(T2, L.r0, L.eps, L.ipon, tab);
			check_cuda(cudaGetLastError(), "pairwise: parameter table");
		}
		L.tab = tab;
		float4* rq = (float4*)scratch.get((size_t)std::max<uint32_t>(L.rec.n, 1) * sizeof(float4), s);
		if (L.rec.n > 0) {
			pack_receptor_kernel<<<std::min<uint32_t>((L.rec.n + 255) / 256, 1024), 256, 0, s>>>(L.rec.n, L.rec.xyzq,
					L.q_rec, rq);
			check_cuda(cudaGetLastError(), "pairwise: receptor records");
		}
		L.rq = rq;
		const int threads = kPairwiseThreads;
		const size_t smem = backward ? sizeof(double) * (2 * (size_t)L.T * L.T + L.lig.n + L.rec.n) : 0;
		if (smem + sizeof(PairStage) * (kPairwiseThreads / 32) > 200 * 1024)
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
