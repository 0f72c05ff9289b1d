/*
 * gba_internal.h -- device-side data layout of libgbattract.
 *
 * Everything the fused kernels read lives in plain device buffers laid out for
 * one-instruction loads:
 *   protein  : float4 {x, y, z, q} per bead + uint32 {type | mapped << 16}
 *              + modes per bead [i][m][axis] (3M contiguous floats), so a
 *              neighbour gather reads one short contiguous record
 *   grids    : the reference's channel-major float4 layout (channel 0 =
 *              charge), one buffer per inner/outer grid; derived constants
 *              (maxDim, 1/dVox, 1/voxelVol) precomputed on the host exactly as
 *              IntrplGrid's constructor does (src/model/IntrplGrid.tpp:29-41)
 *   NL grid  : uint2 {numEl, idx} per voxel + uint32 list + the sqrt-ratio
 *              table of src/model/NLGrid.tpp:45-50 (bit-identical)
 *   params   : float4 {rc, ac, rmin2, emin} + float ipon per type pair
 */
#ifndef GBA_INTERNAL_H_
#define GBA_INTERNAL_H_

#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/gbattract.h"

namespace gba {

struct DevProtein {
	uint32_t n;
	uint32_t n_modes;
	const float4* xyzq;       /* n */
	const uint32_t* tm;       /* n: type | mapped << 16 */
	const float* modes;       /* n * mode_stride(n_modes), [i][m][axis] */
	float mode_force[GBA_MODES_MAX];
};

/* Floats per bead of a device mode array: 3 per mode, padded to whole
 * float4s so that a bead's vectors load as 16-byte words. */
constexpr uint32_t mode_stride(uint32_t n_modes) { return (3 * n_modes + 3) & ~3u; }

struct DevIntrpl {
	uint32_t dimN[3];
	uint32_t numGrids;
	float pos[3];
	float maxDim[3];
	float dVox, dVox_inv, voxelVol_inv;
	const float4* data;       /* numGrids * Nx*Ny*Nz */
	/* optional duplicated-octet copy: per channel and voxel (x<Nx-1, y<Ny-1,
	 * z<Nz-1) the 8 corners d000 d100 d010 d110 d001 d101 d011 d111 in one
	 * 128-byte record, so a lookup reads exactly one aligned L2 line */
	const float4* oct;        /* numGrids * (Nx-1)(Ny-1)(Nz-1) * 8, or nullptr */
};

struct DevNL {
	uint32_t dimN[3];
	uint32_t ratio_size;      /* entries in ratio[] */
	float pos[3];
	float maxDim[3];
	float dVox_inv;
	float dPlateau2, dPlateau2_inv;
	const uint2* grid;        /* Nx*Ny*Nz {numEl, idx} */
	const uint32_t* list;
	const float* ratio;
	/* ratio_computed: the plateau ratio of table bin n is evaluated as
	 * sqrt((n + 0.5) * ratio_scale), ratio_scale = 1e-4 / plateau^2 (within
	 * one ulp of the table entry), instead of being read from ratio[] */
	float ratio_scale;
	int ratio_computed;
	/* plateau below 50 A: the pair term may use the hardware reciprocal */
	int approx_inv;
	/* optional: list[] with the receptor bead's type in bits 24..31 (set per
	 * launch for one receptor; nullptr: the type is gathered per pair) */
	const uint32_t* typed_list;
};

struct DevGrid {
	DevIntrpl inner, outer;
	DevNL nl;
	/* 8 lanes per grid lookup, one octet corner each (needs both octet copies) */
	int coop_lookup;
};

struct DevParams {
	uint32_t num_types;
	int potshape;             /* GBA_POTSHAPE_* */
	int dielec;               /* GBA_DIELEC_* */
	float ffelec;
	const float4* lj;         /* T*T {rc, ac, rmin2, emin} */
	const float* ivor;        /* T*T ipon as float */
	/* T*T pairs of float4 {rc, ac, rmin2, emin}, {ipon, fb_p, e_p, 0}: fb_p and
	 * e_p are LJPotForce's force factor and energy at the plateau distance of
	 * the grid in use, per type pair (set per launch); entry
	 * (ligand type - 1) * T + (receptor type - 1), so the entries one ligand
	 * bead meets lie in one row */
	const float4* pair;
};

/* Per-pose census used for the roofline byte count (same meaning as the
 * oracle's orc_pose_stats counters). */
struct PoseCensus {
	uint32_t n_grid, n_grid_charged, n_nl, n_nl_entries;
};

/* The host C library's sinf/cosf, tabulated (gba_set_host_sincos): entry
 * (sign(a) ? hi - lo : 0) + (|a| bits - lo) holds (sinf(a), cosf(a)) for
 * every float angle a with |a| bits in [lo, hi).  sc == nullptr: off. */
struct DevTrig {
	const float2* sc;
	uint32_t lo, hi;
};

/* ---- launch wrappers (energy_rigid.cu) ----------------------------------- */

/* Everything one rigid receptor-ligand pair's evaluation reads. */
struct RigidModel {
	DevProtein rec, lig;
	DevGrid grid;
	DevParams par;
	DevTrig trig;
};

struct RigidLaunch {
	RigidModel m;
	const gba_dof6d* dofs;
	gba_result6d* out;
	PoseCensus* census;       /* nullptr: no census */
	const uint32_t* order;    /* visiting order (nullptr: submission order) */
	size_t n;
	int bound4;               /* launch the four-blocks-per-SM instantiation */
	int roundwise;            /* the minimizers' round-wise summation order (plain form) */
	int ref_order;            /* the reference CPU path's summation order (GBA_KOPT_REFERENCE_ORDER;
	                             takes precedence over roundwise and bound4, not over census) */
	unsigned long long* next; /* pose counter, zero at launch (PoseFeed); nullptr: fixed stride */
};

cudaError_t launch_rigid_energy(const RigidLaunch& L, int blocks, int threads, cudaStream_t s);

/* ---- persistent minimizer (minimize.cu) ---------------------------------- */

/* Without a caller deadline, no warp of a minimizer kernel runs longer than
 * this (it stops with GBA_ERR_TIMEOUT): every device loop has a bound. */
constexpr unsigned long long kMinimizeHardCapNs = 600ull * 1000000000ull;

struct MinLaunch {
	const RigidModel* models;       /* device array, one per pair */
	const uint32_t* pair_of;        /* per pose pair index; nullptr = pair 0 */
	const uint32_t* order;          /* queue slot -> pose (nullptr: identity) */
	const gba_dof6d* start;
	gba_dof6d* out_state;           /* last evaluated DOF */
	gba_result6d* out_result;       /* last evaluated Result */
	int32_t* out_nevals;            /* energy evaluations (may be nullptr) */
	size_t n;
	int max_evals;
	int chunk;                      /* poses claimed per queue grab */
	unsigned long long* counter;    /* work-queue cursor, zeroed before launch */
	int* status;                    /* GBA_OK or GBA_ERR_TIMEOUT */
	unsigned long long budget_ns;   /* per-warp wall-time budget, 0 = none */
	unsigned long long* t0;         /* earliest warp start (atomicMin), set to ~0 before launch */
	unsigned long long* done_ns;    /* per pose completion time (globaltimer), may be nullptr */
	int ref_order;                  /* GBA_KOPT_REFERENCE_ORDER: the reference's summation order */
};

cudaError_t launch_minimize_rigid(const MinLaunch& L, int blocks, int threads, cudaStream_t s);
int minimize_blocks_per_sm(int threads, bool ref_order = false);
/* the team form: `team` (1..kMaxTeam) warps split each pose's ligand rounds,
 * plus a control warp running VA13; two poses per block; same results bit
 * for bit */
constexpr int kMaxTeam = 7;
cudaError_t launch_minimize_rigid_team(const MinLaunch& L, int blocks, int team, cudaStream_t s);
int minimize_team_blocks_per_sm(int team, bool ref_order = false);
/* the solo form: a block of `team` warps per pose (no control warp: warp 0
 * steps VA13 after each evaluation), for jobs whose poses all fit resident;
 * same results bit for bit */
cudaError_t launch_minimize_rigid_solo(const MinLaunch& L, int blocks, int team, cudaStream_t s);
int minimize_solo_blocks_per_sm(int team, bool ref_order = false);

/* multi-pair scoring: one launch over the poses of many pairs */
struct BatchEnergyLaunch {
	const RigidModel* models;
	const uint32_t* pair_of;
	const gba_dof6d* dofs;
	gba_result6d* out;
	size_t n;
	unsigned long long* next; /* pose counter, zero at launch (PoseFeed); nullptr: fixed stride */
	int ref_order;            /* GBA_KOPT_REFERENCE_ORDER */
};

cudaError_t launch_batch_energy(const BatchEnergyLaunch& L, int blocks, int threads, cudaStream_t s);

/* ---- normal-mode variant (energy_modes.cu) ------------------------------- */

struct ModesLaunch {
	DevProtein rec, lig;
	DevGrid grid_rec;         /* receptor grid: ligand beads + NL */
	DevGrid grid_lig;         /* ligand grid: receptor beads */
	DevParams par;
	DevTrig trig;
	const float* rec_modes;   /* [i][m][axis] */
	uint32_t rec_ms;          /* floats per receptor bead record (mode_stride(Mr)) */
	const float* lig_modes;
	uint32_t lig_ms;
	const gba_dof6d_modes* dofs;
	gba_result6d_modes* out;
	size_t n;
	unsigned long long* next; /* pose counters, zero at launch (PoseFeed): receptor pass, */
	unsigned long long* next2;/* ligand pass; nullptr: fixed stride */
	int ref_order;            /* GBA_KOPT_REFERENCE_ORDER: the reference CPU path's order */
	float4* ref_rf;           /* with ref_order: rec.n float4 per launched warp (modes_ref_warps) */
};

/* the two scoring kernels (receptor pass, then ligand pass), each grid sized
 * to its own occupancy on num_sms SMs */
cudaError_t launch_modes_energy(const ModesLaunch& L, int num_sms, cudaStream_t s);
/* warps the reference-order scoring launch uses for L (its scratch: that many
 * times rec.n float4) */
size_t modes_ref_warps(const ModesLaunch& L, int num_sms);

struct ModesMinLaunch {
	ModesLaunch m;                  /* model fields; dofs/out/n unused */
	const gba_dof6d_modes* start;
	gba_dof6d_modes* out_state;
	gba_result6d_modes* out_result;
	int32_t* out_nevals;
	size_t n;
	int max_evals;
	unsigned long long* counter;    /* zeroed before launch */
	int* status;                    /* GBA_OK, set to TIMEOUT / DEVICE_CHECK by the kernel */
};

cudaError_t launch_minimize_modes(const ModesMinLaunch& M, int blocks, int threads, cudaStream_t s);
int minimize_modes_blocks_per_sm(int threads, const ModesLaunch& L);

/* Number of resident blocks per SM of the rigid kernel for `threads`. */
int rigid_blocks_per_sm(int threads, bool census, bool bound4 = false, bool roundwise = false,
		bool ref_order = false);

}  // namespace gba

#endif
