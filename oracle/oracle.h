/*
 * oracle.h -- CPU oracle of the gpuATTRACT 2.0 docking energy/gradient path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a restatement of the reference's CPU
 * algorithm used as the checker for the CUDA library; only the test suite,
 * the smoke check and the bench's CPU-baseline leg may load it.  The product
 * library never links or calls it.
 *
 * Parity pin: the FP32 path is checked bit-for-bit against the reference's own
 * CPUEnergyService6D<float> (compiled from its sources into oracle/_ref by
 * oracle/build_ref.sh) on the committed golden cases in tests/golden/.
 */
#ifndef ATTRACT_ORACLE_H_
#define ATTRACT_ORACLE_H_

#include <stddef.h>
#include <stdint.h>
#include "../include/gbattract.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
	uint32_t n;
	const float* xyz;          /* 3n, SoA, pivotized */
	const uint32_t* type;      /* raw type after default map (0 = dummy) */
	const uint32_t* mapped;    /* channel in the partner's grid (0 = none) */
	const float* charge;
	uint32_t n_modes;
	const float* modes;        /* 3*n*n_modes, x[i*M+m] then y then z */
	const float* mode_force;   /* n_modes */
} orc_protein;

typedef struct {
	gba_intrpl_desc inner; const float* inner_data;
	gba_intrpl_desc outer; const float* outer_data;
	gba_nl_desc nl; const gba_neighbour_desc* nl_grid; const uint32_t* nl_list;
} orc_grid;

typedef struct {
	uint32_t num_types;
	const gba_ffparam* table;
	int potshape;
	int dielec;
	float ffelec;
} orc_params;

/* Per-pose bookkeeping used for tolerances and for the roofline byte count. */
typedef struct {
	uint32_t n_grid;        /* beads interpolated in the inner or outer grid */
	uint32_t n_grid_charged;/* ... of which also read the charge channel */
	uint32_t n_nl;          /* beads that looked up an NL voxel */
	uint32_t n_nl_entries;  /* sum of numEl over those voxels */
	uint32_t n_pairs;       /* neighbour pairs inside the plateau */
	uint32_t n_rec_lookups; /* modes: channel lookups of the receptor beads in the
	                           ligand grid (type + charge channels; 0 when rigid) */
	double abs_E;           /* sum of |energy term| over every term */
	double abs_F;           /* sum of |force term| (Euclidean) over every term */
	double abs_T;           /* sum over beads of |x_i| * |f_i| */
	uint32_t n_force_lim;   /* times the ForceLim clamp scaled the force sum (0..3) */
	uint32_t pad;
} orc_pose_stats;

/* Rigid energy+gradient, FP32 exactly as CPUEnergyService6D<float>.
 * stats may be NULL.  nthreads <= 0 means all hardware threads. */
int orc_energy_6d(const orc_protein* rec, const orc_protein* lig, const orc_grid* grid,
		const orc_params* par, const gba_dof6d* dofs, size_t n, gba_result6d* out,
		orc_pose_stats* stats, int nthreads);

/* Same formulas in FP64 throughout (including trilinear weights); out7 holds
 * E, pos xyz, ang xyz per pose. */
int orc_energy_6d_f64(const orc_protein* rec, const orc_protein* lig, const orc_grid* grid,
		const orc_params* par, const gba_dof6d* dofs, size_t n, double* out7, int nthreads);

/* Normal-mode variant, FP32 as CPUEnergyService6DModes<float>. */
int orc_energy_6d_modes(const orc_protein* rec, const orc_protein* lig,
		const orc_grid* grid_rec, const orc_grid* grid_lig, const orc_params* par,
		const gba_dof6d_modes* dofs, size_t n, gba_result6d_modes* out,
		orc_pose_stats* stats, int nthreads);

/* The normal-mode variant in FP64 throughout; out27 holds the
 * Result_6D_Modes fields as doubles per pose. */
int orc_energy_6d_modes_f64(const orc_protein* rec, const orc_protein* lig,
		const orc_grid* grid_rec, const orc_grid* grid_lig, const orc_params* par,
		const gba_dof6d_modes* dofs, size_t n, double* out27, int nthreads);

/* VA13 (minfor.f + mc11a.f) driving orc_energy_6d for each pose, one pose
 * per thread.  Reports, per pose, the last evaluated state and objective
 * (what RequestHandler::getResultStates/getResultEnGrads return) and the
 * number of energy evaluations. */
int orc_minimize_6d(const orc_protein* rec, const orc_protein* lig, const orc_grid* grid,
		const orc_params* par, const gba_dof6d* start, size_t n, int max_fun_eval,
		gba_dof6d* out_state, gba_result6d* out_result, int32_t* out_nevals, int nthreads);

/* Same minimizer on the normal-mode energy, DOF vector
 * (ang xyz, pos xyz, modesRec[0..Mr), modesLig[0..Ml)). */
int orc_minimize_6d_modes(const orc_protein* rec, const orc_protein* lig,
		const orc_grid* grid_rec, const orc_grid* grid_lig, const orc_params* par,
		const gba_dof6d_modes* start, size_t n, int max_fun_eval,
		gba_dof6d_modes* out_state, gba_result6d_modes* out_result, int32_t* out_nevals,
		int nthreads);

/* ---- grid builder (CPU, FP64 accumulation) ------------------------------- */

typedef struct {
	float spacing;        /* inner voxel size, 0.9 A */
	float plateau;        /* NL plateau distance, 10 A */
	float nl_cutoff;      /* neighbour-list radius around a voxel centre, 10.8 A */
	float margin;         /* inner box = bead bounding box + margin */
	uint32_t outer_ext;   /* outer extension in inner voxels per side (32) */
	uint32_t n_alphabet;  /* ligand types that get a channel */
	uint32_t alphabet[99]; /* raw ligand type served by channel c+1 */
} orc_grid_opts;

/* Computes descriptors only (sizes), so the caller can allocate. */
int orc_grid_layout(const orc_protein* rec, const orc_grid_opts* opt,
		gba_intrpl_desc* inner, gba_intrpl_desc* outer, gba_nl_desc* nl);

/* Fills the potential grids (inner_data, outer_data: numGrids*N float4) and
 * the neighbour grid; the list is written to nl_list (capacity nl_cap) and
 * nl->numEl set.  Returns GBA_ERR_INVALID_ARGUMENT if nl_cap is too small
 * (nl->numEl then holds the size needed). */
int orc_grid_build(const orc_protein* rec, const orc_params* par, const orc_grid_opts* opt,
		const gba_intrpl_desc* inner, float* inner_data,
		const gba_intrpl_desc* outer, float* outer_data,
		gba_nl_desc* nl, gba_neighbour_desc* nl_grid, uint32_t* nl_list, size_t nl_cap,
		int nthreads);

/* Where the FP32 restatement takes sin/cos from: 0 (default) the C
 * library's sinf/cosf, as the reference; 1 the correctly rounded values
 * (float)sin((double)x) -- what the library's kernels compute.  Global to the
 * process; set it while no oracle call runs. */
void orc_set_exact_sincos(int exact);

/* The neighbour-list part of orc_grid_build alone (nl as orc_grid_layout
 * wrote it; same capacity rule). */
int orc_grid_nl(const orc_protein* rec, const orc_grid_opts* opt, gba_nl_desc* nl,
		gba_neighbour_desc* nl_grid, uint32_t* nl_list, size_t nl_cap, int nthreads);

/* The potentials of orc_grid_build at `count` voxels (linear indices into
 * the grid d): out[i] = numGrids float4, channel-major. */
int orc_grid_voxels(const orc_protein* rec, const orc_params* par, const orc_grid_opts* opt,
		const gba_intrpl_desc* d, const uint64_t* voxels, size_t count, float* out, int nthreads);

/* ---- pairwise (grid-free) path for the adjoint checks --------------------- */

/* Pairwise (grid-free) energy in FP64 with optional analytic dE/dDOF; see
 * attract_oracle.cpp.  dofs6 / ref_dofs6: (pos xyz, ang xyz) per pose. */
int orc_pairwise_energy_f64(const orc_protein* rec, const orc_protein* lig,
		const double* q_rec, const double* q_lig, uint32_t num_types,
		const double* r0, const double* eps, const int32_t* ipon, int dielec, double ffelec,
		double cutoff, const double* dofs6, const double* ref_dofs6, size_t n, double* out_E,
		double* out_grad);

/* minfor on the extended Rosenbrock function; records each evaluated point
 * and f (test of the library's VA13 state machine). */
int orc_minfor_trace(int n, const double* x0, int ivmax, double* trace, int cap);
/* The same with evaluation nan_eval (0-based; -1: none) returning a NaN
 * gradient component. */
int orc_minfor_trace_nan(int n, const double* x0, int ivmax, double* trace, int cap, int nan_eval);

#ifdef __cplusplus
}
#endif

#endif
