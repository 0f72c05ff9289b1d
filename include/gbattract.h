/*
 * gbattract.h -- C ABI of the GB300 docking energy/gradient library (libgbattract).
 *
 * This library replaces the energy backend of gpuATTRACT 2.0 behind its
 * Service/Server request interface.  Every entry point returns an int status
 * (GBA_OK == 0) and never throws or exits; gba_last_error() gives the message.
 * All structs below are plain FP32/uint32 PODs laid out bit-for-bit like the
 * reference's own types, so a WorkItem's input/result slices pass through
 * without conversion.
 *
 * Reference interfaces each declaration stands in for are cited as
 * path:line inside the gpuATTRACT 2.0 source tree.
 */
#ifndef GBATTRACT_H_
#define GBATTRACT_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* MODES_MAX_NUMBER, src/model/Types_6D_Config.h:11 */
#define GBA_MODES_MAX 10

/* ---- status codes ------------------------------------------------------- */
#define GBA_OK                   0
#define GBA_ERR_INVALID_ARGUMENT 1  /* std::invalid_argument in the reference */
#define GBA_ERR_UNKNOWN_ID       2  /* DataManager::get on a missing id, src/server/DataManager.cpp:23-50 */
#define GBA_ERR_CUDA             3  /* CUDA_CHECK -> std::runtime_error, src/commons/macros.h:62-72 */
#define GBA_ERR_OUT_OF_MEMORY    4
#define GBA_ERR_TIMEOUT          5  /* a device-side wait/iteration budget ran out */
#define GBA_ERR_NO_DEVICE        6
#define GBA_ERR_DEVICE_CHECK     7  /* a device-side bounds check recorded a bad index */

typedef struct gba_ctx gba_ctx;
typedef uint32_t gba_id;      /* id of a device-resident data item (protein, grid, table) */

/* ---- pose / result records ---------------------------------------------- */

/* as::DOF_6D<float>, src/model/Types_6D.h:32-37: translation, then ZYZ Euler angles */
typedef struct { float pos[3]; float ang[3]; } gba_dof6d;

/* as::Result_6D<float>, src/model/Types_6D.h:47-54: energy, force sum (= -dE/dpos),
 * Euler-angle "torque" (= -dE/dang) */
typedef struct { float E; float pos[3]; float ang[3]; } gba_result6d;

/* as::DOF_6D_Modes<float>, src/model/Types_6D_Modes.h:33-41 */
typedef struct {
	gba_dof6d rigid;
	float modesRec[GBA_MODES_MAX];
	float modesLig[GBA_MODES_MAX];
} gba_dof6d_modes;

/* as::Result_6D_Modes<float>, src/model/Types_6D_Modes.h:54-60 */
typedef struct {
	gba_result6d rigid;
	float modesRec[GBA_MODES_MAX];
	float modesLig[GBA_MODES_MAX];
} gba_result6d_modes;

/* ---- model data descriptors --------------------------------------------- */

/* ParamTable<float>::attractFFParams_t, src/model/ParamTable.h:24-30 (after the
 * attract.par transform of src/fileIO/readFile.cpp:484-497) */
typedef struct { float rc; float ac; int32_t ipon; float rmin2; float emin; } gba_ffparam;

/* PotShape, src/model/ParamTable.h:12-16 (same enumerator order) */
#define GBA_POTSHAPE_12_6 0
#define GBA_POTSHAPE_8_6  1
/* Dielec, src/model/SimParam.h:41-44 */
#define GBA_DIELEC_CONSTANT 0
#define GBA_DIELEC_VARIABLE 1

/* IntrplGrid<float>::Desc, src/model/IntrplGrid.h:183-207 (typemask dropped,
 * data passed separately).  Data layout: numGrids channels, channel 0 the
 * charge grid, each channel z-major slices of x-fastest rows of float4
 * (fx, fy, fz, E) -- exactly what readGridFromGridFile builds,
 * src/fileIO/readFile.cpp:261-356. posMin is already translated by -pivot. */
typedef struct {
	uint32_t numGrids;
	uint32_t dimN[3];
	float gridSpacing;
	float posMin[3];
} gba_intrpl_desc;

/* NLGrid<float>::Desc, src/model/NLGrid.h:151-165 */
typedef struct {
	uint32_t dimN[3];
	float gridSpacing;
	float dPlateau;
	float posMin[3];
	uint32_t numEl;        /* total entries of the concatenated neighbour list */
} gba_nl_desc;

/* NeighbourDesc, src/model/NLGrid.h:30-35 */
typedef struct { uint32_t numEl; uint32_t idx; } gba_neighbour_desc;

/* ---- context ------------------------------------------------------------ */

/* Version string of the library. */
const char* gba_version(void);

/* Number of device and pinned-host allocations (cudaMalloc, cudaMallocHost,
 * stream-ordered pool allocations) the library has made in this process.
 * No reference counterpart (instrumentation: lets a caller check that a
 * call allocated nothing). */
int gba_allocation_count(uint64_t* out);

/* Opens a context on CUDA device `device`.  Stands in for the per-device state
 * the reference keeps in DeviceManager/DataManager (src/server/DeviceManager.cpp:29-59)
 * plus the per-worker GPUEnergyService6D buffers (src/service/GPUEnergyService6D.tpp:100-160). */
int gba_create(int device, gba_ctx** out);

/* Frees every device copy owned by the context. */
int gba_destroy(gba_ctx* ctx);

/* Message of the last failed call on this context ("" if none).  With ctx ==
 * NULL, the message of the last failed gba_create on this thread. */
const char* gba_last_error(const gba_ctx* ctx);

/* ---- uploads (synchronous; the library owns the device copies) ----------- */

/* Protein, src/model/Protein.h:39-167 uploaded like DeviceDataConfigurator::attach
 * (src/server/DeviceDataConfigurator.tpp:28-95).
 *  xyz        3*n floats, SoA (x[0..n), y[0..n), z[0..n)), pivotized
 *  type       n raw ATTRACT types after the default map (99 -> 0); 0 = dummy bead
 *  mapped     n grid channels of the partner's grid (0 = no grid term)
 *  charge     n charges
 *  n_modes    0..GBA_MODES_MAX; modes = 3*n*n_modes floats in the reference's
 *             layout x[i*n_modes+m], then y, then z (src/model/Protein.h:88-98);
 *             mode_force = n_modes floats (may be NULL when n_modes == 0) */
int gba_upload_protein(gba_ctx* ctx, uint32_t n, const float* xyz, const uint32_t* type,
		const uint32_t* mapped, const float* charge, uint32_t n_modes,
		const float* modes, const float* mode_force, gba_id* out);

/* GridUnion (inner + outer IntrplGrid, NLGrid), src/model/GridUnion.h:20, uploaded
 * like src/server/DeviceDataConfigurator.tpp:141-326 but as plain device buffers.
 *  inner_data / outer_data: numGrids*dimN.x*dimN.y*dimN.z float4 (16 B each)
 *  nl_grid: dimN.x*dimN.y*dimN.z descriptors; nl_list: nl->numEl receptor indices */
int gba_upload_grid(gba_ctx* ctx,
		const gba_intrpl_desc* inner, const float* inner_data,
		const gba_intrpl_desc* outer, const float* outer_data,
		const gba_nl_desc* nl, const gba_neighbour_desc* nl_grid, const uint32_t* nl_list,
		gba_id* out);

/* ParamTable<float> (src/model/ParamTable.h:18-101) + SimParam<float>
 * (src/model/SimParam.h:39-55); table[numTypes*typeA + typeB] as getParams(). */
int gba_upload_params(gba_ctx* ctx, uint32_t num_types, const gba_ffparam* table,
		int potshape, int dielec, float ffelec, gba_id* out);

/* Drops a data item (DataManager::remove). */
int gba_release(gba_ctx* ctx, gba_id id);

/* Batches of >= 4096 poses are visited grouped by translation cell (32^3
 * cells over the outer grid; multi-pair minimizer batches by pair and Morton
 * order) -- results unchanged, each pose keeps its slot -- so that the poses
 * resident on the GPU at a time share grid regions in L2.  Enabled by
 * default; 0 turns it off.  No reference counterpart (a scheduling choice of
 * this library). */
int gba_set_pose_order(gba_ctx* ctx, int enable);

/* Kernel implementation options (no reference counterpart; every option
 * keeps results within the parity bounds and grid indices / neighbour walks
 * bit-exact):
 *   GBA_KOPT_RATIO_COMPUTED  the plateau ratio of table bin n = int(r^2 * 1e4)
 *                            (src/model/NLGrid.tpp:45-50) is evaluated as
 *                            sqrt((n + 0.5) * 1e-4 / plateau^2) in FP32 --
 *                            within one ulp of the table entry -- instead of
 *                            being gathered from the 4 MB table;
 *   GBA_KOPT_COOP_LOOKUP     on grids with the octet layout (gba_grid_octets),
 *                            8 lanes share one grid lookup, one corner each,
 *                            loaded without L1 allocation;
 *   GBA_KOPT_FOUR_BLOCKS     the scoring kernel is compiled for four resident
 *                            256-thread blocks per SM (64 registers a thread);
 *   GBA_KOPT_TYPED_LIST      the rigid kernels read a copy of the neighbour
 *                            list whose entries carry the receptor bead's
 *                            type in their top 8 bits (built on the device at
 *                            the first use of a grid with a receptor, 4 bytes
 *                            per list entry, kept with the grid until either
 *                            is released) instead of gathering the type per
 *                            pair.  Receptors with types above 255 or 2^24
 *                            beads or more keep the gather;
 *   GBA_KOPT_REFERENCE_ORDER every pose is summed in the reference CPU
 *                            path's operation order (CPUEnergyService6D,
 *                            src/service/CPUEnergyService6D.tpp:63-200): bead
 *                            by bead, grid term then neighbour list in list
 *                            order, the reference's float and double steps,
 *                            then the bead sums in bead order -- so energies
 *                            and minimizer trajectories equal the reference's
 *                            bit for bit wherever its sin/cos are correctly
 *                            rounded.  Reads the ratio table and the
 *                            native lookups whatever the other options say.
 *                            Slower; applies to gba_energy_6d, the
 *                            noalloc and batch scoring calls, both minimizer
 *                            forms (teams included), and the
 *                            normal-mode scoring and minimizers
 *                            (CPUEnergyService6DModes,
 *                            src/service/CPUEnergyService6DModes.tpp:121-327;
 *                            a per-warp receptor array of 16 B per receptor
 *                            bead in call scratch); not to gba_census_6d.
 *                            Off by default.
 * The default is the first four.  Changing options drops the cached
 * minimizer graphs; call it while no other call on the context is in
 * flight. */
#define GBA_KOPT_RATIO_COMPUTED 1u
#define GBA_KOPT_COOP_LOOKUP    2u
#define GBA_KOPT_FOUR_BLOCKS    4u
#define GBA_KOPT_TYPED_LIST     8u
#define GBA_KOPT_REFERENCE_ORDER 16u
#define GBA_KOPT_DEFAULT        (GBA_KOPT_RATIO_COMPUTED | GBA_KOPT_COOP_LOOKUP | GBA_KOPT_FOUR_BLOCKS | \
                                 GBA_KOPT_TYPED_LIST)
int gba_set_kernel_options(gba_ctx* ctx, uint32_t flags);

/* Takes each Euler angle's sine and cosine from this process's C library
 * (sinf, cosf) -- the values the reference's euler2rotmat / euler2torquemat
 * receive on this host (src/model/matrixFunctions.h:40-127) -- instead of
 * computing them correctly rounded on the device.  The library is evaluated
 * once, on all host threads, for every float angle with magnitude in
 * [2^-12, max_abs), and the values are kept on the device: 8 bytes per
 * angle, 3.2 GB for max_abs = 4096 (minimization trajectories reach angles
 * beyond 100 rad).  Below 2^-12
 * the correctly rounded values (sin a = a, cos a = 1) are used, as any
 * faithful library returns; at or beyond max_abs the computed ones.  With
 * GBA_KOPT_REFERENCE_ORDER the rigid results then equal the reference's on
 * this host bit for bit.  Applies to every rigid and normal-mode call of the
 * context.  max_abs = 0 (or any value up to 2^-12) turns it off and frees
 * the table; max_abs above 4096, negative or NaN is rejected.  Like gba_set_kernel_options, call it while no other call on
 * the context is in flight (it replaces data those calls read).  No
 * reference counterpart. */
int gba_set_host_sincos(gba_ctx* ctx, float max_abs);

/* While enabled, CUDA events are recorded on the launching stream around
 * every fused rigid energy kernel launch (gba_energy_6d and friends);
 * gba_kernel_time synchronizes on them and returns the summed kernel time
 * and launch count since the last reset (reset != 0 clears them).  Lets a
 * caller time the kernel alone inside a call that also launches the
 * visiting-order pass.  No reference counterpart (instrumentation). */
int gba_kernel_timing(gba_ctx* ctx, int32_t enable);
int gba_kernel_time(gba_ctx* ctx, double* ms_total, uint64_t* launches, int32_t reset);

/* ---- evaluation ----------------------------------------------------------- */

/* One energy+gradient evaluation per pose (rigid body), the work of one
 * CPUEnergyService6D / GPUEnergyService6D item processor
 * (src/service/CPUEnergyService6D.tpp:63-200, src/service/GPUEnergyService6D.tpp:470-510),
 * fused into one kernel launch.  `dofs`/`out` may be device or host pointers.
 * `stream` is a cudaStream_t (NULL = legacy default stream).  With two device
 * pointers the call is asynchronous on `stream`; if either is a host pointer the
 * copies run on `stream` and the call returns after the stream has drained. */
int gba_energy_6d(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_dof6d* dofs, size_t n, gba_result6d* out, void* stream);

/* gba_energy_6d for device pointers that allocates nothing (no counterpart in
 * the reference), for callers that must not allocate while they score: a
 * service running under a fixed device-memory budget, or a host that has
 * reserved all device memory up front.  The pose counter and the
 * visiting-order scratch live in a static 2 MiB device array per device,
 * whose address the first call on each context resolves with
 * cudaGetSymbolAddress -- make that first call before any stream capture.
 * At most 65536 poses per call (more: GBA_ERR_INVALID_ARGUMENT).  Nothing
 * must be zeroed beforehand (the call clears what it needs with
 * cudaMemsetAsync).  The pair-term tables it reads are built when the grids
 * and parameter tables are uploaded; a grid's receptor-typed neighbour list
 * (GBA_KOPT_TYPED_LIST) is built only by an allocating scoring call, and
 * until one has run for that grid and receptor this call gathers each
 * neighbour's type instead (identical results, a little slower).  Calls
 * that overlap on one device (any stream, thread or context) share the
 * array and race: serialize them.  Asynchronous on `stream`; results equal
 * gba_energy_6d's bit for bit. */
int gba_energy_6d_noalloc(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_dof6d* dofs, size_t n, gba_result6d* out, void* stream);

/* Normal-mode variant (CPUEnergyService6DModes, src/service/CPUEnergyService6DModes.tpp:76-336):
 * the receptor is deformed and interpolated in the ligand grid `grid_lig`, the
 * ligand deformed and interpolated in the receptor grid `grid_rec`, one NL pass
 * on the receptor NL grid.  Pointer/stream semantics as gba_energy_6d. */
int gba_energy_6d_modes(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid_rec, gba_id grid_lig,
		gba_id params, const gba_dof6d_modes* dofs, size_t n, gba_result6d_modes* out,
		void* stream);

/* ---- minimization and multi-pair batches ----------------------------------- */

/* One receptor-ligand pair's share of a batch.  For gba_batch_energy_6d,
 * `start` holds the poses and only `out_result` is written. */
typedef struct {
	gba_id rec, lig, grid, params;
	const gba_dof6d* start;      /* n poses (host or device) */
	size_t n;
	gba_dof6d* out_state;        /* last evaluated DOF per pose */
	gba_result6d* out_result;    /* last evaluated Result per pose */
	int32_t* out_nevals;         /* energy evaluations per pose (may be NULL) */
	uint64_t* out_done_ns;       /* gba_batch_minimize_6d: per pose, ns from the kernel's
	                                start to the pose's completion (HOST pointer, may be NULL) */
} gba_pair_job;

/* Minimizes every pose with the VA13 quasi-Newton method the reference runs
 * through emATTRACT (src/apps/em/minfor.f:1-182, src/apps/em/mc11a.f:1-143,
 * driven by RequestHandler::run, src/apps/em/RequestHandler.tpp:102-216),
 * entirely on the device: one persistent work-queue launch, the minimizer
 * state resident on the GPU, the pipeline replayed as a CUDA graph.
 * Per pose it reports the last evaluated DOF and Result (what
 * RequestHandler::getResultStates/getResultEnGrads return) and the number of
 * energy evaluations; max_evals is maxFunEval (500 in the reference,
 * src/apps/em/VA13Solver.h:66).  Synchronous. */
int gba_minimize_6d(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_dof6d* start, size_t n, int max_evals, gba_dof6d* out_state,
		gba_result6d* out_result, int32_t* out_nevals, void* stream);

/* The same minimization over the poses of many pairs of uneven sizes in one
 * persistent launch (poses from every pair share one work queue). */
int gba_batch_minimize_6d(gba_ctx* ctx, const gba_pair_job* jobs, size_t njobs, int max_evals,
		void* stream);

/* One energy+gradient evaluation for the poses of many pairs in one launch. */
int gba_batch_energy_6d(gba_ctx* ctx, const gba_pair_job* jobs, size_t njobs, void* stream);

/* The reference's execution model on the same GPU: VA13 per pose on the host
 * and, per evaluation round, the active poses cut into work items of
 * item_size poses (100 is the reference's DEFAULT_ITEM_SIZE,
 * src/server/Server.h:39; 0 = all active poses in one item), each copied in,
 * evaluated by one fused launch and copied out, then a sync -- as
 * RequestHandler + Server + GPU service do.  Host pointers only; results
 * identical in meaning (and bit for bit) to gba_minimize_6d. */
int gba_minimize_6d_plain(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_dof6d* start, size_t n, int max_evals, size_t item_size, gba_dof6d* out_state,
		gba_result6d* out_result, int32_t* out_nevals, void* stream);

/* Minimization of flexible poses: VA13 over the DOF vector (ang xyz, pos xyz,
 * modesRec[0..Mr), modesLig[0..Ml)) -- minfor.f generalised beyond its fixed
 * 6 DOF (src/apps/em/minfor.f:16,33) -- with the normal-mode energy of
 * gba_energy_6d_modes; persistent device kernel, synchronous.  The gradient
 * is -ang, -pos (those result entries are forces) and +modesRec, +modesLig:
 * reduceModeForce stores -sum f . v (src/model/reduction_modes.h:29-90),
 * which is dE/d(amplitude) plus correctModeForce's term.  The reference's
 * converter negates the mode entries too (src/apps/em/meta.h:193-201), which
 * climbs along the modes; this library descends. */
int gba_minimize_6d_modes(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid_rec, gba_id grid_lig,
		gba_id params, const gba_dof6d_modes* start, size_t n, int max_evals,
		gba_dof6d_modes* out_state, gba_result6d_modes* out_result, int32_t* out_nevals,
		void* stream);

/* Plain per-step form of gba_minimize_6d_modes: host VA13 and, per
 * evaluation round, the active poses cut into work items of item_size poses
 * (0 = all active poses in one item; 100 is the reference server's default),
 * each copied in, evaluated by one launch and copied out, as
 * gba_minimize_6d_plain does.  Host pointers only; results bit-identical to
 * gba_minimize_6d_modes. */
int gba_minimize_6d_modes_plain(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid_rec,
		gba_id grid_lig, gba_id params, const gba_dof6d_modes* start, size_t n, int max_evals,
		size_t item_size, gba_dof6d_modes* out_state, gba_result6d_modes* out_result,
		int32_t* out_nevals, void* stream);

/* Warps per pose of the device minimizer (no reference counterpart; a
 * launch-shape choice): 0 (default) = chosen from the job size -- jobs with
 * fewer poses than the one-warp kernel has resident warps give each pose a
 * team of up to 7 warps, never more than its ligand has 64-bead rounds;
 * 1 = one warp per pose; 2..7 = teams of that many warps (capped by the
 * ligand's rounds): a block per pose, whose first warp steps the pose's VA13
 * after each evaluation, when every pose of the job fits resident that way;
 * otherwise two poses per block and a control warp that runs one pose's
 * VA13 step while the team evaluates the other.  The result of
 * every pose is the same bit for bit whatever the setting: the minimizers
 * reduce each 64-bead round on its own and add the rounds in order (the
 * plain per-step form's launches do the same; gba_energy_6d reduces once
 * per pose, which differs in the last bits). */
int gba_set_minimize_team(gba_ctx* ctx, int warps_per_pose);

/* Wall-time budget for device minimization (0 = none): warps stop claiming
 * poses once it is spent and the call returns GBA_ERR_TIMEOUT; the
 * counterpart of Server::setWaitTime (src/server/Server.h:71). */
int gba_set_deadline(gba_ctx* ctx, uint32_t milliseconds);

/* ---- pairwise (grid-free) path and its adjoint ------------------------------ */

/* Free parameters of the pairwise path.  All arrays are DEVICE pointers.
 * r0/eps/ipon: num_types^2 entries indexed [rec type - 1][lig type - 1]
 * (ParamTable::getParams order, src/model/ParamTable.h:78-80), turned into
 * rc = eps r0^8, ac = eps r0^6 as src/fileIO/readFile.cpp:484-497 does. */
typedef struct {
	uint32_t num_types;
	const float* r0;
	const float* eps;
	const int32_t* ipon;
	const float* q_lig;      /* per ligand bead */
	const float* q_rec;      /* per receptor bead */
	int potshape;            /* GBA_POTSHAPE_8_6 */
	int dielec;
	float ffelec;
	float cutoff;            /* pair cutoff (<= what the grid's NL lists cover) */
} gba_pairwise_params;

/* Exact ATTRACT pair energy over all receptor-ligand pairs within `cutoff`
 * (the NL pair terms of src/model/neighborlist.h:104-157 without the plateau
 * subtraction, src/model/forcefield.h), candidates taken from `grid`'s
 * neighbour lists.  No reference counterpart as an entry point: the reference
 * has no differentiable scoring.  Device pointers; asynchronous on `stream`.
 *  forward  (gE == NULL): E_out[n] = energy per pose
 *  backward (gE != NULL): recomputes everything and writes g_dofs[n*6]
 *           = gE * dE/dDOF in (pos, ang) order -- i.e. -gE * Result, the
 *           convention of src/apps/em/meta.h:114-121 -- and ADDS gE-weighted
 *           dE/dq_lig, dE/dq_rec, dE/dr0, dE/deps into the FP64 arrays. */
int gba_pairwise_6d(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid,
		const gba_pairwise_params* pp, const gba_dof6d* dofs, size_t n, float* E_out,
		const float* gE, float* g_dofs, double* g_qlig, double* g_qrec, double* g_r0,
		double* g_eps, void* stream);

/* ---- autotuner ------------------------------------------------------------ */

typedef struct {
	int energy_threads, energy_blocks_per_sm;   /* scoring kernel launch shape */
	int minimize_threads, minimize_chunk;       /* persistent minimizer: block size, poses per grab */
	float energy_ms, minimize_ms;               /* best sample times (-1 when taken from the cache) */
	int from_cache;                             /* bit 0: energy, bit 1: minimize read from cache */
	int minimize_team;                          /* warps per pose: 1, or a team of 2..7 -- a block per pose
	                                               when all fit resident, else two poses per block with a
	                                               control warp (team + 1 warps: minimize_threads) */
} gba_tune_result;

/* Times candidate launch shapes of the scoring kernel (threads per block x
 * resident blocks per SM) and of the persistent minimizer (threads per block x
 * poses per queue grab with one warp per pose, or teams of 2..7 warps per pose
 * -- poses per CTA below one) on `sample` poses of this pair and keeps the
 * fastest for this pair: gba_energy_6d, gba_minimize_6d and the plain form
 * launch the pair with them, and a gba_batch_minimize_6d batch launches the
 * pairs of each tuned shape as one persistent kernel, the groups running
 * concurrently in one CUDA graph.  A tuned team applies to minimizations of
 * at most the sample's size.  With cache_path, results are read from /
 * appended to that text file (keyed by device, SM count and pair size).  No
 * reference counterpart: the reference fixes 128-thread blocks
 * (src/service/GPUEnergyService6D.tpp:440-441) and sizes its reduction block
 * from the device (src/service/GPUEnergyService6D.tpp:184-198). */
int gba_autotune(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_dof6d* sample, size_t n, int max_evals, const char* cache_path,
		gba_tune_result* out);

/* Sets the pair's launch shapes directly (for instance ones an earlier
 * gba_autotune reported), as gba_autotune would keep them; energy_ms,
 * minimize_ms and from_cache are ignored.  energy_threads 32..256 (multiple
 * of 32), energy_blocks_per_sm >= 1; minimize_team 1..7; with team 1,
 * minimize_threads 32..256 (multiple of 32) and minimize_chunk 1..16.  A team
 * set here applies to minimizations of any size.  No reference counterpart. */
int gba_set_pair_shape(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_tune_result* shape);

/* ---- grid builder --------------------------------------------------------- */

/* Options of the device grid builder (inner 0.9 A, outer 1.8 A, plateau 10 A,
 * neighbour radius 10.8 A, outer extension 32 inner voxels). */
typedef struct {
	float spacing;          /* inner voxel size */
	float plateau;          /* NL plateau distance */
	float nl_cutoff;        /* neighbour-list radius around a voxel centre */
	float margin;           /* inner box = receptor bounding box + margin */
	uint32_t outer_ext;     /* outer extension, in inner voxels per side */
	uint32_t n_alphabet;    /* ligand types that get a channel (<= 98) */
	uint32_t alphabet[99];  /* raw ligand type served by channel c+1 */
} gba_grid_build_opts;

/* Builds the inner, outer and neighbour-list grids of receptor `rec` on the
 * device, in the layout of readGridFromGridFile (src/fileIO/readFile.cpp:261-422)
 * -- the step the reference delegates to ATTRACT's grid program
 * (attract::Grid::calculate_std, declared at src/fileIO/grid_orig.h:143). */
int gba_build_grid(gba_ctx* ctx, gba_id rec, gba_id params, const gba_grid_build_opts* opt,
		gba_id* out);

/* Adds (enable != 0) or drops a duplicated-octet copy of a grid's inner and
 * outer potentials: per channel and voxel the 8 interpolation corners in one
 * aligned 128-byte record, so each lookup reads a single L2 line instead of
 * four rows of the reference layout.  Costs 8x the potential grids' memory;
 * results are unchanged.  No reference counterpart (a layout choice). */
int gba_grid_octets(gba_ctx* ctx, gba_id grid, int enable);

/* Descriptors of a device grid (sizes for gba_download_grid). */
int gba_grid_info(gba_ctx* ctx, gba_id grid, gba_intrpl_desc* inner, gba_intrpl_desc* outer,
		gba_nl_desc* nl);

/* Copies a device grid to host buffers sized from gba_grid_info (any may be NULL). */
int gba_download_grid(gba_ctx* ctx, gba_id grid, float* inner, float* outer,
		gba_neighbour_desc* nl_grid, uint32_t* nl_list);

/* ---- instrumentation ---------------------------------------------------------- */

/* gba_energy_6d plus, per pose, 4 counters {beads interpolated, of which
 * charged, beads with an NL lookup, sum of their voxels' numEl}: the inputs of
 * the roofline byte count.  No reference counterpart (measurement only).
 * Synchronous; pointers may be host or device. */
int gba_census_6d(gba_ctx* ctx, gba_id rec, gba_id lig, gba_id grid, gba_id params,
		const gba_dof6d* dofs, size_t n, gba_result6d* out, uint32_t* census);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* GBATTRACT_H_ */
