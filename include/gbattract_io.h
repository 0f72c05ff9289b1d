/*
 * gbattract_io.h -- file formats on either side of the docking energy path
 * (part of libgbattract, host code only, no device needed).
 *
 * The readers and writers follow gpuATTRACT 2.0's own file IO so that its
 * inputs load unchanged and its tools read what this library writes:
 *   reduced PDB        src/fileIO/readFile.cpp:103-175 (readProteinFromPDB)
 *   ATTRACT .par       src/fileIO/readFile.cpp:431-520 (readParamTableFromFile)
 *   grid alphabet      src/fileIO/readFile.cpp (readGridAlphabetFromFile)
 *   DOF files          src/fileIO/readFile.cpp:579-651 (readDOF),
 *                      src/fileIO/readFile.cpp:747-871 (readDOFHeader)
 *   score output       src/model/Types_6D.tpp:40-68, src/model/Types_6D_Modes.tpp:50-90
 *                      (operator<< of the result records), read back by
 *                      src/fileIO/readFile.cpp:653-745 (readResult)
 *   ATTRACT .grid      src/fileIO/grid_orig.cpp:85-300 (read_std),
 *                      src/fileIO/grid_orig.cpp:303-484 (write_std),
 *                      src/fileIO/readFile.cpp:261-422 (readGridFromGridFile)
 *   pivots / frames    src/model/Protein.tpp:145-157 (auto_pivotize),
 *                      src/model/DOFTransform.cpp:35-90 (transformDOF_glob2rec)
 *
 * Every function returns GBA_OK (0) or a gbattract.h status code and never
 * exits; gba_io_last_error() gives the message of the calling thread's last
 * failure.  Where the reference prints and calls exit(), these return
 * GBA_ERR_INVALID_ARGUMENT.  Readers are two-phase: called with NULL output
 * buffers they report the sizes, then fill caller-owned buffers.
 */
#ifndef GBATTRACT_IO_H_
#define GBATTRACT_IO_H_

#include "gbattract.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Message of the calling thread's last failed gba_io call ("" if none). */
const char* gba_io_last_error(void);

/* ---- reduced PDB --------------------------------------------------------- */

/* Columns 31-38, 39-46, 47-54 (x, y, z), 55-59 (type), 60-67 (charge) of every
 * non-empty line, as readProteinFromPDB takes them.  *n receives the bead
 * count; xyz (SoA, 3*n floats), type and charge may be NULL to query it;
 * cap is the capacity of the given arrays in beads. */
int gba_read_pdb(const char* path, uint32_t* n, float* xyz, uint32_t* type, float* charge,
		uint32_t cap);

/* ---- ATTRACT force-field parameter file --------------------------------- */

/* Reads potshape, the type count and the rc/ac/ipon matrices and applies the
 * file transform of readParamTableFromFile (8-6 and 12-6 shapes) in the
 * reference's arithmetic.  *num_types receives T; table (T*T records, row
 * [i*T + j]) may be NULL to query; *potshape receives GBA_POTSHAPE_*;
 * swi_on / swi_off (may be NULL) the switching radii of the header. */
int gba_read_params(const char* path, uint32_t* num_types, gba_ffparam* table, uint32_t cap,
		int32_t* potshape, float* swi_on, float* swi_off);

/* Grid alphabet file: the listed type numbers, in file order. */
int gba_read_alphabet(const char* path, uint32_t* n, uint32_t* types, uint32_t cap);

/* ---- DOF files ----------------------------------------------------------- */

/* Header of a DOF file (readDOFHeader): explicit pivots or "#pivot auto",
 * and the centering flags. */
typedef struct {
	int32_t auto_pivot;
	int32_t centered_receptor;
	int32_t centered_ligands;
	uint32_t num_pivots;          /* explicit pivots (<= 16 kept) */
	float pivots[16][3];
} gba_dof_header;

/* DOF body (readDOF): structures separated by '#' lines, one line per
 * molecule holding ang xyz, pos xyz and up to 10 further values (mode
 * amplitudes).  Output layout: values[(s * num_molecules + m) * 16 + k] for
 * structure s, molecule m, value k (ang xyz, pos xyz, extras), counts[s *
 * num_molecules + m] = values on that line (6..16).  Pass NULL values /
 * counts to query num_structures and num_molecules; cap is in lines
 * (structures * molecules).  Values are parsed as double and stored as float
 * (the reference converts to its REAL the same way, DOFConverter). */
int gba_read_dof(const char* path, gba_dof_header* header, uint32_t* num_structures,
		uint32_t* num_molecules, float* values, int32_t* counts, size_t cap);

/* Writes a DOF file that readDOF / readDOFHeader accept: the header, then per
 * structure "#<s+1>", an optional "## Energy: <E>" comment (energies may be
 * NULL) and one line per molecule with counts[] values, in %.9g (float
 * values round-trip exactly). Same value layout as gba_read_dof. */
int gba_write_dof(const char* path, const gba_dof_header* header, uint32_t num_structures,
		uint32_t num_molecules, const float* values, const int32_t* counts, const float* energies);

/* ---- types and frames ---------------------------------------------------- */

/* The ligand type mapping of Configurator_6D::init
 * (src/service/Configurator_6D.tpp:49-54): the default map (identity, 99 ->
 * 0, src/model/defaultTypeInitializerList.h) rewrites the raw types in
 * place, then the receptor grid alphabet maps them to grid channels
 * (createTypeMapFromVector, src/model/TypeMap.h:53-61: alphabet[i] -> i+1,
 * 99 -> 0, 0 -> 0).  A type the maps do not hold is an error (std::map::at
 * throws in the reference).  types_out / mapped_out may alias types_in. */
int gba_map_types(const uint32_t* alphabet, uint32_t n_alphabet, const uint32_t* types_in, uint32_t n,
		uint32_t* types_out, uint32_t* mapped_out);

/* auto_pivotize: centroid of the n beads (SoA xyz), summed in the precision
 * of the reference's Protein<float> (float accumulators, divided by
 * (double)n). */
int gba_auto_pivot(const float* xyz, uint32_t n, float pivot[3]);

/* transformDOF_glob2rec for n (receptor, ligand) DOF pairs in place:
 * ligand DOFs end in the frame of the pivotized receptor at the origin,
 * receptor DOFs become zero.  dof_rec / dof_lig are gba_dof6d arrays with a
 * stride of `stride` bytes (sizeof(gba_dof6d) or sizeof(gba_dof6d_modes)). */
int gba_dof_glob2rec(void* dof_rec, void* dof_lig, size_t n, size_t stride, const float pivot_rec[3],
		const float pivot_lig[3], int32_t centered_rec, int32_t centered_lig);

/* ---- score output -------------------------------------------------------- */

/* Writes n results.  style 0: the text of operator<<(Result_6D) (records
 * gba_result6d, n_modes_rec == n_modes_lig == 0) or operator<<(Result_6D_Modes)
 * (records gba_result6d_modes), each followed by a newline as the
 * reference's apps print them (src/apps/em/emATTRACT.tpp:55-57).  style 1:
 * ATTRACT's .score layout that readResult parses -- energy, energy-term line,
 * then a "Gradients:" line (and with modes a "Mode gradients:" block) for the
 * receptor (rigid part zero: it is the fixed frame) and for the ligand
 * (ang xyz, pos xyz).  append != 0 appends to an existing file. */
#define GBA_RESULTS_STREAM 0
#define GBA_RESULTS_SCORE  1
int gba_write_results(const char* path, int32_t append, int32_t style, const void* results, size_t n,
		uint32_t n_modes_rec, uint32_t n_modes_lig);

/* readResult: per " Energy:" record the energy followed by every value of its
 * gradient blocks in file order (per molecule the six "Gradients:" values as
 * printed, then its "Mode gradients:" values).  out[r * stride + k], k = 0
 * the energy; counts[r] = values stored for record r.  NULL out and counts
 * query *n (records) and *width (largest value count).  The text of
 * operator<<(Result_6D_Modes) has no "Gradients:" tag and is rejected (the
 * reference's readResult does not terminate on it). */
int gba_read_results(const char* path, size_t* n, uint32_t* width, double* out, int32_t* counts,
		size_t cap, uint32_t stride);

/* ---- ATTRACT binary grid (.grid) ---------------------------------------- */

/* Fields of the .grid header besides the grid arrays. */
typedef struct {
	double gridspacing;       /* inner spacing; the outer grid has twice it */
	int32_t gridextension;    /* outer extension in inner voxels (even) */
	double plateaudis;
	double neighbourdis;
	uint8_t alphabet[99];     /* alphabet[t-1] != 0: type t has a channel */
	float ori[3];             /* inner grid origin (absolute frame) */
	int32_t inner_dim[3];
	int32_t outer_dim[3];
	int32_t natoms;           /* receptor beads */
	double pivot[3];          /* receptor pivot stored with the grid */
	uint16_t architecture;    /* 64 (or 32) -- must match the reader's */
	int32_t nr_energrads;
	int32_t nr_neighbours;
} gba_grid_file_info;

/* Header only; sizes needed by gba_read_grid_file. */
int gba_grid_file_info_read(const char* path, gba_grid_file_info* info);

/* readGridFromGridFile: inner / outer interpolation grids with the charge
 * channel first (numGrids = alphabet size + 1), unset potentials zero, and
 * the NL grid (idx = stored list start - 1, as the reference sets it).
 * Data buffers: inner_data numGrids*Ni float4, outer_data numGrids*No float4,
 * nl_grid Ni descriptors, nl_list nr_neighbours indices; any may be NULL to
 * skip it.  Descriptors are in the file's absolute frame (the reference
 * translates them by -pivot afterwards, Configurator_6D.tpp:104). */
int gba_read_grid_file(const char* path, gba_intrpl_desc* inner, float* inner_data,
		gba_intrpl_desc* outer, float* outer_data, gba_nl_desc* nl, gba_neighbour_desc* nl_grid,
		uint32_t* nl_list);

/* write_std with every voxel populated: the energy/gradient records in the
 * order write_std re-sorts them (inner voxels, then outer, each over the
 * alphabet types ascending and the charge channel last), the neighbour lists
 * concatenated in voxel order.  alphabet lists the type of each channel
 * 1..numGrids-1 (channel c holds type alphabet[c-1]); rec_xyz (SoA, natoms
 * beads, NULL allowed) sets each neighbour's plateau flag (1 inside
 * plateaudis of the voxel centre, else 2).  The descriptors must describe an
 * ATTRACT layout: outer spacing twice the inner one and outer origin =
 * ori - gridextension * gridspacing (checked).  The architecture field is
 * taken from info. */
int gba_write_grid_file(const char* path, const gba_grid_file_info* info, const uint32_t* alphabet,
		const gba_intrpl_desc* inner, const float* inner_data, const gba_intrpl_desc* outer,
		const float* outer_data, const gba_nl_desc* nl, const gba_neighbour_desc* nl_grid,
		const uint32_t* nl_list, const float* rec_xyz);

#ifdef __cplusplus
}
#endif

#endif /* GBATTRACT_IO_H_ */
