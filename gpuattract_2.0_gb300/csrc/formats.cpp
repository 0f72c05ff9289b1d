/*
 * formats.cpp -- readers and writers of the files on either side of the
 * docking energy path (host code; C ABI in include/gbattract_io.h).
 *
 * Each function states the reference routine whose behaviour it keeps,
 * including its quirks where files depend on them (an unterminated last PDB
 * line is dropped; the DOF body starts at the first line that is not a '#'
 * comment).  Failures that make the reference print and exit() return
 * GBA_ERR_INVALID_ARGUMENT with a message instead; undefined behaviour of
 * the reference on malformed input (unchecked vector indexing, overlong DOF
 * lines) is reported as an error as well.
 */
#include "gbattract_io.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <new>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

thread_local std::string g_io_error;

struct IoError : std::runtime_error {
	int code;
	IoError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(const std::string& m) { throw IoError(GBA_ERR_INVALID_ARGUMENT, m); }

template <class F>
int guarded(F&& f) {
	try {
		f();
		g_io_error.clear();
		return GBA_OK;
	} catch (const IoError& e) {
		g_io_error = e.what();
		return e.code;
	} catch (const std::bad_alloc&) {
		g_io_error = "out of host memory";
		return GBA_ERR_OUT_OF_MEMORY;
	} catch (const std::exception& e) {
		g_io_error = e.what();
		return GBA_ERR_INVALID_ARGUMENT;
	}
}

void need(const void* p, const char* what) {
	if (!p) fail(std::string("null argument: ") + what);
}

std::ifstream open_in(const char* path, std::ios::openmode m = std::ios::in) {
	need(path, "path");
	std::ifstream f(path, m);
	if (!f.is_open()) fail(std::string("failed to open file ") + path);
	return f;
}

std::vector<std::string> split_ws(const std::string& line) {
	std::istringstream iss(line);
	return std::vector<std::string>{std::istream_iterator<std::string>{iss},
			std::istream_iterator<std::string>{}};
}

bool starts_with(const std::string& s, const char* p) { return s.compare(0, std::strlen(p), p) == 0; }

/* ---------------------------------------------------------------- PDB -- */

struct PdbBeads {
	std::vector<float> x, y, z, q;
	std::vector<uint32_t> t;
};

/* readProteinFromPDB, src/fileIO/readFile.cpp:103-175 with pdbLine2Strings
 * (:58-74): fixed columns, whitespace stripped, stream extraction. */
PdbBeads read_pdb_file(const char* path) {
	std::ifstream f = open_in(path);
	static const int cols[5][2] = {{30, 38}, {38, 46}, {46, 54}, {54, 59}, {59, 67}};
	PdbBeads B;
	std::string line;
	size_t lineno = 1;
	std::getline(f, line);
	while (!f.eof()) {
		if (line.empty()) {
			std::getline(f, line);
			++lineno;
			continue;
		}
		std::string tok[5];
		for (int c = 0; c < 5; ++c) {
			if ((size_t)cols[c][0] > line.size())
				fail(std::string(path) + ": line " + std::to_string(lineno) + " is too short for a reduced PDB record");
			std::string s = line.substr(cols[c][0], cols[c][1] - cols[c][0]);
			s.erase(std::remove_if(s.begin(), s.end(), [](unsigned char ch) { return std::isspace(ch) != 0; }),
					s.end());
			tok[c] = s;
		}
		float x = 0.f, y = 0.f, z = 0.f, q = 0.f;
		unsigned t = 0;
		std::istringstream(tok[0]) >> x;
		std::istringstream(tok[1]) >> y;
		std::istringstream(tok[2]) >> z;
		std::istringstream(tok[3]) >> t;
		std::istringstream(tok[4]) >> q;
		B.x.push_back(x);
		B.y.push_back(y);
		B.z.push_back(z);
		B.t.push_back(t);
		B.q.push_back(q);
		std::getline(f, line);
		++lineno;
	}
	return B;
}

/* ---------------------------------------------------------- DOF files -- */

constexpr int kDofValues = 16;   /* DOF_MAX_NUMBER, src/fileIO/readFile.h:103 */

struct DofFile {
	gba_dof_header h{};
	uint32_t molecules = 0;
	std::vector<std::vector<std::vector<double>>> mol;   /* [molecule][structure] -> values */
};

/* readDOFHeader, src/fileIO/readFile.cpp:747-871. */
gba_dof_header read_dof_header(const char* path) {
	std::ifstream f = open_in(path);
	gba_dof_header h{};
	bool pivots_done = false, rec_done = false, lig_done = false;
	std::vector<float> piv;
	std::string line;
	while (!f.eof()) {
		if (pivots_done && rec_done && lig_done) break;
		std::getline(f, line);
		if (starts_with(line, "##")) continue;
		const std::vector<std::string> tok = split_ws(line);
		if (tok.empty()) continue;
		if (tok[0] == "#pivot") {
			if (pivots_done) fail(std::string(path) + ": incorrect pivot definition");
			if (tok.size() > 1 && tok[1] == "auto") {
				h.auto_pivot = 1;
				pivots_done = true;
				continue;
			}
			if (tok.size() != 5) fail(std::string(path) + ": incorrect pivot definition");
			float p[3] = {0.f, 0.f, 0.f};
			for (int a = 0; a < 3; ++a) std::istringstream(tok[2 + a]) >> p[a];
			piv.insert(piv.end(), p, p + 3);
			continue;
		}
		if (tok[0] == "#centered" && (!rec_done || !lig_done)) {
			pivots_done = true;
			if (tok.size() < 3) fail(std::string(path) + ": centering definition invalid");
			int v;
			if (tok[2] == "true") v = 1;
			else if (tok[2] == "false") v = 0;
			else fail(std::string(path) + ": centering definition invalid");
			if (tok[1] == "receptor:") {
				h.centered_receptor = v;
				rec_done = true;
			} else if (tok[1] == "ligand:" || tok[1] == "ligands:") {
				h.centered_ligands = v;
				lig_done = true;
			} else {
				fail(std::string(path) + ": centering definition invalid");
			}
		}
	}
	const size_t np = piv.size() / 3;
	h.num_pivots = (uint32_t)std::min<size_t>(np, 16);
	for (size_t k = 0; k < h.num_pivots; ++k)
		for (int a = 0; a < 3; ++a) h.pivots[k][a] = piv[3 * k + a];
	return h;
}

/* readDOF, src/fileIO/readFile.cpp:579-651: blocks of molecule lines
 * separated by '#' lines; the first block fixes the molecule count. */
DofFile read_dof_file(const char* path) {
	DofFile D;
	D.h = read_dof_header(path);
	std::ifstream f = open_in(path);
	std::string line;
	size_t lineno = 0;
	uint32_t block = 0;
	while (!f.eof()) {
		std::getline(f, line);
		++lineno;
		if (starts_with(line, "#")) continue;
		uint32_t i = 0;
		while (!starts_with(line, "#") && !f.eof()) {
			if (block == 0) D.mol.emplace_back();
			if (i >= D.mol.size())
				fail(std::string(path) + ": structure #" + std::to_string(block + 1) + " has more molecules than the first (line " +
						std::to_string(lineno) + ")");
			std::istringstream ss(line);
			std::vector<double> v;
			double x;
			while (ss >> x) v.push_back(x);
			if (v.size() < 6)
				fail(std::string(path) + ": line " + std::to_string(lineno) + " holds fewer than 6 DOF values");
			if (v.size() > (size_t)kDofValues)
				fail(std::string(path) + ": line " + std::to_string(lineno) + " holds more than 16 DOF values");
			D.mol[i].push_back(std::move(v));
			++i;
			std::getline(f, line);
			++lineno;
		}
		if (i != D.mol.size())
			fail(std::string(path) + ": the DOF definition is incomplete at #" + std::to_string(block) + " (line " +
					std::to_string(lineno) + ")");
		++block;
	}
	D.molecules = (uint32_t)D.mol.size();
	return D;
}

/* ------------------------------------------------------------- frames -- */

/* euler2rotmat<float>, src/model/matrixFunctions.h:40-77 */
void euler2rotmat_f(float phi, float ssi, float rot, float m[9]) {
	const float cSSI = std::cos(ssi), cPHI = std::cos(phi), sSSI = std::sin(ssi), sPHI = std::sin(phi);
	const float cSSI_cPHI = cSSI * cPHI, cSSI_sPHI = cSSI * sPHI;
	const float sSSI_cPHI = sSSI * cPHI, sSSI_sPHI = sSSI * sPHI;
	const float cROT = std::cos(rot), sROT = std::sin(rot);
	m[0] = cROT * cSSI_cPHI + sROT * sPHI;
	m[1] = sROT * cSSI_cPHI - cROT * sPHI;
	m[2] = sSSI_cPHI;
	m[3] = cROT * cSSI_sPHI - sROT * cPHI;
	m[4] = sROT * cSSI_sPHI + cROT * cPHI;
	m[5] = sSSI_sPHI;
	m[6] = -cROT * sSSI;
	m[7] = -sROT * sSSI;
	m[8] = cSSI;
}

/* rotmat2euler<float>, src/model/matrixFunctions.h:131-165 (the gimbal test
 * there is abs(bool), i.e. plainly m[8] >= 0.9999) */
void rotmat2euler_f(const float m[9], float& phi, float& ssi, float& rot) {
	phi = std::atan2(m[5], m[2]);
	ssi = (float)std::acos(std::fmin(std::fmax((double)m[8], -1.0), 1.0));
	rot = std::atan2(-m[7], -m[6]);
	if ((double)m[8] >= 0.9999) {
		phi = 0.0f;
		if ((double)std::fabs(m[0]) >= 0.9999) {
			rot = m[0] < 0.0f ? (float)M_PI : 0.0f;
			ssi = m[8] < 0.0f ? (float)M_PI : 0.0f;
		} else {
			if (m[8] < 0.0f) {
				ssi = (float)M_PI;
				rot = -std::acos(-m[0]);
			} else {
				ssi = 0.0f;
				rot = std::acos(m[0]);
			}
		}
		if (m[1] < 0.0f) rot = (float)(rot * -1.0);
	}
}

/* transformDOF_glob2rec<float>, src/model/DOFTransform.cpp:35-90 */
void glob2rec_one(gba_dof6d& rec, gba_dof6d& lig, const float pr[3], const float pl[3], bool crec, bool clig) {
	if (!clig)
		for (int a = 0; a < 3; ++a) lig.pos[a] += pl[a];
	if (!crec && !(pr[0] == 0.0f && pr[1] == 0.0f && pr[2] == 0.0f))
		for (int a = 0; a < 3; ++a) lig.pos[a] -= pr[a];
	if (rec.pos[0] != 0.0f || rec.pos[1] != 0.0f || rec.pos[2] != 0.0f)
		for (int a = 0; a < 3; ++a) lig.pos[a] = lig.pos[a] - rec.pos[a];
	if (rec.ang[0] != 0.0f || rec.ang[1] != 0.0f || rec.ang[2] != 0.0f) {
		float Ri[9], Rl[9], M[9];
		euler2rotmat_f(-rec.ang[0], -rec.ang[1], -rec.ang[2], Ri);
		euler2rotmat_f(lig.ang[0], lig.ang[1], lig.ang[2], Rl);
		const float x = lig.pos[0], y = lig.pos[1], z = lig.pos[2];
		lig.pos[0] = Ri[0] * x + Ri[1] * y + Ri[2] * z;
		lig.pos[1] = Ri[3] * x + Ri[4] * y + Ri[5] * z;
		lig.pos[2] = Ri[6] * x + Ri[7] * y + Ri[8] * z;
		for (int i = 0; i < 3; ++i)
			for (int j = 0; j < 3; ++j) {
				float s = 0.0f;
				for (int k = 0; k < 3; ++k) s += Ri[i * 3 + k] * Rl[k * 3 + j];
				M[i * 3 + j] = s;
			}
		rotmat2euler_f(M, lig.ang[0], lig.ang[1], lig.ang[2]);
	}
	for (int a = 0; a < 3; ++a) rec.pos[a] = rec.ang[a] = 0.0f;
}

/* ------------------------------------------------------- score output -- */

/* operator<<(Result_6D), src/model/Types_6D.tpp:40-68, followed by the endl
 * of the apps' print loop (src/apps/em/emATTRACT.tpp:56). */
void put_result_stream(std::FILE* f, const float* r, uint32_t nmr, uint32_t nml, bool modes) {
	const double E = r[0];
	std::fprintf(f, " Energy: %.8e\n", E);
	std::fprintf(f, "%12.3f\n", E);
	if (!modes) {
		std::fprintf(f, " Gradients: ");
		for (int k = 4; k < 7; ++k) std::fprintf(f, "%20.8e", (double)r[k]);
		for (int k = 1; k < 4; ++k) std::fprintf(f, "%20.8e", (double)r[k]);
	} else {
		/* operator<<(Result_6D_Modes), src/model/Types_6D_Modes.tpp:50-90 */
		for (int k = 0; k < 6; ++k) std::fprintf(f, "%20d", 0);
		for (uint32_t m = 0; m < nmr; ++m) std::fprintf(f, "%20.8e", (double)r[7 + m]);
		for (int k = 4; k < 7; ++k) std::fprintf(f, "%20.8e", (double)r[k]);
		for (int k = 1; k < 4; ++k) std::fprintf(f, "%20.8e", (double)r[k]);
		for (uint32_t m = 0; m < nml; ++m) std::fprintf(f, "%20.8e", (double)r[17 + m]);
	}
	std::fprintf(f, "\n");
}

/* ATTRACT's .score layout as readResult parses it (src/fileIO/readFile.cpp:
 * 653-745): energy, energy-term line, then per molecule a Gradients line and,
 * with modes, a Mode gradients block.  The receptor is the fixed frame: its
 * rigid gradients are zero and its mode gradients are the receptor ones. */
void put_result_score(std::FILE* f, const float* r, uint32_t nmr, uint32_t nml, bool modes) {
	const double E = r[0];
	std::fprintf(f, " Energy: %24.16e\n", E);
	std::fprintf(f, "%12.3f%12.3f%12.3f%12.3f%12.3f%12.3f\n", E, 0.0, 0.0, 0.0, 0.0, 0.0);
	std::fprintf(f, " Gradients: ");
	for (int k = 0; k < 6; ++k) std::fprintf(f, "%26.16e", 0.0);
	std::fprintf(f, "\n");
	if (modes && nmr) {
		std::fprintf(f, " Mode gradients:\n");
		for (uint32_t m = 0; m < nmr; ++m) std::fprintf(f, "%26.16e\n", (double)r[7 + m]);
	}
	std::fprintf(f, " Gradients: ");
	for (int k = 4; k < 7; ++k) std::fprintf(f, "%26.16e", (double)r[k]);
	for (int k = 1; k < 4; ++k) std::fprintf(f, "%26.16e", (double)r[k]);
	std::fprintf(f, "\n");
	if (modes && nml) {
		std::fprintf(f, " Mode gradients:\n");
		for (uint32_t m = 0; m < nml; ++m) std::fprintf(f, "%26.16e\n", (double)r[17 + m]);
	}
}

bool is_number(const std::string& s) {
	try {
		(void)std::stod(s);
	} catch (...) {
		return false;
	}
	return true;
}

/* readResult, src/fileIO/readFile.cpp:653-745: per " Energy:" record the
 * energy, then every " Gradients:" line (6 values) and " Mode gradients:"
 * block until the next record.  A line that is neither ends the record's
 * parse with an error (the reference loops on it forever). */
std::vector<std::vector<double>> read_results_file(const char* path) {
	std::ifstream f = open_in(path);
	std::vector<std::vector<double>> out;
	std::string line;
	bool have = false;
	size_t lineno = 0;
	auto next = [&]() -> bool {
		if (!std::getline(f, line)) return false;
		++lineno;
		return true;
	};
	while (true) {
		if (!have && !next()) break;
		have = false;
		if (starts_with(line, "#")) continue;
		if (!starts_with(line, " Energy:")) continue;
		std::vector<double> rec;
		{
			std::istringstream ss(line);
			std::string tmp;
			double E = 0.0;
			ss >> tmp >> E;
			rec.push_back(E);
		}
		if (!next()) fail(std::string(path) + ": truncated result record");   /* energy terms */
		if (!next()) {
			out.push_back(rec);
			break;
		}
		bool more = true;
		while (more && !starts_with(line, " Energy:")) {
			if (starts_with(line, " Gradients:")) {
				std::istringstream ss(line);
				std::string tmp;
				ss >> tmp;
				for (int k = 0; k < 6; ++k) {
					double v = 0.0;
					ss >> v;
					rec.push_back(v);
				}
				if (!next()) { more = false; break; }
			}
			if (starts_with(line, " Mode gradients:")) {
				if (!next()) { more = false; break; }
				while (is_number(line)) {
					rec.push_back(std::stod(line));
					if (!next()) { more = false; break; }
				}
				continue;
			}
			if (more && !starts_with(line, " Energy:") && !starts_with(line, " Gradients:")) {
				if (split_ws(line).empty()) {
					if (!next()) more = false;
					continue;
				}
				fail(std::string(path) + ": line " + std::to_string(lineno) + " is not part of a result record");
			}
		}
		out.push_back(rec);
		if (!more) break;
		have = true;   /* line holds the next " Energy:" */
	}
	return out;
}

/* ------------------------------------------------------ ATTRACT .grid -- */

constexpr int kMaxAtomTypes = 99;           /* MAXATOMTYPES, src/fileIO/grid_orig.h:27 */
constexpr size_t kPotentialBytes = 4 * (kMaxAtomTypes + 1);
constexpr size_t kVoxelBytes = kPotentialBytes + 8;   /* Potential, int, short, 2 B padding */
constexpr size_t kNeighbourBytes = 8;                 /* char, 3 B padding, unsigned int */

struct GridHeader {
	gba_grid_file_info info{};
	int32_t shm_energrads = -1, shm_neighbours = -1;
	long energrad_offset = 0;   /* file offsets of the arrays */
	long neighbour_offset = 0;
	long inner_offset = 0;
	long innergridsize = 0, biggridsize = 0;
	long big_offset = 0;
};

template <class T>
void rd(std::FILE* f, T* v, size_t n, const char* path) {
	if (n && std::fread(v, sizeof(T), n, f) != n) fail(std::string("reading error in grid file ") + path);
}

/* attract::Grid::read_std, src/fileIO/grid_orig.cpp:85-300: the header and
 * the array offsets (arrays are read by the caller). */
GridHeader read_grid_header(std::FILE* f, const char* path) {
	GridHeader G;
	gba_grid_file_info& I = G.info;
	uint8_t torque = 0;
	rd(f, &torque, 1, path);
	if (torque) fail(std::string(path) + ": grid was computed as a torque grid, but it was specified as a normal grid");
	rd(f, &I.architecture, 1, path);
	if (I.architecture != 64 && I.architecture != 32)
		fail(std::string(path) + ": not an ATTRACT grid file (architecture field " + std::to_string(I.architecture) + ")");
	rd(f, &I.gridspacing, 1, path);
	rd(f, &I.gridextension, 1, path);
	rd(f, &I.plateaudis, 1, path);
	rd(f, &I.neighbourdis, 1, path);
	rd(f, I.alphabet, kMaxAtomTypes, path);
	rd(f, I.ori, 3, path);
	int32_t dims[6];
	rd(f, dims, 6, path);
	for (int a = 0; a < 3; ++a) {
		I.inner_dim[a] = dims[a];
		I.outer_dim[a] = dims[3 + a];
	}
	rd(f, &I.natoms, 1, path);
	rd(f, I.pivot, 3, path);
	rd(f, &I.nr_energrads, 1, path);
	rd(f, &G.shm_energrads, 1, path);
	if (I.nr_energrads && G.shm_energrads != -1)
		fail(std::string(path) + ": energy records in a shared-memory segment are not supported");
	G.energrad_offset = std::ftell(f);
	if (std::fseek(f, (long)I.nr_energrads * 16, SEEK_CUR) != 0) fail(std::string("reading error in grid file ") + path);
	rd(f, &I.nr_neighbours, 1, path);
	rd(f, &G.shm_neighbours, 1, path);
	if (G.shm_neighbours != -1)
		fail(std::string(path) + ": neighbour lists in a shared-memory segment are not supported");
	G.neighbour_offset = std::ftell(f);
	if (std::fseek(f, (long)I.nr_neighbours * (long)kNeighbourBytes, SEEK_CUR) != 0)
		fail(std::string("reading error in grid file ") + path);
	rd(f, &G.innergridsize, 1, path);
	G.inner_offset = std::ftell(f);
	if (std::fseek(f, G.innergridsize * (long)kVoxelBytes, SEEK_CUR) != 0)
		fail(std::string("reading error in grid file ") + path);
	rd(f, &G.biggridsize, 1, path);
	G.big_offset = std::ftell(f);
	for (int a = 0; a < 3; ++a)
		if (I.inner_dim[a] < 2 || (G.biggridsize && I.outer_dim[a] < 2))
			fail(std::string(path) + ": grid dimensions below 2");
	if ((long)I.inner_dim[0] * I.inner_dim[1] * I.inner_dim[2] != G.innergridsize)
		fail(std::string(path) + ": inner grid size does not match its dimensions");
	if (G.biggridsize && (long)I.outer_dim[0] * I.outer_dim[1] * I.outer_dim[2] != G.biggridsize)
		fail(std::string(path) + ": outer grid size does not match its dimensions");
	return G;
}

std::FILE* open_bin(const char* path, const char* mode) {
	need(path, "path");
	std::FILE* f = std::fopen(path, mode);
	if (!f) fail(std::string("failed to open file ") + path);
	return f;
}

struct FileCloser {
	std::FILE* f;
	~FileCloser() {
		if (f) std::fclose(f);
	}
};

uint32_t alphabet_size(const uint8_t* a) {
	uint32_t n = 0;
	for (int i = 0; i < kMaxAtomTypes; ++i) n += a[i] ? 1u : 0u;
	return n;
}

/* readGridFromGridFile's channel walk (src/fileIO/readFile.cpp:286-356):
 * for each alphabet type ascending then the charge slot, every voxel's record
 * (zero when the index is 0), charge channel rotated to the front. */
void fill_channels(const uint32_t* pots, long nvox, const gba_grid_file_info& I, const std::vector<float>& eg,
		float* out, const char* path) {
	int c = 1;
	for (int slot = 0; slot <= kMaxAtomTypes; ++slot) {
		if (slot < kMaxAtomTypes && !I.alphabet[slot]) continue;
		const int ch = slot == kMaxAtomTypes ? 0 : c++;
		float* dst = out + (size_t)ch * nvox * 4;
		for (long v = 0; v < nvox; ++v) {
			const uint32_t idx = pots[(size_t)v * (kMaxAtomTypes + 1) + slot];
			float* d = dst + 4 * (size_t)v;
			if (idx > 0) {
				if (idx > (uint32_t)I.nr_energrads)
					fail(std::string(path) + ": energy record index out of range at voxel " + std::to_string(v + 1));
				const float* e = &eg[4 * (size_t)(idx - 1)];
				d[0] = e[1];
				d[1] = e[2];
				d[2] = e[3];
				d[3] = e[0];
			} else {
				d[0] = d[1] = d[2] = d[3] = 0.0f;
			}
		}
	}
}

/* write_std, src/fileIO/grid_orig.cpp:303-484, for a grid whose every
 * voxel holds all channels. */
void write_grid(const char* path, const gba_grid_file_info& info, const uint32_t* alphabet, const gba_intrpl_desc& in,
		const float* in_data, const gba_intrpl_desc& out, const float* out_data, const gba_nl_desc& nl,
		const gba_neighbour_desc* nl_grid, const uint32_t* nl_list, const float* rec_xyz) {
	const uint32_t C = in.numGrids;
	if (C < 1 || out.numGrids != C) fail("gba_write_grid_file: inner and outer grids need the same channel count >= 1");
	/* channel of each file slot */
	std::vector<int> slot_channel(kMaxAtomTypes, -1);
	uint8_t mask[kMaxAtomTypes] = {0};
	for (uint32_t c = 1; c < C; ++c) {
		const uint32_t t = alphabet[c - 1];
		if (t < 1 || t > (uint32_t)kMaxAtomTypes - 1)
			fail("gba_write_grid_file: alphabet types must lie in 1..98 (99 is the dummy type)");
		if (mask[t - 1]) fail("gba_write_grid_file: alphabet lists a type twice");
		mask[t - 1] = 1;
		slot_channel[t - 1] = (int)c;
	}
	const double s = info.gridspacing;
	for (int a = 0; a < 3; ++a) {
		if ((int)in.dimN[a] != info.inner_dim[a] || (int)out.dimN[a] != info.outer_dim[a] ||
				(int)nl.dimN[a] != info.inner_dim[a])
			fail("gba_write_grid_file: descriptor dimensions differ from the header's");
		if (in.posMin[a] != info.ori[a] || nl.posMin[a] != info.ori[a])
			fail("gba_write_grid_file: inner / NL origin differs from the header's ori");
		if (out.posMin[a] != (float)((double)info.ori[a] - info.gridextension * s))
			fail("gba_write_grid_file: outer origin is not ori - gridextension * gridspacing");
	}
	if (in.gridSpacing != (float)s || out.gridSpacing != (float)(2 * s) || nl.gridSpacing != (float)s)
		fail("gba_write_grid_file: spacings differ from gridspacing (outer: twice it)");
	if (nl.dPlateau != (float)info.plateaudis) fail("gba_write_grid_file: NL plateau differs from plateaudis");

	const long Ni = (long)in.dimN[0] * in.dimN[1] * in.dimN[2];
	const long No = (long)out.dimN[0] * out.dimN[1] * out.dimN[2];
	const double nrg = (double)(Ni + No) * C;
	if (nrg > 2147483647.0) fail("gba_write_grid_file: more than 2^31 energy records");
	const int32_t nr_energrads = (int32_t)nrg;
	if (nl.numEl > 2147483647u) fail("gba_write_grid_file: more than 2^31 neighbours");

	std::FILE* f = open_bin(path, "wb");
	FileCloser fc{f};
	auto wr = [&](const void* p, size_t sz, size_t n) {
		if (n && std::fwrite(p, sz, n, f) != n) fail(std::string("write error on grid file ") + path);
	};
	const uint8_t torque = 0;
	wr(&torque, 1, 1);
	wr(&info.architecture, 2, 1);
	wr(&info.gridspacing, 8, 1);
	wr(&info.gridextension, 4, 1);
	wr(&info.plateaudis, 8, 1);
	wr(&info.neighbourdis, 8, 1);
	wr(mask, 1, kMaxAtomTypes);
	wr(info.ori, 4, 3);
	const int32_t dims[6] = {info.inner_dim[0], info.inner_dim[1], info.inner_dim[2], info.outer_dim[0],
			info.outer_dim[1], info.outer_dim[2]};
	wr(dims, 4, 6);
	wr(&info.natoms, 4, 1);
	wr(info.pivot, 8, 3);
	wr(&nr_energrads, 4, 1);
	const int32_t shm = -1;
	wr(&shm, 4, 1);
	/* energy records: per voxel the alphabet slots ascending, then the charge slot */
	std::vector<float> buf;
	auto put_records = [&](const float* data, long nvox) {
		const long chunk = 4096;
		for (long v0 = 0; v0 < nvox; v0 += chunk) {
			const long v1 = std::min(nvox, v0 + chunk);
			buf.clear();
			for (long v = v0; v < v1; ++v)
				for (int slot = 0; slot <= kMaxAtomTypes; ++slot) {
					if (slot < kMaxAtomTypes && !mask[slot]) continue;
					const int ch = slot == kMaxAtomTypes ? 0 : slot_channel[slot];
					const float* d = data + ((size_t)ch * nvox + v) * 4;
					buf.push_back(d[3]);
					buf.push_back(d[0]);
					buf.push_back(d[1]);
					buf.push_back(d[2]);
				}
			wr(buf.data(), sizeof(float), buf.size());
		}
	};
	put_records(in_data, Ni);
	put_records(out_data, No);
	/* neighbours, concatenated in voxel order */
	const int32_t nn = (int32_t)nl.numEl;
	wr(&nn, 4, 1);
	wr(&shm, 4, 1);
	std::vector<uint32_t> starts((size_t)Ni, 0);
	{
		std::vector<uint8_t> nb;
		uint64_t run = 0;
		for (long v = 0; v < Ni; ++v) {
			const uint32_t ne = nl_grid[v].numEl;
			if (ne > 32767u) fail("gba_write_grid_file: a voxel lists more than 32767 neighbours");
			if (!ne) continue;
			if ((uint64_t)nl_grid[v].idx + ne > nl.numEl) fail("gba_write_grid_file: NL descriptor beyond the list");
			starts[(size_t)v] = (uint32_t)run + 1;
			const long x = v % in.dimN[0], y = (v / in.dimN[0]) % in.dimN[1], z = v / ((long)in.dimN[0] * in.dimN[1]);
			const double cx = (double)nl.posMin[0] + x * (double)nl.gridSpacing;
			const double cy = (double)nl.posMin[1] + y * (double)nl.gridSpacing;
			const double cz = (double)nl.posMin[2] + z * (double)nl.gridSpacing;
			nb.assign((size_t)ne * kNeighbourBytes, 0);
			for (uint32_t k = 0; k < ne; ++k) {
				const uint32_t j = nl_list[nl_grid[v].idx + k];
				uint8_t type = 2;
				if (rec_xyz) {
					if (j >= (uint32_t)info.natoms) fail("gba_write_grid_file: neighbour index beyond natoms");
					const double dx = rec_xyz[j] - cx, dy = rec_xyz[info.natoms + j] - cy,
							dz = rec_xyz[2 * (size_t)info.natoms + j] - cz;
					type = dx * dx + dy * dy + dz * dz < info.plateaudis * info.plateaudis ? 1 : 2;
				}
				nb[(size_t)k * kNeighbourBytes] = type;
				std::memcpy(&nb[(size_t)k * kNeighbourBytes + 4], &j, 4);
			}
			wr(nb.data(), 1, nb.size());
			run += ne;
		}
		if (run != nl.numEl) fail("gba_write_grid_file: NL descriptors do not cover the list exactly");
	}
	/* inner voxels */
	const long innergridsize = Ni, biggridsize = No;
	wr(&innergridsize, 8, 1);
	{
		std::vector<uint8_t> vb;
		const long chunk = 1024;
		for (long v0 = 0; v0 < Ni; v0 += chunk) {
			const long v1 = std::min(Ni, v0 + chunk);
			vb.assign((size_t)(v1 - v0) * kVoxelBytes, 0);
			for (long v = v0; v < v1; ++v) {
				uint8_t* rec = &vb[(size_t)(v - v0) * kVoxelBytes];
				uint32_t pot[kMaxAtomTypes + 1] = {0};
				uint32_t r = 0;
				for (int slot = 0; slot <= kMaxAtomTypes; ++slot) {
					if (slot < kMaxAtomTypes && !mask[slot]) continue;
					pot[slot] = (uint32_t)(v * C) + r + 1;
					++r;
				}
				std::memcpy(rec, pot, kPotentialBytes);
				const int32_t nlstart = (int32_t)starts[(size_t)v];
				const int16_t nr = (int16_t)nl_grid[v].numEl;
				std::memcpy(rec + kPotentialBytes, &nlstart, 4);
				std::memcpy(rec + kPotentialBytes + 4, &nr, 2);
			}
			wr(vb.data(), 1, vb.size());
		}
	}
	wr(&biggridsize, 8, 1);
	{
		std::vector<uint32_t> pb;
		const long chunk = 1024;
		for (long v0 = 0; v0 < No; v0 += chunk) {
			const long v1 = std::min(No, v0 + chunk);
			pb.assign((size_t)(v1 - v0) * (kMaxAtomTypes + 1), 0);
			for (long v = v0; v < v1; ++v) {
				uint32_t r = 0;
				for (int slot = 0; slot <= kMaxAtomTypes; ++slot) {
					if (slot < kMaxAtomTypes && !mask[slot]) continue;
					pb[(size_t)(v - v0) * (kMaxAtomTypes + 1) + slot] = (uint32_t)((Ni + v) * C) + r + 1;
					++r;
				}
			}
			wr(pb.data(), 4, pb.size());
		}
	}
}

}  // namespace

extern "C" {

const char* gba_io_last_error(void) { return g_io_error.c_str(); }

int gba_read_pdb(const char* path, uint32_t* n, float* xyz, uint32_t* type, float* charge, uint32_t cap) {
	return guarded([&] {
		need(n, "n");
		const PdbBeads B = read_pdb_file(path);
		const size_t nb = B.t.size();
		if (nb > 0xffffffffu) fail("too many beads");
		*n = (uint32_t)nb;
		if (!xyz && !type && !charge) return;
		if (nb > cap) fail("gba_read_pdb: capacity " + std::to_string(cap) + " below " + std::to_string(nb) + " beads");
		if (xyz) {
			std::copy(B.x.begin(), B.x.end(), xyz);
			std::copy(B.y.begin(), B.y.end(), xyz + nb);
			std::copy(B.z.begin(), B.z.end(), xyz + 2 * nb);
		}
		if (type) std::copy(B.t.begin(), B.t.end(), type);
		if (charge) std::copy(B.q.begin(), B.q.end(), charge);
	});
}

/* readParamTableFromFile, src/fileIO/readFile.cpp:431-520 */
int gba_read_params(const char* path, uint32_t* num_types, gba_ffparam* table, uint32_t cap, int32_t* potshape,
		float* swi_on, float* swi_off) {
	return guarded([&] {
		need(num_types, "num_types");
		std::ifstream f = open_in(path);
		unsigned shape = 0, T = 0;
		float on = 0.f, off = 0.f;
		if (!(f >> shape >> T >> on >> off)) fail(std::string(path) + ": bad parameter file header");
		if (shape != 8 && shape != 12)
			fail("unknown potential shape " + std::to_string(shape) + " in file: " + path);
		if (T == 0 || T > 4096) fail(std::string(path) + ": implausible type count " + std::to_string(T));
		*num_types = T;
		if (potshape) *potshape = shape == 8 ? GBA_POTSHAPE_8_6 : GBA_POTSHAPE_12_6;
		if (swi_on) *swi_on = on;
		if (swi_off) *swi_off = off;
		if (!table) return;
		if ((uint64_t)T * T > cap) fail("gba_read_params: table capacity below T*T");
		const size_t TT = (size_t)T * T;
		std::vector<gba_ffparam> P(TT);
		for (size_t k = 0; k < TT; ++k)
			if (!(f >> P[k].rc)) fail(std::string(path) + ": truncated rc matrix");
		for (size_t k = 0; k < TT; ++k)
			if (!(f >> P[k].ac)) fail(std::string(path) + ": truncated ac matrix");
		for (size_t k = 0; k < TT; ++k)
			if (!(f >> P[k].ipon)) fail(std::string(path) + ": truncated ipon matrix");
		for (size_t k = 0; k < TT; ++k) {
			gba_ffparam& p = P[k];
			const float rbc = p.rc, abc = p.ac;
			/* std::pow(float, unsigned) promotes both to double */
			p.rc = (float)(abc * std::pow((double)rbc, (double)shape));
			p.ac = (float)(abc * std::pow((double)rbc, 6.0));
			if (shape == 8) {
				if (p.ac > 0 && p.rc > 0) {
					p.emin = (float)(-27.0f * std::pow((double)p.ac, 4.0) / (256.0f * std::pow((double)p.rc, 3.0)));
					p.rmin2 = 4.0f * p.rc / (3.0f * p.ac);
				} else {
					p.emin = 0;
					p.rmin2 = 0;
				}
			} else {
				p.emin = (float)(-0.25 * abc);
				p.rmin2 = 1.25992105f * rbc * rbc;
			}
			table[k] = p;
		}
	});
}

/* readGridAlphabetFromFile, src/fileIO/readFile.cpp:901-926 */
int gba_read_alphabet(const char* path, uint32_t* n, uint32_t* types, uint32_t cap) {
	return guarded([&] {
		need(n, "n");
		std::ifstream f = open_in(path);
		std::vector<uint32_t> v;
		std::string line;
		while (std::getline(f, line)) {
			std::istringstream iss(line);
			int key = 0;
			if (!(iss >> key) || key < 0) fail(std::string("grid alphabet file ") + path + " has an invalid line");
			v.push_back((uint32_t)key);
		}
		*n = (uint32_t)v.size();
		if (!types) return;
		if (v.size() > cap) fail("gba_read_alphabet: capacity too small");
		std::copy(v.begin(), v.end(), types);
	});
}

int gba_read_dof(const char* path, gba_dof_header* header, uint32_t* num_structures, uint32_t* num_molecules,
		float* values, int32_t* counts, size_t cap) {
	return guarded([&] {
		need(num_structures, "num_structures");
		need(num_molecules, "num_molecules");
		const DofFile D = read_dof_file(path);
		if (header) *header = D.h;
		const uint32_t M = D.molecules;
		const size_t S = M ? D.mol[0].size() : 0;
		*num_molecules = M;
		*num_structures = (uint32_t)S;
		if (!values && !counts) return;
		if (S * M > cap) fail("gba_read_dof: capacity below structures * molecules");
		for (size_t s = 0; s < S; ++s)
			for (uint32_t m = 0; m < M; ++m) {
				const std::vector<double>& v = D.mol[m][s];
				if (values) {
					float* o = values + (s * M + m) * kDofValues;
					for (int k = 0; k < kDofValues; ++k) o[k] = k < (int)v.size() ? (float)v[k] : 0.0f;
				}
				if (counts) counts[s * M + m] = (int32_t)v.size();
			}
	});
}

int gba_write_dof(const char* path, const gba_dof_header* header, uint32_t num_structures, uint32_t num_molecules,
		const float* values, const int32_t* counts, const float* energies) {
	return guarded([&] {
		need(header, "header");
		need(values, "values");
		if (num_molecules == 0) fail("gba_write_dof: no molecules");
		std::FILE* f = open_bin(path, "w");
		FileCloser fc{f};
		if (header->auto_pivot) {
			std::fprintf(f, "#pivot auto\n");
		} else {
			if (header->num_pivots > 16) fail("gba_write_dof: more than 16 pivots");
			for (uint32_t k = 0; k < header->num_pivots; ++k)
				std::fprintf(f, "#pivot %u %.9g %.9g %.9g\n", k + 1, (double)header->pivots[k][0],
						(double)header->pivots[k][1], (double)header->pivots[k][2]);
		}
		std::fprintf(f, "#centered receptor: %s\n", header->centered_receptor ? "true" : "false");
		std::fprintf(f, "#centered ligands: %s\n", header->centered_ligands ? "true" : "false");
		for (uint32_t s = 0; s < num_structures; ++s) {
			std::fprintf(f, "#%u\n", s + 1);
			if (energies) std::fprintf(f, "## Energy: %.9g\n", (double)energies[s]);
			for (uint32_t m = 0; m < num_molecules; ++m) {
				const size_t line = (size_t)s * num_molecules + m;
				const int nv = counts ? counts[line] : 6;
				if (nv < 6 || nv > kDofValues) fail("gba_write_dof: a line needs 6..16 values");
				const float* v = values + line * kDofValues;
				for (int k = 0; k < nv; ++k) std::fprintf(f, " %.9g", (double)v[k]);
				std::fprintf(f, "\n");
			}
		}
		if (std::ferror(f)) fail(std::string("write error on ") + path);
	});
}

int gba_map_types(const uint32_t* alphabet, uint32_t n_alphabet, const uint32_t* types_in, uint32_t n,
		uint32_t* types_out, uint32_t* mapped_out) {
	return guarded([&] {
		if (n == 0) return;
		need(types_in, "types_in");
		if (n_alphabet) need(alphabet, "alphabet");
		/* createTypeMapFromVector: later entries overwrite earlier ones */
		std::vector<int64_t> chan(100, -1);
		std::vector<std::pair<uint32_t, uint32_t>> extra;
		for (uint32_t i = 0; i < n_alphabet; ++i) {
			const uint32_t key = alphabet[i], val = key == 99 ? 0 : i + 1;
			if (key < 100) chan[key] = val;
			else extra.emplace_back(key, val);
		}
		chan[0] = 0;
		for (uint32_t k = 0; k < n; ++k) {
			const uint32_t raw = types_in[k];
			if (raw > 99) fail("gba_map_types: type " + std::to_string(raw) + " is not in the default type map");
			const uint32_t t = raw == 99 ? 0 : raw;
			const int64_t c = chan[t];
			if (c < 0) fail("gba_map_types: type " + std::to_string(t) + " is not in the grid alphabet");
			if (types_out) types_out[k] = t;
			if (mapped_out) mapped_out[k] = (uint32_t)c;
		}
	});
}

/* Protein::auto_pivotize, src/model/Protein.tpp:145-157 */
int gba_auto_pivot(const float* xyz, uint32_t n, float pivot[3]) {
	return guarded([&] {
		need(xyz, "xyz");
		need(pivot, "pivot");
		if (n == 0) fail("gba_auto_pivot: no beads");
		float p[3] = {0.f, 0.f, 0.f};
		for (int a = 0; a < 3; ++a)
			for (uint32_t i = 0; i < n; ++i) p[a] += xyz[(size_t)a * n + i];
		const float d = (float)(double)n;
		for (int a = 0; a < 3; ++a) pivot[a] = p[a] / d;
	});
}

int gba_dof_glob2rec(void* dof_rec, void* dof_lig, size_t n, size_t stride, const float pivot_rec[3],
		const float pivot_lig[3], int32_t centered_rec, int32_t centered_lig) {
	return guarded([&] {
		if (n == 0) return;
		need(dof_rec, "dof_rec");
		need(dof_lig, "dof_lig");
		need(pivot_rec, "pivot_rec");
		need(pivot_lig, "pivot_lig");
		if (stride < sizeof(gba_dof6d)) fail("gba_dof_glob2rec: stride below sizeof(gba_dof6d)");
		for (size_t i = 0; i < n; ++i) {
			gba_dof6d r, l;
			std::memcpy(&r, (char*)dof_rec + i * stride, sizeof r);
			std::memcpy(&l, (char*)dof_lig + i * stride, sizeof l);
			glob2rec_one(r, l, pivot_rec, pivot_lig, centered_rec != 0, centered_lig != 0);
			std::memcpy((char*)dof_rec + i * stride, &r, sizeof r);
			std::memcpy((char*)dof_lig + i * stride, &l, sizeof l);
		}
	});
}

int gba_write_results(const char* path, int32_t append, int32_t style, const void* results, size_t n,
		uint32_t n_modes_rec, uint32_t n_modes_lig) {
	return guarded([&] {
		if (n && !results) fail("null argument: results");
		if (style != GBA_RESULTS_STREAM && style != GBA_RESULTS_SCORE)
			fail("gba_write_results: style must be GBA_RESULTS_STREAM or GBA_RESULTS_SCORE");
		if (n_modes_rec > GBA_MODES_MAX || n_modes_lig > GBA_MODES_MAX) fail("gba_write_results: more than 10 modes");
		const bool modes = n_modes_rec + n_modes_lig > 0;
		std::FILE* f = open_bin(path, append ? "a" : "w");
		FileCloser fc{f};
		const size_t stride = modes ? sizeof(gba_result6d_modes) / 4 : sizeof(gba_result6d) / 4;
		for (size_t i = 0; i < n; ++i) {
			const float* r = (const float*)results + i * stride;
			if (style == GBA_RESULTS_SCORE) put_result_score(f, r, n_modes_rec, n_modes_lig, modes);
			else put_result_stream(f, r, n_modes_rec, n_modes_lig, modes);
		}
		if (std::ferror(f)) fail(std::string("write error on ") + path);
	});
}

int gba_read_results(const char* path, size_t* n, uint32_t* width, double* out, int32_t* counts, size_t cap,
		uint32_t stride) {
	return guarded([&] {
		need(n, "n");
		const std::vector<std::vector<double>> R = read_results_file(path);
		size_t w = 0;
		for (const auto& r : R) w = std::max(w, r.size());
		*n = R.size();
		if (width) *width = (uint32_t)w;
		if (!out && !counts) return;
		if (R.size() > cap) fail("gba_read_results: capacity below the record count");
		if (out && stride < w) fail("gba_read_results: stride below the widest record");
		for (size_t i = 0; i < R.size(); ++i) {
			if (out) {
				for (size_t k = 0; k < stride; ++k) out[i * stride + k] = k < R[i].size() ? R[i][k] : 0.0;
			}
			if (counts) counts[i] = (int32_t)R[i].size();
		}
	});
}

int gba_grid_file_info_read(const char* path, gba_grid_file_info* info) {
	return guarded([&] {
		need(info, "info");
		std::FILE* f = open_bin(path, "rb");
		FileCloser fc{f};
		*info = read_grid_header(f, path).info;
	});
}

int gba_read_grid_file(const char* path, gba_intrpl_desc* inner, float* inner_data, gba_intrpl_desc* outer,
		float* outer_data, gba_nl_desc* nl, gba_neighbour_desc* nl_grid, uint32_t* nl_list) {
	return guarded([&] {
		std::FILE* f = open_bin(path, "rb");
		FileCloser fc{f};
		const GridHeader G = read_grid_header(f, path);
		const gba_grid_file_info& I = G.info;
		const uint32_t C = alphabet_size(I.alphabet) + 1;
		const long Ni = G.innergridsize, No = (long)I.outer_dim[0] * I.outer_dim[1] * I.outer_dim[2];
		if (inner) {
			inner->numGrids = C;
			inner->gridSpacing = (float)I.gridspacing;
			for (int a = 0; a < 3; ++a) {
				inner->dimN[a] = (uint32_t)I.inner_dim[a];
				inner->posMin[a] = I.ori[a];
			}
		}
		if (outer) {
			outer->numGrids = C;
			outer->gridSpacing = (float)(2 * I.gridspacing);
			for (int a = 0; a < 3; ++a) {
				outer->dimN[a] = (uint32_t)I.outer_dim[a];
				outer->posMin[a] = (float)((double)I.ori[a] - I.gridextension * I.gridspacing);
			}
		}
		if (nl) {
			for (int a = 0; a < 3; ++a) {
				nl->dimN[a] = (uint32_t)I.inner_dim[a];
				nl->posMin[a] = I.ori[a];
			}
			nl->gridSpacing = (float)I.gridspacing;
			nl->dPlateau = (float)I.plateaudis;
			nl->numEl = (uint32_t)I.nr_neighbours;
		}
		std::vector<float> eg;
		std::vector<uint32_t> pots;
		if (inner_data || outer_data) {
			eg.resize((size_t)I.nr_energrads * 4);
			std::fseek(f, G.energrad_offset, SEEK_SET);
			rd(f, eg.data(), eg.size(), path);
		}
		if (inner_data || nl_grid) {
			std::vector<uint8_t> vox((size_t)Ni * kVoxelBytes);
			std::fseek(f, G.inner_offset, SEEK_SET);
			rd(f, vox.data(), vox.size(), path);
			if (inner_data) {
				pots.resize((size_t)Ni * (kMaxAtomTypes + 1));
				for (long v = 0; v < Ni; ++v)
					std::memcpy(&pots[(size_t)v * (kMaxAtomTypes + 1)], &vox[(size_t)v * kVoxelBytes], kPotentialBytes);
				fill_channels(pots.data(), Ni, I, eg, inner_data, path);
			}
			if (nl_grid) {
				for (long v = 0; v < Ni; ++v) {
					int32_t start;
					int16_t nr;
					uint32_t elec;
					std::memcpy(&start, &vox[(size_t)v * kVoxelBytes + kPotentialBytes], 4);
					std::memcpy(&nr, &vox[(size_t)v * kVoxelBytes + kPotentialBytes + 4], 2);
					std::memcpy(&elec, &vox[(size_t)v * kVoxelBytes + 4 * kMaxAtomTypes], 4);
					/* read_std checks voxels that hold potentials; a negative count is never valid */
					if (nr < 0 || (elec && ((start == 0) != (nr == 0) || (long)start + nr - 1 > I.nr_neighbours)))
						fail(std::string("reading error in ") + path + ", innergrid voxel " + std::to_string(v + 1) +
								" neighbourlist");
					nl_grid[v].numEl = (uint32_t)nr;
					nl_grid[v].idx = (uint32_t)start - 1u;   /* as readGridFromGridFile sets it */
				}
			}
		}
		if (outer_data) {
			if (G.biggridsize) {
				pots.assign((size_t)No * (kMaxAtomTypes + 1), 0);
				std::fseek(f, G.big_offset, SEEK_SET);
				rd(f, pots.data(), pots.size(), path);
				fill_channels(pots.data(), No, I, eg, outer_data, path);
			} else {
				std::fill(outer_data, outer_data + (size_t)C * No * 4, 0.0f);
			}
		}
		if (nl_list) {
			std::vector<uint8_t> nb((size_t)I.nr_neighbours * kNeighbourBytes);
			std::fseek(f, G.neighbour_offset, SEEK_SET);
			rd(f, nb.data(), nb.size(), path);
			for (int32_t k = 0; k < I.nr_neighbours; ++k) std::memcpy(&nl_list[k], &nb[(size_t)k * kNeighbourBytes + 4], 4);
		}
	});
}

int gba_write_grid_file(const char* path, const gba_grid_file_info* info, const uint32_t* alphabet,
		const gba_intrpl_desc* inner, const float* inner_data, const gba_intrpl_desc* outer, const float* outer_data,
		const gba_nl_desc* nl, const gba_neighbour_desc* nl_grid, const uint32_t* nl_list, const float* rec_xyz) {
	return guarded([&] {
		need(info, "info");
		need(inner, "inner");
		need(inner_data, "inner_data");
		need(outer, "outer");
		need(outer_data, "outer_data");
		need(nl, "nl");
		need(nl_grid, "nl_grid");
		if (nl->numEl) need(nl_list, "nl_list");
		if (inner->numGrids > 1) need(alphabet, "alphabet");
		write_grid(path, *info, alphabet, *inner, inner_data, *outer, outer_data, *nl, nl_grid, nl_list, rec_xyz);
	});
}

}  // extern "C"
