/*
 * attract_oracle.cpp -- CPU oracle (test infrastructure, see oracle.h).
 *
 * A restatement, in plain C++, of gpuATTRACT 2.0's CPU energy path.  Every
 * function cites the reference lines it follows.  The FP32 instantiation keeps
 * the reference's exact operation order and its float/double promotions
 * (double literals such as 6.0 and 0.01, double divisions assigned to float),
 * and is built with -ffp-contract=off so no FMA is introduced on any host.
 */
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <type_traits>
#include <vector>

namespace {

/* ------------------------------------------------------------------------ */
/* rotation / torque matrices                                               */
/* ------------------------------------------------------------------------ */

/* Source of sin/cos in FP32.  The reference calls the C library's sinf/cosf,
 * whose last-ulp rounding the C standard leaves to the implementation (glibc
 * misrounds a few percent of arguments by one ulp).  With exact set (test
 * infrastructure, orc_set_exact_sincos) the FP32 restatement takes the
 * correctly rounded values, (float)sin((double)x), instead. */
std::atomic<int> g_exact_sincos{0};

inline float osin(float a) { return g_exact_sincos.load(std::memory_order_relaxed) ? (float)std::sin((double)a) : std::sin(a); }
inline float ocos(float a) { return g_exact_sincos.load(std::memory_order_relaxed) ? (float)std::cos((double)a) : std::cos(a); }
inline double osin(double a) { return std::sin(a); }
inline double ocos(double a) { return std::cos(a); }

/* euler2rotmat, src/model/matrixFunctions.h:40-77 (row-major 3x3) */
template <typename R>
void euler2rotmat(R phi, R ssi, R rot, R m[9]) {
	R cSSI = ocos(ssi);
	R cPHI = ocos(phi);
	R sSSI = osin(ssi);
	R sPHI = osin(phi);
	R cSSI_cPHI = cSSI * cPHI;
	R cSSI_sPHI = cSSI * sPHI;
	R sSSI_cPHI = sSSI * cPHI;
	R sSSI_sPHI = sSSI * sPHI;
	R cROT = ocos(rot);
	R sROT = osin(rot);
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

/* euler2torquemat, src/model/matrixFunctions.h:81-127; t[k][j][l] */
template <typename R>
void euler2torquemat(R phi, R ssi, R rot, R t[3][3][3]) {
	R cSSI = ocos(ssi);
	R cPHI = ocos(phi);
	R sSSI = osin(ssi);
	R sPHI = osin(phi);
	R cSSI_cPHI = cSSI * cPHI;
	R cSSI_sPHI = cSSI * sPHI;
	R sSSI_cPHI = sSSI * cPHI;
	R sSSI_sPHI = sSSI * sPHI;
	R cROT = ocos(rot);
	R sROT = osin(rot);
	t[0][0][0] = -cROT * cSSI_sPHI + sROT * cPHI;
	t[0][0][1] = -sROT * cSSI_sPHI - cROT * cPHI;
	t[0][0][2] = -sSSI_sPHI;
	t[1][0][0] = cROT * cSSI_cPHI + sROT * sPHI;
	t[1][0][1] = sROT * cSSI_cPHI - cROT * sPHI;
	t[1][0][2] = sSSI_cPHI;
	t[2][0][0] = 0.0;
	t[2][0][1] = 0.0;
	t[2][0][2] = 0.0;
	t[0][1][0] = -cROT * sSSI_cPHI;
	t[0][1][1] = -sROT * sSSI_cPHI;
	t[0][1][2] = cSSI_cPHI;
	t[1][1][0] = -cROT * sSSI_sPHI;
	t[1][1][1] = -sROT * sSSI_sPHI;
	t[1][1][2] = cSSI_sPHI;
	t[2][1][0] = -cROT * cSSI;
	t[2][1][1] = -sROT * cSSI;
	t[2][1][2] = -sSSI;
	t[0][2][0] = -sROT * cSSI_cPHI + cROT * sPHI;
	t[0][2][1] = cROT * cSSI_cPHI + sROT * sPHI;
	t[0][2][2] = 0.0;
	t[1][2][0] = -sROT * cSSI_sPHI - cROT * cPHI;
	t[1][2][1] = cROT * cSSI_sPHI - sROT * cPHI;
	t[1][2][2] = 0.0;
	t[2][2][0] = sROT * sSSI;
	t[2][2][1] = -cROT * sSSI;
	t[2][2][2] = 0.0;
}

/* RotMat * Vec3, src/commons/RotMat.h:170-176 */
template <typename R>
inline void matvec(const R m[9], R x, R y, R z, R& ox, R& oy, R& oz) {
	ox = m[0] * x + m[1] * y + m[2] * z;
	oy = m[3] * x + m[4] * y + m[5] * z;
	oz = m[6] * x + m[7] * y + m[8] * z;
}

/* RotMat::getInv (transpose), src/commons/RotMat.h:119-131 */
template <typename R>
inline void transpose(const R m[9], R t[9]) {
	t[0] = m[0]; t[1] = m[3]; t[2] = m[6];
	t[3] = m[1]; t[4] = m[4]; t[5] = m[7];
	t[6] = m[2]; t[7] = m[5]; t[8] = m[8];
}

/* ------------------------------------------------------------------------ */
/* force field, src/model/forcefield.h                                     */
/* ------------------------------------------------------------------------ */

/* Wide type used where the reference writes a double literal or a double
 * local: double for both instantiations. */
typedef double W;

/* LJPotForce, src/model/forcefield.h:30-83 (swi fixed to 1 by its callers) */
template <typename R>
inline void lj_pot_force(R dr2, R dr2_inv, R dx, R dy, R dz, const gba_ffparam& p,
		int potshape, R& fx, R& fy, R& fz, R& energy) {
	const R alen = (R)p.ac;
	const R rlen = (R)p.rc;
	const R ivor = (R)p.ipon;     /* REAL const& bound to an int member */
	const R rmin2 = (R)p.rmin2;
	const R emin = (R)p.emin;
	const R swi = 1;
	const R rr23 = dr2_inv * dr2_inv * dr2_inv;
	R rrd, shapedelta;
	if (potshape == GBA_POTSHAPE_8_6) {
		rrd = dr2_inv;
		shapedelta = 2;
	} else {
		rrd = rr23;
		shapedelta = 6;
	}
	R rep = rlen * rrd;
	R vlj = (rep - alen) * rr23;
	if (dr2 < rmin2) {
		energy = swi * (vlj + (ivor - 1) * emin);
		R fb_swi = (R)((6.0 * (W)vlj + (W)(shapedelta * (rep * rr23))) * (W)swi);
		fx = fb_swi * dx;
		fy = fb_swi * dy;
		fz = fb_swi * dz;
	} else {
		R swi_ivor = swi * ivor;
		energy = swi_ivor * vlj;
		R ivor_fb_swi = (R)((W)swi_ivor * (6.0 * (W)vlj + (W)(shapedelta * (rep * rr23))));
		fx = ivor_fb_swi * dx;
		fy = ivor_fb_swi * dy;
		fz = ivor_fb_swi * dz;
	}
}

/* ChargePotForce, src/model/forcefield.h:87-146 (swi = 1) */
template <typename R>
inline void charge_pot_force(R dr2_inv, R dx, R dy, R dz, R chargeLigRec, int dielec,
		R& fx, R& fy, R& fz, R& energy) {
	const R swi = 1;
	R dd;
	if (dielec == GBA_DIELEC_CONSTANT)
		dd = (R)((W)std::sqrt(dr2_inv) - 1.0 / 50.0);
	else
		dd = (R)((W)dr2_inv - 1.0 / (50.0 * 50.0));
	if (dd < 0) dd = 0;
	energy = swi * chargeLigRec * dd;
	if (dd <= 0) {
		fx = 0; fy = 0; fz = 0;
		return;
	}
	if (dielec == GBA_DIELEC_CONSTANT) {
		W et2 = (W)(swi * chargeLigRec * std::sqrt(dr2_inv));
		fx = (R)(et2 * (W)dx);
		fy = (R)(et2 * (W)dy);
		fz = (R)(et2 * (W)dz);
	} else {
		W et2 = (W)(swi * chargeLigRec * dr2_inv);
		fx = (R)(2 * et2 * (W)dx);
		fy = (R)(2 * et2 * (W)dy);
		fz = (R)(2 * et2 * (W)dz);
	}
}

/* ------------------------------------------------------------------------ */
/* grids                                                                     */
/* ------------------------------------------------------------------------ */

/* IntrplGrid, src/model/IntrplGrid.h + IntrplGrid.tpp:29-41 (derived members) */
template <typename R>
struct IGrid {
	uint32_t dimN[3];
	R pos[3], maxDim[3];
	R dVox, dVox_inv, voxelVol, voxelVol_inv;
	const float* data;
	void init(const gba_intrpl_desc& d, const float* g) {
		for (int a = 0; a < 3; ++a) { dimN[a] = d.dimN[a]; pos[a] = (R)d.posMin[a]; }
		dVox = (R)d.gridSpacing;
		voxelVol = dVox * dVox * dVox;
		voxelVol_inv = (R)1.f / voxelVol;
		dVox_inv = (R)1.f / dVox;
		for (int a = 0; a < 3; ++a) maxDim[a] = pos[a] + (R)(dimN[a] - 1) * dVox;
		data = g;
	}
	/* outOfBounds_byPos, src/model/IntrplGrid.h:113-117, as a negated inside
	 * test: the same answer for every finite position, and a NaN position
	 * counts as outside (the reference's comparisons count it as inside and
	 * index the grid with it -- undefined behaviour; a minimization whose mode
	 * amplitudes overflow reaches such positions).  The kernels test alike. */
	bool out_of_bounds(R x, R y, R z) const {
		return !((x >= pos[0]) && (x <= maxDim[0]) && (y >= pos[1]) && (y <= maxDim[1]) &&
				(z >= pos[2]) && (z <= maxDim[2]));
	}
};

/* NLGrid, src/model/NLGrid.h + NLGrid.tpp:29-51 (derived members, ratio table) */
template <typename R>
struct NGrid {
	uint32_t dimN[3];
	R pos[3], maxDim[3];
	R dVox, dVox_inv, dPlateau2, dPlateau2_inv;
	const gba_neighbour_desc* grid;
	const uint32_t* list;
	std::vector<R> ratio;
	void init(const gba_nl_desc& d, const gba_neighbour_desc* g, const uint32_t* l) {
		for (int a = 0; a < 3; ++a) { dimN[a] = d.dimN[a]; pos[a] = (R)d.posMin[a]; }
		dVox = (R)d.gridSpacing;
		R dPlateau = (R)d.dPlateau;
		dPlateau2 = dPlateau * dPlateau;
		dPlateau2_inv = 1 / dPlateau2;
		dVox_inv = 1 / dVox;
		for (int a = 0; a < 3; ++a) maxDim[a] = pos[a] + (R)(dimN[a] - 1) * dVox;
		int size = int(10000 * dPlateau2);
		ratio.resize(size + 1);
		for (int n = 0; n <= size; n++) {
			double d2 = ((n + 0.5) / 10000);
			ratio[n] = (R)std::sqrt(d2 / (double)dPlateau2);
		}
		grid = g;
		list = l;
	}
	/* outOfBounds(x,y,z), src/model/NLGrid.h:128-133 */
	/* NLGrid::outOfBounds, src/model/NLGrid.h:128-133, NaN-safe as above */
	bool out_of_bounds(R x, R y, R z) const {
		return !((x >= pos[0]) && (x <= maxDim[0]) && (y >= pos[1]) && (y <= maxDim[1]) &&
				(z >= pos[2]) && (z <= maxDim[2]));
	}
	/* getIndex, src/model/NLGrid.h:100-108 */
	void index(R x, R y, R z, int& ix, int& iy, int& iz) const {
		ix = (int)std::round((x - pos[0]) * dVox_inv);
		iy = (int)std::round((y - pos[1]) * dVox_inv);
		iz = (int)std::round((z - pos[2]) * dVox_inv);
	}
	/* getRatio, src/model/NLGrid.h:141-143 */
	R get_ratio(R d2) const { return ratio[int(d2 * 10000)]; }
};

template <typename R>
struct Sys {
	IGrid<R> inner, outer;
	NGrid<R> nl;
	bool has_nl;
	void init(const orc_grid* g) {
		inner.init(g->inner, g->inner_data);
		outer.init(g->outer, g->outer_data);
		has_nl = g->nl_grid != nullptr;
		if (has_nl) nl.init(g->nl, g->nl_grid, g->nl_list);
	}
};

template <typename R> struct R4 { R x, y, z, w; };

/* IntrplGrid::getIndex + getVoxelByIndex + trilinearInterpolation,
 * src/model/IntrplGrid.h:96-104,130-163, src/model/trilinIntrpl.h:29-66.
 * FP32: the octet is combined in float exactly as the reference
 * (float4 * weight, left-to-right float4 sums); FP64: all in double. */
template <typename R>
R4<R> interpolate_channel(const IGrid<R>& g, R px, R py, R pz, int ix, int iy, int iz,
		uint32_t type) {
	R minx = ix * g.dVox + g.pos[0];
	R miny = iy * g.dVox + g.pos[1];
	R minz = iz * g.dVox + g.pos[2];
	R maxx = minx + g.dVox, maxy = miny + g.dVox, maxz = minz + g.dVox;
	size_t idxGrid = (size_t)type * g.dimN[2] * g.dimN[1] * g.dimN[0];
	idxGrid += (size_t)g.dimN[0] * (iz * g.dimN[1] + iy) + ix;
	const float* D = g.data;
	auto V = [&](size_t k) { return R4<R>{(R)D[4 * k], (R)D[4 * k + 1], (R)D[4 * k + 2], (R)D[4 * k + 3]}; };
	R4<R> d000 = V(idxGrid), d100 = V(idxGrid + 1), d010 = V(idxGrid + g.dimN[0]),
			d110 = V(idxGrid + g.dimN[0] + 1);
	size_t up = idxGrid + (size_t)g.dimN[0] * g.dimN[1];
	R4<R> d001 = V(up), d101 = V(up + 1), d011 = V(up + g.dimN[0]), d111 = V(up + g.dimN[0] + 1);

	R pmn_x = px - minx, pmn_y = py - miny, pmn_z = pz - minz;
	R pmx_x = maxx - px, pmx_y = maxy - py, pmx_z = maxz - pz;
	R tmpMax_xy = pmx_x * pmx_y;
	R tmpMin_xy = pmn_x * pmn_y;
	R w000 = tmpMax_xy * pmx_z;
	R w100 = (pmn_x * pmx_y) * pmx_z;
	R w010 = (pmx_x * pmn_y) * pmx_z;
	R w001 = tmpMax_xy * pmn_z;
	R w101 = (pmn_x * pmx_y) * pmn_z;
	R w011 = (pmx_x * pmn_y) * pmn_z;
	R w110 = tmpMin_xy * pmx_z;
	R w111 = tmpMin_xy * pmn_z;
	R4<R> out;
#define ORC_TRI(c) out.c = d000.c * w000 + d100.c * w100 + d010.c * w010 + d001.c * w001 + \
		d101.c * w101 + d011.c * w011 + d110.c * w110 + d111.c * w111; out.c = out.c * g.voxelVol_inv;
	ORC_TRI(x) ORC_TRI(y) ORC_TRI(z) ORC_TRI(w)
#undef ORC_TRI
	return out;
}

/* interpolate, src/model/interpolation.h:27-53 */
template <typename R>
R4<R> interpolate(const IGrid<R>& g, R px, R py, R pz, uint32_t type, R charge, bool& charged) {
	int ix = (int)std::min((unsigned)std::floor((px - g.pos[0]) * g.dVox_inv), g.dimN[0] - 2);
	int iy = (int)std::min((unsigned)std::floor((py - g.pos[1]) * g.dVox_inv), g.dimN[1] - 2);
	int iz = (int)std::min((unsigned)std::floor((pz - g.pos[2]) * g.dVox_inv), g.dimN[2] - 2);
	R4<R> pot = interpolate_channel(g, px, py, pz, ix, iy, iz, type);
	charged = std::fabs(charge) > (R)0.001;
	if (charged) {
		R4<R> el = interpolate_channel(g, px, py, pz, ix, iy, iz, 0);
		el.x = el.x * charge; el.y = el.y * charge; el.z = el.z * charge; el.w = el.w * charge;
		pot.x = pot.x + el.x; pot.y = pot.y + el.y; pot.z = pot.z + el.z; pot.w = pot.w + el.w;
	}
	return pot;
}

struct Stats {
	orc_pose_stats* s;
	void add_E(double e) { if (s) s->abs_E += std::fabs(e); }
	void add_F(double x, double y, double z) { if (s) s->abs_F += std::sqrt(x * x + y * y + z * z); }
};

/* potForce, src/model/interpolation.h:57-101 (one protein, both grids) */
template <typename R>
void pot_force(const Sys<R>& S, const orc_protein* prot, const R* X, const R* Y, const R* Z,
		R* fx, R* fy, R* fz, R* E, Stats st) {
	for (unsigned i = 0; i < prot->n; ++i) {
		unsigned type = prot->mapped[i];
		R4<R> pot = {0, 0, 0, 0};
		if (type != 0) {
			R px = X[i], py = Y[i], pz = Z[i];
			R charge = (R)prot->charge[i];
			bool charged = false, used = false;
			if (S.inner.out_of_bounds(px, py, pz)) {
				if (!S.outer.out_of_bounds(px, py, pz)) {
					pot = interpolate(S.outer, px, py, pz, type, charge, charged);
					used = true;
				}
			} else {
				pot = interpolate(S.inner, px, py, pz, type, charge, charged);
				used = true;
			}
			if (used && st.s) {
				st.s->n_grid++;
				if (charged) st.s->n_grid_charged++;
				st.add_E(pot.w);
				st.add_F(pot.x, pot.y, pot.z);
			}
		}
		fx[i] = pot.x; fy[i] = pot.y; fz[i] = pot.z; E[i] = pot.w;
	}
}

/* NLPotForce, src/model/neighborlist.h:29-168 (rigid) and
 * src/model/neighborlist_modes.h:21-206 (modes: receptor positions given,
 * receptor reaction forces accumulated when outRec != nullptr) */
template <typename R>
void nl_pot_force(const Sys<R>& S, const orc_protein* rec, const orc_protein* lig,
		const orc_params* par, const R* RX, const R* RY, const R* RZ,
		const R* LX, const R* LY, const R* LZ, R* ofx, R* ofy, R* ofz, R* oE,
		R* rfx, R* rfy, R* rfz, Stats st) {
	const NGrid<R>& g = S.nl;
	const R ffelec = (R)par->ffelec;
	for (unsigned i = 0; i < lig->n; ++i) {
		const unsigned atomTypeLig = lig->type[i];
		if (atomTypeLig == 0) continue;
		const R posLigX = LX[i], posLigY = LY[i], posLigZ = LZ[i];
		if (g.out_of_bounds(posLigX, posLigY, posLigZ)) continue;
		int ix, iy, iz;
		g.index(posLigX, posLigY, posLigZ, ix, iy, iz);
		const gba_neighbour_desc& nDesc = g.grid[(size_t)g.dimN[0] * (iz * g.dimN[1] + iy) + ix];
		if (st.s) { st.s->n_nl++; st.s->n_nl_entries += nDesc.numEl; }
		R fAccx = 0, fAccy = 0, fAccz = 0, eAcc = 0;
		for (unsigned j = 0; j < nDesc.numEl; ++j) {
			const unsigned nIdx = g.list[nDesc.idx + j];
			R dx = posLigX - RX[nIdx];
			R dy = posLigY - RY[nIdx];
			R dz = posLigZ - RZ[nIdx];
			const R dr2 = dx * dx + dy * dy + dz * dz;
			if (dr2 > g.dPlateau2) continue;
			if (st.s) st.s->n_pairs++;
			const R dr2_inv = (R)(1.0 / (W)dr2);
			dx *= dr2_inv; dy *= dr2_inv; dz *= dr2_inv;
			const unsigned atomTypeRec = rec->type[nIdx];
			const gba_ffparam& P = par->table[(size_t)par->num_types * (atomTypeRec - 1) + (atomTypeLig - 1)];
			R fx, fy, fz, e;
			R frx = 0, fry = 0, frz = 0;
			lj_pot_force<R>(dr2, dr2_inv, dx, dy, dz, P, par->potshape, fx, fy, fz, e);
			fAccx += fx; fAccy += fy; fAccz += fz; eAcc += e;
			frx -= fx; fry -= fy; frz -= fz;
			st.add_E(e); st.add_F(fx, fy, fz);
			const R chargeLig = (R)lig->charge[i];
			const R chargeRec = (R)rec->charge[nIdx];
			const R chargeLigRec = chargeLig * chargeRec * ffelec;
			const bool calc_elec = std::fabs(chargeLigRec) > 0.001;
			R ratio = g.get_ratio(dr2);
			R rdx = ratio * dx, rdy = ratio * dy, rdz = ratio * dz;
			lj_pot_force<R>(g.dPlateau2, g.dPlateau2_inv, rdx, rdy, rdz, P, par->potshape, fx, fy, fz, e);
			fAccx -= fx; fAccy -= fy; fAccz -= fz; eAcc -= e;
			frx += fx; fry += fy; frz += fz;
			st.add_E(e); st.add_F(fx, fy, fz);
			if (calc_elec) {
				charge_pot_force<R>(dr2_inv, dx, dy, dz, chargeLigRec, par->dielec, fx, fy, fz, e);
				fAccx += fx; fAccy += fy; fAccz += fz; eAcc += e;
				frx -= fx; fry -= fy; frz -= fz;
				st.add_E(e); st.add_F(fx, fy, fz);
				charge_pot_force<R>(g.dPlateau2_inv, rdx, rdy, rdz, chargeLigRec, par->dielec, fx, fy, fz, e);
				fAccx -= fx; fAccy -= fy; fAccz -= fz; eAcc -= e;
				frx += fx; fry += fy; frz += fz;
				st.add_E(e); st.add_F(fx, fy, fz);
			}
			if (rfx) { rfx[nIdx] += frx; rfy[nIdx] += fry; rfz[nIdx] += frz; }
		}
		ofx[i] += fAccx; ofy[i] += fAccy; ofz[i] += fAccz; oE[i] += eAcc;
	}
}

/* reducePotForce, src/model/reduction.h:40-75 (sum + ForceLim clamp) */
template <typename R>
void reduce_pot_force(const R* fx, const R* fy, const R* fz, const R* E, unsigned n,
		R& oE, R& ox, R& oy, R& oz, orc_pose_stats* stats = nullptr) {
	R e = 0, x = 0, y = 0, z = 0;
	for (unsigned i = 0; i < n; ++i) { e += E[i]; x += fx[i]; y += fy[i]; z += fz[i]; }
	for (unsigned i = 0; i < 3; ++i) {
		R magn2 = x * x + y * y + z * z;
		if (magn2 > (R)1.0e18f) {
			x = (R)((W)x * 0.01); y = (R)((W)y * 0.01); z = (R)((W)z * 0.01);
			if (stats) stats->n_force_lim++;
		}
	}
	oE = e; ox = x; oy = y; oz = z;
}

/* reduceTorque + TorqueMat::rotateReduce, src/model/reduction.h:81-103,
 * src/commons/TorqueMat.h:27-37 */
template <typename R>
void reduce_torque(const orc_protein* lig, const R* fx, const R* fy, const R* fz,
		R ang_x, R ang_y, R ang_z, R out[3], Stats st) {
	R T[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
	const float* X = lig->xyz;
	const float* Y = lig->xyz + lig->n;
	const float* Z = lig->xyz + 2 * lig->n;
	for (unsigned i = 0; i < lig->n; ++i) {
		R x = X[i], y = Y[i], z = Z[i];
		T[0][0] += x * fx[i]; T[0][1] += y * fx[i]; T[0][2] += z * fx[i];
		T[1][0] += x * fy[i]; T[1][1] += y * fy[i]; T[1][2] += z * fy[i];
		T[2][0] += x * fz[i]; T[2][1] += y * fz[i]; T[2][2] += z * fz[i];
		if (st.s)
			st.s->abs_T += std::sqrt((double)x * x + (double)y * y + (double)z * z) *
					std::sqrt((double)fx[i] * fx[i] + (double)fy[i] * fy[i] + (double)fz[i] * fz[i]);
	}
	R M[3][3][3];
	euler2torquemat<R>(ang_x, ang_y, ang_z, M);
	R rx = 0, ry = 0, rz = 0;
	for (unsigned k = 0; k < 3; ++k)
		for (unsigned l = 0; l < 3; ++l) {
			rx += M[k][0][l] * T[k][l];
			ry += M[k][1][l] * T[k][l];
			rz += M[k][2][l] * T[k][l];
		}
	out[0] = rx; out[1] = ry; out[2] = rz;
}

/* ------------------------------------------------------------------------ */
/* rigid item processor, src/service/CPUEnergyService6D.tpp:63-200          */
/* ------------------------------------------------------------------------ */

template <typename R>
struct RigidWork {
	std::vector<R> tx, ty, tz, fx, fy, fz, E, rx, ry, rz;
	void alloc(unsigned n, const orc_protein* rec) {
		tx.resize(n); ty.resize(n); tz.resize(n); fx.resize(n); fy.resize(n); fz.resize(n); E.resize(n);
		const float* X = rec->xyz;
		rx.assign(X, X + rec->n);
		ry.assign(X + rec->n, X + 2 * rec->n);
		rz.assign(X + 2 * rec->n, X + 3 * rec->n);
	}
};

template <typename R>
void eval_rigid(const Sys<R>& S, const orc_protein* rec, const orc_protein* lig,
		const orc_params* par, const R pos[3], const R ang[3], R out7[7], RigidWork<R>& w,
		orc_pose_stats* stats) {
	Stats st{stats};
	if (stats) std::memset(stats, 0, sizeof(*stats));
	const unsigned n = lig->n;
	/* rotate_translate, src/model/transform.h:22-44 */
	R m[9];
	euler2rotmat<R>(ang[0], ang[1], ang[2], m);
	const float* X = lig->xyz; const float* Y = X + n; const float* Z = Y + n;
	for (unsigned i = 0; i < n; ++i) {
		R ox, oy, oz;
		matvec<R>(m, (R)X[i], (R)Y[i], (R)Z[i], ox, oy, oz);
		w.tx[i] = ox + pos[0]; w.ty[i] = oy + pos[1]; w.tz[i] = oz + pos[2];
	}
	pot_force<R>(S, lig, w.tx.data(), w.ty.data(), w.tz.data(), w.fx.data(), w.fy.data(),
			w.fz.data(), w.E.data(), st);
	if (S.has_nl) {
		nl_pot_force<R>(S, rec, lig, par, w.rx.data(), w.ry.data(), w.rz.data(), w.tx.data(),
				w.ty.data(), w.tz.data(), w.fx.data(), w.fy.data(), w.fz.data(), w.E.data(),
				nullptr, nullptr, nullptr, st);
	}
	reduce_pot_force<R>(w.fx.data(), w.fy.data(), w.fz.data(), w.E.data(), n, out7[0], out7[1],
			out7[2], out7[3], stats);
	reduce_torque<R>(lig, w.fx.data(), w.fy.data(), w.fz.data(), ang[0], ang[1], ang[2], out7 + 4, st);
}

/* ------------------------------------------------------------------------ */
/* modes item processor, src/service/CPUEnergyService6DModes.tpp:76-336     */
/* ------------------------------------------------------------------------ */

template <typename R>
struct ModesWork {
	std::vector<R> rdx, rdy, rdz, rtx, rty, rtz, ltx, lty, ltz;
	std::vector<R> rfx, rfy, rfz, rE, lfx, lfy, lfz, lE;
	void alloc(unsigned nr, unsigned nl) {
		for (auto* v : {&rdx, &rdy, &rdz, &rtx, &rty, &rtz, &rfx, &rfy, &rfz, &rE}) v->resize(nr);
		for (auto* v : {&ltx, &lty, &ltz, &lfx, &lfy, &lfz, &lE}) v->resize(nl);
	}
};

/* reduceModeForce (with / without rotation), src/model/reduction_modes.h:29-90 */
template <typename R>
void reduce_mode_force(const R* rot /* nullable */, const R* fx, const R* fy, const R* fz,
		const orc_protein* p, R* result) {
	const unsigned M = p->n_modes, n = p->n;
	const float* mx = p->modes; const float* my = mx + (size_t)n * M; const float* mz = my + (size_t)n * M;
	for (unsigned m = 0; m < M; ++m) result[m] = 0;
	for (unsigned i = 0; i < n; ++i) {
		R x = fx[i], y = fy[i], z = fz[i];
		if (rot) { R ox, oy, oz; matvec<R>(rot, x, y, z, ox, oy, oz); x = ox; y = oy; z = oz; }
		for (unsigned m = 0; m < M; ++m)
			result[m] -= x * (R)mx[i * M + m] + y * (R)my[i * M + m] + z * (R)mz[i * M + m];
	}
}

/* correctModeForce, src/model/reduction_modes.h:101-115 */
template <typename R>
void correct_mode_force(const float* k, unsigned M, R* delta) {
	const R factor = 4.0;
	for (unsigned m = 0; m < M; ++m) {
		R counterForce = (R)((W)(factor * (R)k[m]) * std::pow((W)delta[m], 4));
		delta[m] = delta[m] + counterForce;
	}
}

/* deform (+ rotate + translate), src/model/transform_modes.h:54-93 and
 * src/model/transform.h:47-80 */
template <typename R>
void deform_transform(const orc_protein* p, const R* amp, const R m[9], const R t[3], R* dx,
		R* dy, R* dz, R* tx, R* ty, R* tz) {
	const unsigned M = p->n_modes, n = p->n;
	const float* X = p->xyz; const float* Y = X + n; const float* Z = Y + n;
	const float* mx = p->modes; const float* my = mx + (size_t)n * M; const float* mz = my + (size_t)n * M;
	for (unsigned i = 0; i < n; ++i) {
		R x = X[i], y = Y[i], z = Z[i];
		for (unsigned k = 0; k < M; ++k) {
			x += amp[k] * (R)mx[i * M + k];
			y += amp[k] * (R)my[i * M + k];
			z += amp[k] * (R)mz[i * M + k];
		}
		if (dx) { dx[i] = x; dy[i] = y; dz[i] = z; }
		R ox, oy, oz;
		matvec<R>(m, x, y, z, ox, oy, oz);
		tx[i] = ox + t[0]; ty[i] = oy + t[1]; tz[i] = oz + t[2];
	}
}

/* Result_6D_Modes with double fields, for the FP64 evaluation */
struct result6d_modes_f64 {
	struct { double E, pos[3], ang[3]; } rigid;
	double modesRec[GBA_MODES_MAX], modesLig[GBA_MODES_MAX];
};

template <typename R, typename Res = gba_result6d_modes>
void eval_modes(const Sys<R>& SR, const Sys<R>& SL, const orc_protein* rec, const orc_protein* lig,
		const orc_params* par, const gba_dof6d_modes& dof, Res& res, ModesWork<R>& w,
		orc_pose_stats* stats) {
	typedef typename std::remove_reference<decltype(res.rigid.E)>::type T;
	Stats st{stats};
	if (stats) std::memset(stats, 0, sizeof(*stats));
	const R pos[3] = {dof.rigid.pos[0], dof.rigid.pos[1], dof.rigid.pos[2]};
	const R ang[3] = {dof.rigid.ang[0], dof.rigid.ang[1], dof.rigid.ang[2]};
	R ampR[GBA_MODES_MAX], ampL[GBA_MODES_MAX];
	for (int m = 0; m < GBA_MODES_MAX; ++m) { ampR[m] = dof.modesRec[m]; ampL[m] = dof.modesLig[m]; }
	/* invertDOF, src/model/transform_modes.h:27-41 */
	R R0[9], RT[9];
	euler2rotmat<R>(ang[0], ang[1], ang[2], R0);
	transpose<R>(R0, RT);
	const R iang[3] = {-ang[0], -ang[1], -ang[2]};
	R ipos[3];
	matvec<R>(RT, -pos[0], -pos[1], -pos[2], ipos[0], ipos[1], ipos[2]);
	R Rinv[9];
	euler2rotmat<R>(iang[0], iang[1], iang[2], Rinv);
	/* receptor: deformed (receptor frame) and moved into the ligand frame */
	deform_transform<R>(rec, ampR, Rinv, ipos, w.rdx.data(), w.rdy.data(), w.rdz.data(),
			w.rtx.data(), w.rty.data(), w.rtz.data());
	/* ligand: deformed and moved into the receptor frame */
	deform_transform<R>(lig, ampL, R0, pos, nullptr, nullptr, nullptr, w.ltx.data(),
			w.lty.data(), w.ltz.data());
	/* receptor beads in the ligand grid, forces rotated back by R(ang)
	 * (rotate_forces with invertedDOF.ang.inv(), src/model/transform_modes.h:146-166) */
	orc_pose_stats rec_st;
	std::memset(&rec_st, 0, sizeof(rec_st));
	pot_force<R>(SL, rec, w.rtx.data(), w.rty.data(), w.rtz.data(), w.rfx.data(), w.rfy.data(),
			w.rfz.data(), w.rE.data(), Stats{stats ? &rec_st : nullptr});
	if (stats) stats->n_rec_lookups = rec_st.n_grid + rec_st.n_grid_charged;
	for (unsigned i = 0; i < rec->n; ++i) {
		R ox, oy, oz;
		matvec<R>(R0, w.rfx[i], w.rfy[i], w.rfz[i], ox, oy, oz);
		w.rfx[i] = ox; w.rfy[i] = oy; w.rfz[i] = oz;
	}
	/* ligand beads in the receptor grid */
	pot_force<R>(SR, lig, w.ltx.data(), w.lty.data(), w.ltz.data(), w.lfx.data(), w.lfy.data(),
			w.lfz.data(), w.lE.data(), st);
	if (SR.has_nl)
		nl_pot_force<R>(SR, rec, lig, par, w.rdx.data(), w.rdy.data(), w.rdz.data(), w.ltx.data(),
				w.lty.data(), w.ltz.data(), w.lfx.data(), w.lfy.data(), w.lfz.data(), w.lE.data(),
				w.rfx.data(), w.rfy.data(), w.rfz.data(), st);
	R E, fx, fy, fz;
	reduce_pot_force<R>(w.lfx.data(), w.lfy.data(), w.lfz.data(), w.lE.data(), lig->n, E, fx, fy, fz);
	R modesLig[GBA_MODES_MAX] = {0}, modesRec[GBA_MODES_MAX] = {0};
	reduce_mode_force<R>(RT, w.lfx.data(), w.lfy.data(), w.lfz.data(), lig, modesLig);
	correct_mode_force<R>(lig->mode_force, lig->n_modes, modesLig);
	reduce_mode_force<R>(nullptr, w.rfx.data(), w.rfy.data(), w.rfz.data(), rec, modesRec);
	correct_mode_force<R>(rec->mode_force, rec->n_modes, modesRec);
	std::memset(&res, 0, sizeof(res));
	for (unsigned m = 0; m < lig->n_modes; ++m) res.modesLig[m] = (T)modesLig[m];
	for (unsigned m = 0; m < rec->n_modes; ++m) res.modesRec[m] = (T)modesRec[m];
	res.rigid.E = (T)E;
	res.rigid.pos[0] = (T)fx; res.rigid.pos[1] = (T)fy; res.rigid.pos[2] = (T)fz;
	R a[3];
	reduce_torque<R>(lig, w.lfx.data(), w.lfy.data(), w.lfz.data(), ang[0], ang[1], ang[2], a, st);
	res.rigid.ang[0] = (T)a[0]; res.rigid.ang[1] = (T)a[1]; res.rigid.ang[2] = (T)a[2];
}

/* ------------------------------------------------------------------------ */
/* threading helper                                                         */
/* ------------------------------------------------------------------------ */

template <typename F>
void parallel_for(size_t n, int nthreads, F f) {
	if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
	if ((size_t)nthreads > n) nthreads = (int)std::max<size_t>(1, n);
	if (nthreads == 1) { f(0, (size_t)0, n); return; }
	std::vector<std::thread> th;
	size_t chunk = (n + nthreads - 1) / nthreads;
	for (int t = 0; t < nthreads; ++t) {
		size_t b = t * chunk, e = std::min(n, b + chunk);
		if (b >= e) break;
		th.emplace_back([=] { f(t, b, e); });
	}
	for (auto& x : th) x.join();
}

/* ------------------------------------------------------------------------ */
/* VA13: minfor.f:1-182 and mc11a.f:1-143 (mc11e entry at :114)             */
/* Arrays are 1-based to mirror the Fortran.                                */
/* ------------------------------------------------------------------------ */

void mc11a(double* a, int n, double* z, double sig, double* w, int& ir, int mk, double eps) {
	double ti = 0, v, tim, b, r, y, gm, al;
	int np, ij, ip, mm, j;
	if (n > 1) goto L1;
	a[1] = a[1] + sig * z[1] * z[1];
	ir = 1;
	if (a[1] > 0.0) return;
	a[1] = 0.0;
	ir = 0;
	return;
L1:
	np = n + 1;
	if (sig > 0.0) goto L40;
	if (sig == 0.0 || ir == 0) return;
	ti = 1.0 / sig;
	ij = 1;
	if (mk == 0) goto L10;
	for (int i = 1; i <= n; ++i) {
		if (a[ij] != 0.0) ti = ti + w[i] * w[i] / a[ij];
		ij = ij + np - i;
	}
	goto L20;
L10:
	for (int i = 1; i <= n; ++i) w[i] = z[i];
	for (int i = 1; i <= n; ++i) {
		ip = i + 1;
		v = w[i];
		if (a[ij] > 0.0) goto L12;
		w[i] = 0.0;
		ij = ij + np - i;
		continue;
	L12:
		ti = ti + v * v / a[ij];
		if (i == n) goto L14;
		for (j = ip; j <= n; ++j) {
			ij = ij + 1;
			w[j] = w[j] - v * a[ij];
		}
	L14:
		ij = ij + 1;
	}
L20:
	if (ir <= 0) goto L21;
	if (ti > 0.0) goto L22;
	if (mk - 1 <= 0) goto L40;
	goto L23;
L21:
	ti = 0.;
	ir = -ir - 1;
	goto L23;
L22:
	ti = eps / sig;
	if (eps == 0.0) ir = ir - 1;
L23:
	mm = 1;
	tim = ti;
	for (int i = 1; i <= n; ++i) {
		j = np - i;
		ij = ij - i;
		if (a[ij] != 0.0) tim = ti - w[j] * w[j] / a[ij];
		w[j] = ti;
		ti = tim;
	}
	goto L41;
L40:
	mm = 0;
	tim = 1.0 / sig;
L41:
	ij = 1;
	for (int i = 1; i <= n; ++i) {
		ip = i + 1;
		v = z[i];
		if (a[ij] > 0.0) goto L53;
		if (ir > 0 || sig < 0.0 || v == 0.0) goto L52;
		ir = 1 - ir;
		a[ij] = v * v / tim;
		if (i == n) return;
		for (j = ip; j <= n; ++j) {
			ij = ij + 1;
			a[ij] = z[j] / v;
		}
		return;
	L52:
		ti = tim;
		ij = ij + np - i;
		continue;
	L53:
		al = v / a[ij];
		if (mm <= 0) ti = tim + v * al;
		else ti = w[i];
		r = ti / tim;
		a[ij] = a[ij] * r;
		if (r == 0.0) goto L70;
		if (i == n) goto L70;
		b = al / ti;
		if (r > 4.0) goto L62;
		for (j = ip; j <= n; ++j) {
			ij = ij + 1;
			z[j] = z[j] - v * a[ij];
			a[ij] = a[ij] + b * z[j];
		}
		goto L64;
	L62:
		gm = tim / ti;
		for (j = ip; j <= n; ++j) {
			ij = ij + 1;
			y = a[ij];
			a[ij] = b * z[j] + y * gm;
			z[j] = z[j] - v * y;
		}
	L64:
		tim = ti;
		ij = ij + 1;
	}
L70:
	if (ir < 0) ir = -ir;
}

void mc11e(const double* a, int n, double* z, double* w, int ir) {
	int ij, i1, np, ii, ip, i;
	double v;
	if (ir < n) return;
	w[1] = z[1];
	if (n > 1) goto L400;
	z[1] = z[1] / a[1];
	return;
L400:
	ij = 0;
	for (i = 2; i <= n; ++i) {
		ij = i;
		i1 = i - 1;
		v = z[i];
		for (int j = 1; j <= i1; ++j) {
			v = v - a[ij] * z[j];
			ij = ij + n - j;
		}
		w[i] = v;
		z[i] = v;
	}
	z[n] = z[n] / a[ij];
	np = n + 1;
	for (int nip = 2; nip <= n; ++nip) {
		i = np - nip;
		ii = ij - nip;
		v = z[i] / a[ii];
		ip = i + 1;
		ij = ii;
		for (int j = ip; j <= n; ++j) {
			ii = ii + 1;
			v = v - a[ii] * z[j];
		}
		z[i] = v;
	}
}

/* minfor with an energy callback; jn = n DOF (the Fortran fixes jn = 6). */
template <typename F>
void minfor(F&& energy, int ivmax, double* x /* 1-based, size jn+1 */, int jn) {
	const int NMAX = 32;
	double gesa = 0, c, acc, dff, dgb, fa, fmin, gl1, gl2, gmin, dga, xnull, fb = 0;
	double step, stepbd, steplb, stmin;
	double h[NMAX * NMAX + 1], g[NMAX + 1], ga[NMAX + 1], gb[NMAX + 1], w[NMAX + 1];
	double xaa[NMAX + 1], xbb[NMAX + 1], d[NMAX + 1];
	int i, k, ir, isfv, itr, nfun, np;
	xnull = 0.0;
	dga = xnull;
	for (i = 1; i <= jn; ++i) { ga[i] = xnull; d[i] = xnull; xaa[i] = x[i]; }
	nfun = 0;
	itr = 0;
	np = jn + 1;
	acc = 0.000000001;
	c = 1.0;
	k = (jn * np) / 2;
	for (i = 1; i <= k; ++i) h[i] = xnull;
	k = 1;
	for (i = 1; i <= jn; ++i) { h[k] = 0.01 * c; k = k + np - i; }
	dff = xnull;
	energy(xaa, gesa, g);
L110:
	fa = gesa;
	isfv = 1;
	for (i = 1; i <= jn; ++i) ga[i] = g[i];
L135:
	itr = itr + 1;
	for (i = 1; i <= jn; ++i) d[i] = -ga[i];
	mc11e(h, jn, d, w, jn);
	c = xnull;
	dga = xnull;
	for (i = 1; i <= jn; ++i) { c = std::max(c, std::fabs(d[i])); dga = dga + ga[i] * d[i]; }
	if (dga >= xnull) goto L240;
	stmin = xnull;
	stepbd = xnull;
	steplb = acc / c;
	fmin = fa;
	gmin = dga;
	step = 1.0;
	if (dff <= xnull) step = std::min(step, 1.0 / c);
	if (dff > xnull) step = std::min(step, (dff + dff) / (-dga));
L170:
	c = stmin + step;
	if (nfun >= ivmax) goto L250;
	nfun = nfun + 1;
	for (i = 1; i <= jn; ++i) xbb[i] = xaa[i] + c * d[i];
	energy(xbb, fb, gb);
	isfv = std::min(2, isfv);
	if (fb > gesa) goto L220;
	if (fb < gesa) goto L200;
	gl1 = xnull;
	gl2 = xnull;
	for (i = 1; i <= jn; ++i) { gl1 = gl1 + g[i] * g[i]; gl2 = gl2 + gb[i] * gb[i]; }
	if (gl2 >= gl1) goto L220;
L200:
	isfv = 3;
	gesa = fb;
	for (i = 1; i <= jn; ++i) { x[i] = xbb[i]; g[i] = gb[i]; }
L220:
	dgb = xnull;
	for (i = 1; i <= jn; ++i) dgb = dgb + gb[i] * d[i];
	if (fb - fa <= 0.1 * c * dga) goto L280;
	if (step > steplb) goto L270;
L240:
	if (isfv >= 2) goto L110;
L250:
	return;
L270:
	stepbd = step;
	c = gmin + dgb - 3.0 * (fb - fmin) / step;
	c = gmin / (c + gmin - std::sqrt(c * c - gmin * dgb));
	step = step * std::max(0.1, c);
	goto L170;
L280:
	stepbd = stepbd - step;
	stmin = c;
	fmin = fb;
	gmin = dgb;
	step = 9.0 * stmin;
	if (stepbd > xnull) step = 0.5 * stepbd;
	c = dga + 3.0 * dgb - 4.0 * (fb - fa) / stmin;
	if (c > xnull) step = std::min(step, stmin * std::max(1.0, -dgb / c));
	if (dgb < 0.7 * dga) goto L170;
	isfv = 4 - isfv;
	if (stmin + step <= steplb) goto L240;
	ir = -jn;
	for (i = 1; i <= jn; ++i) {
		xaa[i] = xbb[i];
		xbb[i] = ga[i];
		d[i] = gb[i] - ga[i];
		ga[i] = gb[i];
	}
	mc11a(h, jn, xbb, 1.0 / dga, w, ir, 1, xnull);
	ir = -ir;
	mc11a(h, jn, d, 1.0 / (stmin * (dgb - dga)), d, ir, 0, xnull);
	if (ir < jn) goto L250;
	dff = fa - fb;
	fa = fb;
	goto L135;
}

/* ------------------------------------------------------------------------ */
/* grid builder                                                             */
/* ------------------------------------------------------------------------ */

/* Pair force and energy of the grid builder for one receptor bead and one
 * ligand type: LJPotForce (src/model/forcefield.h:30-83) evaluated with the
 * operations of the library's device builder -- IEEE-rounded FP32, the one
 * fused multiply-add where the device has it -- so that both builders give
 * the same bits. */
inline void grid_lj(float e2, float rr2, float ux, float uy, float uz, const gba_ffparam& p, bool shape86,
		float* o) {
	const float rr23 = (rr2 * rr2) * rr2;
	const float rrd = shape86 ? rr2 : rr23;
	const float sd = shape86 ? 2.0f : 6.0f;
	const float rep = p.rc * rrd;
	const float vlj = (rep - p.ac) * rr23;
	float fb = std::fmaf(6.0f, vlj, sd * (rep * rr23));
	const float ivor = (float)p.ipon;
	float e;
	if (e2 < p.rmin2) {
		e = std::fmaf(ivor - 1.0f, p.emin, vlj);
	} else {
		e = ivor * vlj;
		fb = ivor * fb;
	}
	o[0] = fb * ux; o[1] = fb * uy; o[2] = fb * uz; o[3] = e;
}

/* ChargePotForce (src/model/forcefield.h:87-146) per unit ligand charge, in
 * the device builder's FP32 operations. */
inline void grid_coulomb(float rr2, float ux, float uy, float uz, float qq, bool cdiel, float* o) {
	float dd, et2;
	if (cdiel) {
		const float sr = std::sqrt(rr2);
		dd = sr - 0.02f;
		et2 = qq * sr;
	} else {
		dd = rr2 - 4.0e-4f;
		et2 = 2.0f * (qq * rr2);
	}
	if (dd <= 0.0f) {
		o[0] = o[1] = o[2] = o[3] = 0.0f;
		return;
	}
	o[3] = qq * dd;
	o[0] = et2 * ux; o[1] = et2 * uy; o[2] = et2 * uz;
}

/* All channels of one voxel centre (px, py, pz): each receptor bead's
 * contribution is evaluated at max(r, plateau) along the bead->voxel
 * direction (so that grid + NL(r) - NL(plateau) is the exact pair term
 * inside the plateau, src/model/neighborlist.h:104-157).  The sum runs over
 * the receptor beads in blocks of 256 consecutive indices: FP32 partial sums in
 * bead order inside a block, those partials added in double block after
 * block -- the device builder's order (csrc/gridbuild.cu). */
void voxel_terms(float px, float py, float pz, const orc_protein* rec, const orc_params* par,
		const orc_grid_opts* opt, double* acc /* numGrids*4 */, float* tacc /* numGrids*4 */) {
	const float* X = rec->xyz; const float* Y = X + rec->n; const float* Z = Y + rec->n;
	const float plateau = opt->plateau;
	const float plat2 = plateau * plateau;
	const unsigned C = opt->n_alphabet + 1;
	const bool shape86 = par->potshape == GBA_POTSHAPE_8_6;
	const bool cdiel = par->dielec == GBA_DIELEC_CONSTANT;
	constexpr unsigned kBlock = 256;
	for (unsigned t0 = 0; t0 < rec->n; t0 += kBlock) {
		std::fill(tacc, tacc + 4 * C, 0.0f);
		const unsigned t1 = std::min(rec->n, t0 + kBlock);
		for (unsigned j = t0; j < t1; ++j) {
			const unsigned tr = rec->type[j];
			if (tr == 0) continue;
			float ex = px - X[j], ey = py - Y[j], ez = pz - Z[j];
			float e2 = (ex * ex + ey * ey) + ez * ez;
			bool dirless = false;
			if (e2 < plat2) {
				if (e2 > 0.0f) {
					const float sc = plateau / std::sqrt(e2);
					ex = ex * sc; ey = ey * sc; ez = ez * sc;
				} else {
					dirless = true;
				}
				e2 = plat2;
			}
			const float rr2 = 1.0f / e2;
			const float ux = dirless ? 0.0f : ex * rr2, uy = dirless ? 0.0f : ey * rr2,
					uz = dirless ? 0.0f : ez * rr2;
			float o[4];
			for (unsigned c = 0; c < C; ++c) {
				if (c == 0) {
					const float qf = rec->charge[j] * par->ffelec;
					if (!(std::fabs(qf) > 0.001f)) continue;
					grid_coulomb(rr2, ux, uy, uz, qf, cdiel, o);
				} else {
					const unsigned tl = opt->alphabet[c - 1];
					if (tl == 0 || tl > par->num_types || tr > par->num_types) continue;
					grid_lj(e2, rr2, ux, uy, uz, par->table[(size_t)par->num_types * (tr - 1) + (tl - 1)],
							shape86, o);
				}
				for (int k = 0; k < 4; ++k) tacc[4 * c + k] = tacc[4 * c + k] + o[k];
			}
		}
		for (unsigned k = 0; k < 4 * C; ++k) acc[k] = acc[k] + (double)tacc[k];
	}
}

void fill_grid(const gba_intrpl_desc* d, float* data, const orc_protein* rec, const orc_params* par,
		const orc_grid_opts* opt, int nthreads) {
	const size_t N = (size_t)d->dimN[0] * d->dimN[1] * d->dimN[2];
	const unsigned C = d->numGrids;
	parallel_for(d->dimN[2], nthreads, [&](int, size_t zb, size_t ze) {
		std::vector<double> acc(4 * C);
		std::vector<float> tacc(4 * C);
		for (size_t z = zb; z < ze; ++z)
			for (unsigned y = 0; y < d->dimN[1]; ++y)
				for (unsigned x = 0; x < d->dimN[0]; ++x) {
					std::fill(acc.begin(), acc.end(), 0.0);
					const float px = (float)((double)d->posMin[0] + x * (double)d->gridSpacing);
					const float py = (float)((double)d->posMin[1] + y * (double)d->gridSpacing);
					const float pz = (float)((double)d->posMin[2] + z * (double)d->gridSpacing);
					voxel_terms(px, py, pz, rec, par, opt, acc.data(), tacc.data());
					size_t v = (size_t)d->dimN[0] * (z * d->dimN[1] + y) + x;
					for (unsigned c = 0; c < C; ++c)
						for (int k = 0; k < 4; ++k) data[4 * (c * N + v) + k] = (float)acc[4 * c + k];
				}
	});
}

}  // namespace

/* ======================================================================== */
/* C ABI                                                                     */
/* ======================================================================== */

extern "C" void orc_set_exact_sincos(int exact) { g_exact_sincos.store(exact ? 1 : 0); }

extern "C" {

int orc_energy_6d(const orc_protein* rec, const orc_protein* lig, const orc_grid* grid,
		const orc_params* par, const gba_dof6d* dofs, size_t n, gba_result6d* out,
		orc_pose_stats* stats, int nthreads) {
	if (!rec || !lig || !grid || !par || (n && (!dofs || !out))) return GBA_ERR_INVALID_ARGUMENT;
	Sys<float> S;
	S.init(grid);
	parallel_for(n, nthreads, [&](int, size_t b, size_t e) {
		RigidWork<float> w;
		w.alloc(lig->n, rec);
		for (size_t p = b; p < e; ++p) {
			float o[7];
			eval_rigid<float>(S, rec, lig, par, dofs[p].pos, dofs[p].ang, o, w, stats ? stats + p : nullptr);
			out[p].E = o[0];
			out[p].pos[0] = o[1]; out[p].pos[1] = o[2]; out[p].pos[2] = o[3];
			out[p].ang[0] = o[4]; out[p].ang[1] = o[5]; out[p].ang[2] = o[6];
		}
	});
	return GBA_OK;
}

int orc_energy_6d_f64(const orc_protein* rec, const orc_protein* lig, const orc_grid* grid,
		const orc_params* par, const gba_dof6d* dofs, size_t n, double* out7, int nthreads) {
	if (!rec || !lig || !grid || !par || (n && (!dofs || !out7))) return GBA_ERR_INVALID_ARGUMENT;
	Sys<double> S;
	S.init(grid);
	parallel_for(n, nthreads, [&](int, size_t b, size_t e) {
		RigidWork<double> w;
		w.alloc(lig->n, rec);
		for (size_t p = b; p < e; ++p) {
			double pos[3] = {dofs[p].pos[0], dofs[p].pos[1], dofs[p].pos[2]};
			double ang[3] = {dofs[p].ang[0], dofs[p].ang[1], dofs[p].ang[2]};
			eval_rigid<double>(S, rec, lig, par, pos, ang, out7 + 7 * p, w, nullptr);
		}
	});
	return GBA_OK;
}

int orc_energy_6d_modes(const orc_protein* rec, const orc_protein* lig,
		const orc_grid* grid_rec, const orc_grid* grid_lig, const orc_params* par,
		const gba_dof6d_modes* dofs, size_t n, gba_result6d_modes* out,
		orc_pose_stats* stats, int nthreads) {
	if (!rec || !lig || !grid_rec || !grid_lig || !par || (n && (!dofs || !out)))
		return GBA_ERR_INVALID_ARGUMENT;
	if (rec->n_modes > GBA_MODES_MAX || lig->n_modes > GBA_MODES_MAX) return GBA_ERR_INVALID_ARGUMENT;
	Sys<float> SR, SL;
	SR.init(grid_rec);
	SL.init(grid_lig);
	parallel_for(n, nthreads, [&](int, size_t b, size_t e) {
		ModesWork<float> w;
		w.alloc(rec->n, lig->n);
		for (size_t p = b; p < e; ++p)
			eval_modes<float>(SR, SL, rec, lig, par, dofs[p], out[p], w, stats ? stats + p : nullptr);
	});
	return GBA_OK;
}

int orc_energy_6d_modes_f64(const orc_protein* rec, const orc_protein* lig,
		const orc_grid* grid_rec, const orc_grid* grid_lig, const orc_params* par,
		const gba_dof6d_modes* dofs, size_t n, double* out27, int nthreads) {
	if (!rec || !lig || !grid_rec || !grid_lig || !par || (n && (!dofs || !out27)))
		return GBA_ERR_INVALID_ARGUMENT;
	if (rec->n_modes > GBA_MODES_MAX || lig->n_modes > GBA_MODES_MAX) return GBA_ERR_INVALID_ARGUMENT;
	Sys<double> SR, SL;
	SR.init(grid_rec);
	SL.init(grid_lig);
	parallel_for(n, nthreads, [&](int, size_t b, size_t e) {
		ModesWork<double> w;
		w.alloc(rec->n, lig->n);
		for (size_t p = b; p < e; ++p) {
			result6d_modes_f64 r;
			eval_modes<double>(SR, SL, rec, lig, par, dofs[p], r, w, nullptr);
			double* o = out27 + 27 * p;
			o[0] = r.rigid.E;
			for (int k = 0; k < 3; ++k) { o[1 + k] = r.rigid.pos[k]; o[4 + k] = r.rigid.ang[k]; }
			for (int m = 0; m < GBA_MODES_MAX; ++m) { o[7 + m] = r.modesRec[m]; o[17 + m] = r.modesLig[m]; }
		}
	});
	return GBA_OK;
}

int orc_minimize_6d(const orc_protein* rec, const orc_protein* lig, const orc_grid* grid,
		const orc_params* par, const gba_dof6d* start, size_t n, int max_fun_eval,
		gba_dof6d* out_state, gba_result6d* out_result, int32_t* out_nevals, int nthreads) {
	if (!rec || !lig || !grid || !par || (n && (!start || !out_state || !out_result)))
		return GBA_ERR_INVALID_ARGUMENT;
	Sys<float> S;
	S.init(grid);
	parallel_for(n, nthreads, [&](int, size_t b, size_t e) {
		RigidWork<float> w;
		w.alloc(lig->n, rec);
		for (size_t p = b; p < e; ++p) {
			/* TypesConverter<DOF_6D, Vector>, src/apps/em/meta.h:66-97 */
			double x[7] = {0, start[p].ang[0], start[p].ang[1], start[p].ang[2], start[p].pos[0],
					start[p].pos[1], start[p].pos[2]};
			gba_dof6d last_state = start[p];
			gba_result6d last_res{};
			int nev = 0;
			auto energy = [&](const double* s, double& f, double* g) {
				gba_dof6d dof;
				dof.ang[0] = (float)s[1]; dof.ang[1] = (float)s[2]; dof.ang[2] = (float)s[3];
				dof.pos[0] = (float)s[4]; dof.pos[1] = (float)s[5]; dof.pos[2] = (float)s[6];
				float o[7];
				eval_rigid<float>(S, rec, lig, par, dof.pos, dof.ang, o, w, nullptr);
				last_state = dof;
				last_res.E = o[0];
				last_res.pos[0] = o[1]; last_res.pos[1] = o[2]; last_res.pos[2] = o[3];
				last_res.ang[0] = o[4]; last_res.ang[1] = o[5]; last_res.ang[2] = o[6];
				/* objective = E, gradient = -(ang, pos), src/apps/em/meta.h:114-121 */
				f = o[0];
				g[1] = -(double)o[4]; g[2] = -(double)o[5]; g[3] = -(double)o[6];
				g[4] = -(double)o[1]; g[5] = -(double)o[2]; g[6] = -(double)o[3];
				++nev;
			};
			minfor(energy, max_fun_eval, x, 6);
			out_state[p] = last_state;
			out_result[p] = last_res;
			if (out_nevals) out_nevals[p] = nev;
		}
	});
	return GBA_OK;
}

int orc_minimize_6d_modes(const orc_protein* rec, const orc_protein* lig,
		const orc_grid* grid_rec, const orc_grid* grid_lig, const orc_params* par,
		const gba_dof6d_modes* start, size_t n, int max_fun_eval,
		gba_dof6d_modes* out_state, gba_result6d_modes* out_result, int32_t* out_nevals,
		int nthreads) {
	if (!rec || !lig || !grid_rec || !grid_lig || !par || (n && (!start || !out_state || !out_result)))
		return GBA_ERR_INVALID_ARGUMENT;
	const int Mr = rec->n_modes, Ml = lig->n_modes;
	if (Mr > GBA_MODES_MAX || Ml > GBA_MODES_MAX) return GBA_ERR_INVALID_ARGUMENT;
	const int jn = 6 + Mr + Ml;
	Sys<float> SR, SL;
	SR.init(grid_rec);
	SL.init(grid_lig);
	parallel_for(n, nthreads, [&](int, size_t b, size_t e) {
		ModesWork<float> w;
		w.alloc(rec->n, lig->n);
		for (size_t p = b; p < e; ++p) {
			double x[33] = {0};
			const gba_dof6d_modes& s0 = start[p];
			for (int k = 0; k < 3; ++k) { x[1 + k] = s0.rigid.ang[k]; x[4 + k] = s0.rigid.pos[k]; }
			for (int m = 0; m < Mr; ++m) x[7 + m] = s0.modesRec[m];
			for (int m = 0; m < Ml; ++m) x[7 + Mr + m] = s0.modesLig[m];
			gba_dof6d_modes last_state = s0;
			gba_result6d_modes last_res{};
			int nev = 0;
			auto energy = [&](const double* s, double& f, double* g) {
				gba_dof6d_modes dof;
				std::memset(&dof, 0, sizeof(dof));
				for (int k = 0; k < 3; ++k) { dof.rigid.ang[k] = (float)s[1 + k]; dof.rigid.pos[k] = (float)s[4 + k]; }
				for (int m = 0; m < Mr; ++m) dof.modesRec[m] = (float)s[7 + m];
				for (int m = 0; m < Ml; ++m) dof.modesLig[m] = (float)s[7 + Mr + m];
				gba_result6d_modes r;
				eval_modes<float>(SR, SL, rec, lig, par, dof, r, w, nullptr);
				last_state = dof;
				last_res = r;
				f = r.rigid.E;
				for (int k = 0; k < 3; ++k) { g[1 + k] = -(double)r.rigid.ang[k]; g[4 + k] = -(double)r.rigid.pos[k]; }
				/* reduceModeForce stores -sum f . v = dE/d(amplitude)
				 * (src/model/reduction_modes.h:29-90): a gradient already,
				 * unlike the force-signed ang/pos entries */
				for (int m = 0; m < Mr; ++m) g[7 + m] = (double)r.modesRec[m];
				for (int m = 0; m < Ml; ++m) g[7 + Mr + m] = (double)r.modesLig[m];
				++nev;
			};
			minfor(energy, max_fun_eval, x, jn);
			out_state[p] = last_state;
			out_result[p] = last_res;
			if (out_nevals) out_nevals[p] = nev;
		}
	});
	return GBA_OK;
}

int orc_grid_layout(const orc_protein* rec, const orc_grid_opts* opt,
		gba_intrpl_desc* inner, gba_intrpl_desc* outer, gba_nl_desc* nl) {
	if (!rec || !opt || !inner || !outer || !nl || rec->n == 0 || opt->spacing <= 0)
		return GBA_ERR_INVALID_ARGUMENT;
	const float* P[3] = {rec->xyz, rec->xyz + rec->n, rec->xyz + 2 * rec->n};
	const double s = opt->spacing;
	inner->numGrids = outer->numGrids = opt->n_alphabet + 1;
	for (int a = 0; a < 3; ++a) {
		double lo = P[a][0], hi = P[a][0];
		for (unsigned i = 1; i < rec->n; ++i) { lo = std::min(lo, (double)P[a][i]); hi = std::max(hi, (double)P[a][i]); }
		lo -= opt->margin;
		hi += opt->margin;
		unsigned N = (unsigned)std::ceil((hi - lo) / s) + 1;
		inner->dimN[a] = N;
		inner->posMin[a] = (float)lo;
		/* outer origin from the stored float inner origin, as
		 * readGridFromGridFile derives it (src/fileIO/readFile.cpp:322-324) */
		outer->posMin[a] = (float)((double)inner->posMin[a] - opt->outer_ext * s);
		outer->dimN[a] = (unsigned)std::ceil(((N - 1) * s + 2.0 * opt->outer_ext * s) / (2 * s)) + 1;
		nl->dimN[a] = N;
		nl->posMin[a] = inner->posMin[a];
	}
	inner->gridSpacing = opt->spacing;
	outer->gridSpacing = 2 * opt->spacing;
	nl->gridSpacing = opt->spacing;
	nl->dPlateau = opt->plateau;
	nl->numEl = 0;
	return GBA_OK;
}

int orc_grid_nl(const orc_protein* rec, const orc_grid_opts* opt, gba_nl_desc* nl,
		gba_neighbour_desc* nl_grid, uint32_t* nl_list, size_t nl_cap, int nthreads) {
	if (!rec || !opt || !nl || !nl_grid) return GBA_ERR_INVALID_ARGUMENT;
	/* receptor beads (type != 0) within nl_cutoff of the voxel centre */
	const float* X = rec->xyz; const float* Y = X + rec->n; const float* Z = Y + rec->n;
	const double cut2 = (double)opt->nl_cutoff * opt->nl_cutoff;
	std::vector<std::vector<uint32_t>> per_z(nl->dimN[2]);
	parallel_for(nl->dimN[2], nthreads, [&](int, size_t zb, size_t ze) {
		for (size_t z = zb; z < ze; ++z) {
			auto& out = per_z[z];
			for (unsigned y = 0; y < nl->dimN[1]; ++y)
				for (unsigned x = 0; x < nl->dimN[0]; ++x) {
					double px = (double)nl->posMin[0] + x * (double)nl->gridSpacing;
					double py = (double)nl->posMin[1] + y * (double)nl->gridSpacing;
					double pz = (double)nl->posMin[2] + z * (double)nl->gridSpacing;
					size_t v = (size_t)nl->dimN[0] * (z * nl->dimN[1] + y) + x;
					uint32_t cnt = 0;
					for (unsigned j = 0; j < rec->n; ++j) {
						if (rec->type[j] == 0) continue;
						double dx = px - X[j], dy = py - Y[j], dz = pz - Z[j];
						if (dx * dx + dy * dy + dz * dz <= cut2) { out.push_back(j); ++cnt; }
					}
					nl_grid[v].numEl = cnt;
				}
		}
	});
	size_t total = 0;
	for (auto& v : per_z) total += v.size();
	nl->numEl = (uint32_t)total;
	if (total > nl_cap || (total && !nl_list)) return GBA_ERR_INVALID_ARGUMENT;
	size_t off = 0, vox = 0;
	for (unsigned z = 0; z < nl->dimN[2]; ++z) {
		std::copy(per_z[z].begin(), per_z[z].end(), nl_list + off);
		size_t slice_end = vox + (size_t)nl->dimN[0] * nl->dimN[1];
		for (; vox < slice_end; ++vox) {
			nl_grid[vox].idx = (uint32_t)off;
			off += nl_grid[vox].numEl;
		}
	}
	return GBA_OK;
}

int orc_grid_voxels(const orc_protein* rec, const orc_params* par, const orc_grid_opts* opt,
		const gba_intrpl_desc* d, const uint64_t* voxels, size_t count, float* out, int nthreads) {
	if (!rec || !par || !opt || !d || (count && (!voxels || !out))) return GBA_ERR_INVALID_ARGUMENT;
	if (d->numGrids != opt->n_alphabet + 1) return GBA_ERR_INVALID_ARGUMENT;
	const uint64_t N = (uint64_t)d->dimN[0] * d->dimN[1] * d->dimN[2];
	for (size_t i = 0; i < count; ++i)
		if (voxels[i] >= N) return GBA_ERR_INVALID_ARGUMENT;
	const unsigned C = d->numGrids;
	parallel_for(count, nthreads, [&](int, size_t b, size_t e) {
		std::vector<double> acc(4 * C);
		std::vector<float> tacc(4 * C);
		for (size_t i = b; i < e; ++i) {
			const uint64_t v = voxels[i];
			const unsigned x = (unsigned)(v % d->dimN[0]), y = (unsigned)((v / d->dimN[0]) % d->dimN[1]),
					z = (unsigned)(v / ((uint64_t)d->dimN[0] * d->dimN[1]));
			std::fill(acc.begin(), acc.end(), 0.0);
			const float px = (float)((double)d->posMin[0] + x * (double)d->gridSpacing);
			const float py = (float)((double)d->posMin[1] + y * (double)d->gridSpacing);
			const float pz = (float)((double)d->posMin[2] + z * (double)d->gridSpacing);
			voxel_terms(px, py, pz, rec, par, opt, acc.data(), tacc.data());
			for (unsigned k = 0; k < 4 * C; ++k) out[4 * C * i + k] = (float)acc[k];
		}
	});
	return GBA_OK;
}

int orc_grid_build(const orc_protein* rec, const orc_params* par, const orc_grid_opts* opt,
		const gba_intrpl_desc* inner, float* inner_data,
		const gba_intrpl_desc* outer, float* outer_data,
		gba_nl_desc* nl, gba_neighbour_desc* nl_grid, uint32_t* nl_list, size_t nl_cap,
		int nthreads) {
	if (!rec || !par || !opt || !inner || !outer || !nl || !inner_data || !outer_data || !nl_grid)
		return GBA_ERR_INVALID_ARGUMENT;
	if (inner->numGrids != opt->n_alphabet + 1 || outer->numGrids != opt->n_alphabet + 1)
		return GBA_ERR_INVALID_ARGUMENT;
	fill_grid(inner, inner_data, rec, par, opt, nthreads);
	fill_grid(outer, outer_data, rec, par, opt, nthreads);
	return orc_grid_nl(rec, opt, nl, nl_grid, nl_list, nl_cap, nthreads);
}

/* Pairwise path in FP64 (the reference for the adjoint checks).  Poses are
 * DOF_6D records (pos xyz, ang xyz) in double.  A pair (i, j) counts when
 * r_ij < cutoff at the pose itself, or -- with ref_dofs6 -- at the reference
 * pose, so central differences see one smooth function.  LJ follows
 * LJPotForce (src/model/forcefield.h:30-83) with the ipon/rmin2/emin branch,
 * Coulomb follows ChargePotForce (:87-146) without the |q q| switch.
 * out_E[n]; out_grad[n*6] (may be NULL) = dE/dDOF from the analytic forces and
 * the TorqueMat reduction of src/model/reduction.h:81-103. */
int orc_pairwise_energy_f64(const orc_protein* rec, const orc_protein* lig,
		const double* q_rec, const double* q_lig, uint32_t T,
		const double* r0, const double* eps, const int32_t* ipon, int dielec, double ffelec,
		double cutoff, const double* dofs6, const double* ref_dofs6, size_t n, double* out_E,
		double* out_grad) {
	if (!rec || !lig || !q_rec || !q_lig || !r0 || !eps || !ipon || (n && (!dofs6 || !out_E)))
		return GBA_ERR_INVALID_ARGUMENT;
	const float* RX = rec->xyz; const float* RY = RX + rec->n; const float* RZ = RY + rec->n;
	const float* LX = lig->xyz; const float* LY = LX + lig->n; const float* LZ = LY + lig->n;
	const double cut2 = cutoff * cutoff;
	/* per type pair: rc, ac, emin, rmin2 (readFile.cpp:484-497 in double) */
	std::vector<double> tab(4 * (size_t)T * T);
	for (size_t k = 0; k < (size_t)T * T; ++k) {
		const double rc = eps[k] * std::pow(r0[k], 8), ac = eps[k] * std::pow(r0[k], 6);
		const bool ok = ac > 0 && rc > 0;
		tab[4 * k] = rc;
		tab[4 * k + 1] = ac;
		tab[4 * k + 2] = ok ? -27.0 * std::pow(ac, 4) / (256.0 * std::pow(rc, 3)) : 0.0;
		tab[4 * k + 3] = ok ? 4.0 * rc / (3.0 * ac) : 0.0;
	}
	parallel_for(n, 0, [&](int, size_t pb, size_t pe) {
	for (size_t p = pb; p < pe; ++p) {
		const double* s = dofs6 + 6 * p;
		const double* sr = ref_dofs6 ? ref_dofs6 + 6 * p : s;
		double m[9], mr[9];
		euler2rotmat<double>(s[3], s[4], s[5], m);
		euler2rotmat<double>(sr[3], sr[4], sr[5], mr);
		double E = 0, F[3] = {0, 0, 0}, Tq[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
		for (unsigned i = 0; i < lig->n; ++i) {
			const unsigned tl = lig->type[i];
			if (tl == 0) continue;
			double x, y, z, xr, yr, zr;
			matvec<double>(m, LX[i], LY[i], LZ[i], x, y, z);
			x += s[0]; y += s[1]; z += s[2];
			matvec<double>(mr, LX[i], LY[i], LZ[i], xr, yr, zr);
			xr += sr[0]; yr += sr[1]; zr += sr[2];
			double fi[3] = {0, 0, 0};
			for (unsigned j = 0; j < rec->n; ++j) {
				const unsigned tr = rec->type[j];
				if (tr == 0) continue;
				const double ex = xr - RX[j], ey = yr - RY[j], ez = zr - RZ[j];
				if (ex * ex + ey * ey + ez * ez >= cut2) continue;
				const double dx = x - RX[j], dy = y - RY[j], dz = z - RZ[j];
				const double r2 = dx * dx + dy * dy + dz * dz;
				const size_t k = (size_t)T * (tr - 1) + (tl - 1);
				const double rc = tab[4 * k], ac = tab[4 * k + 1], emin = tab[4 * k + 2], rmin2 = tab[4 * k + 3];
				const double ir2 = 1.0 / r2, ir6 = ir2 * ir2 * ir2;
				const double vlj = (rc * ir2 - ac) * ir6;
				double fb = 6.0 * vlj + 2.0 * rc * ir2 * ir6;
				if (r2 < rmin2) {
					E += vlj + (ipon[k] - 1) * emin;
				} else {
					E += ipon[k] * vlj;
					fb *= ipon[k];
				}
				const double qq = q_lig[i] * q_rec[j] * ffelec;
				double dd, fcf;
				if (dielec == GBA_DIELEC_CONSTANT) {
					dd = std::sqrt(ir2) - 1.0 / 50.0;
					fcf = std::sqrt(ir2);
				} else {
					dd = ir2 - 1.0 / 2500.0;
					fcf = 2.0 * ir2;
				}
				if (dd > 0) E += qq * dd;
				else fcf = 0.0;
				const double ff = (fb + qq * fcf) * ir2;
				fi[0] += ff * dx; fi[1] += ff * dy; fi[2] += ff * dz;
			}
			const double u[3] = {LX[i], LY[i], LZ[i]};
			for (int a = 0; a < 3; ++a) {
				F[a] += fi[a];
				for (int b = 0; b < 3; ++b) Tq[a][b] += u[b] * fi[a];
			}
		}
		out_E[p] = E;
		if (out_grad) {
			double M[3][3][3];
			euler2torquemat<double>(s[3], s[4], s[5], M);
			double ang[3] = {0, 0, 0};
			for (int k = 0; k < 3; ++k)
				for (int l = 0; l < 3; ++l)
					for (int c = 0; c < 3; ++c) ang[c] += M[k][c][l] * Tq[k][l];
			for (int a = 0; a < 3; ++a) {
				out_grad[6 * p + a] = -F[a];
				out_grad[6 * p + 3 + a] = -ang[a];
			}
		}
	}
	});
	return GBA_OK;
}

}  // extern "C"

/* ------------------------------------------------------------------------ */
/* minfor on an analytic function (checks the device VA13 state machine)    */
/* ------------------------------------------------------------------------ */

extern "C" {

/* Runs minfor on the extended Rosenbrock function from x0 (n <= 32) and
 * records every evaluated point followed by its f: trace[k*(n+1) + ...].
 * Returns the number of evaluations recorded (at most cap). */
int orc_minfor_trace(int n, const double* x0, int ivmax, double* trace, int cap) {
	return orc_minfor_trace_nan(n, x0, ivmax, trace, cap, -1);
}

/* The same with evaluation nan_eval (0-based; -1: none) handing minfor a NaN
 * gradient component, as an energy that overflowed does. */
int orc_minfor_trace_nan(int n, const double* x0, int ivmax, double* trace, int cap, int nan_eval) {
	if (n < 1 || n > 32 || !x0 || !trace) return -1;
	double x[33];
	for (int i = 0; i < n; ++i) x[i + 1] = x0[i];
	int k = 0;
	auto energy = [&](const double* s, double& f, double* g) {
		f = 0.0;
		for (int i = 1; i <= n; ++i) g[i] = 0.0;
		for (int i = 1; i < n; ++i) {
			const double a = s[i + 1] - s[i] * s[i], b = 1.0 - s[i];
			f = f + 100.0 * a * a + b * b;
			g[i] = g[i] - 400.0 * s[i] * a - 2.0 * b;
			g[i + 1] = g[i + 1] + 200.0 * a;
		}
		if (k == nan_eval) g[1] = std::nan("");
		if (k < cap) {
			for (int i = 0; i < n; ++i) trace[(size_t)k * (n + 1) + i] = s[i + 1];
			trace[(size_t)k * (n + 1) + n] = f;
		}
		++k;
	};
	minfor(energy, ivmax, x, n);
	return k < cap ? k : cap;
}

}  // extern "C"
