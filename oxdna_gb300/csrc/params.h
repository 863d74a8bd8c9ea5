// Host-side derivation of the oxDNA2 parameter tables from the user settings.
//
// Restates DNAInteraction::DNAInteraction + init and DNA2Interaction::DNA2Interaction +
// get_settings + init (src/Interactions/DNAInteraction.cpp:12-213,290-380,
// src/Interactions/DNA2Interaction.cpp:5-21,62-155) with the reference's mixed float/double
// arithmetic: model constants are floats, so float-only sub-expressions are evaluated in float
// (the Morse-shift exponent, the Debye-Hueckel T / 0.1f, the salt read as a float) while the
// math functions are double.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstring>

#include "../../include/oxgb.h"
#include "dna2_pair.cuh"

namespace oxgb {

inline void default_settings(oxgb_dna2_settings *s, double T, double salt) {
	std::memset(s, 0, sizeof(*s));
	s->T = T;
	s->salt = salt;
	s->average = 1;
	s->hb_multiplier = 1.0;
	s->dh_half_charged_ends = 1;
	s->dh_lambda = OXM_DH_LAMBDA_DEFAULT;
	s->dh_strength = OXM_DH_STRENGTH_DEFAULT;
	s->mbf_finf = 0.04;
}

// returns 0, or -1 for invalid settings
inline int build_table(const oxgb_dna2_settings &s, double box, DNA2Table<double> &P, double &rcut) {
	static const float f1a[2] = OXM_F1_TABLE_A, f1rc[2] = OXM_F1_TABLE_RC, f1r0[2] = OXM_F1_TABLE_R0,
			f1bl[2] = OXM_F1_TABLE_BLOW, f1bh[2] = OXM_F1_TABLE_BHIGH, f1rl[2] = OXM_F1_TABLE_RLOW,
			f1rh[2] = OXM_F1_TABLE_RHIGH, f1rcl[2] = OXM_F1_TABLE_RCLOW, f1rch[2] = OXM_F1_TABLE_RCHIGH;
	static const float f2k[2] = OXM_F2_TABLE_K, f2rc[2] = OXM_F2_TABLE_RC, f2r0[2] = OXM_F2_TABLE_R0,
			f2bl[2] = OXM_F2_TABLE_BLOW, f2rl[2] = OXM_F2_TABLE_RLOW, f2rcl[2] = OXM_F2_TABLE_RCLOW,
			f2bh[2] = OXM_F2_TABLE_BHIGH, f2rh[2] = OXM_F2_TABLE_RHIGH, f2rch[2] = OXM_F2_TABLE_RCHIGH;
	static const float f4a[13] = OXM_F4_TABLE_A, f4b[13] = OXM_F4_TABLE_B, f4t0[13] = OXM_F4_TABLE_T0,
			f4ts[13] = OXM_F4_TABLE_TS, f4tc[13] = OXM_F4_TABLE_TC;
	static const float f5a[4] = OXM_F5_TABLE_A, f5b[4] = OXM_F5_TABLE_B, f5xc[4] = OXM_F5_TABLE_XC,
			f5xs[4] = OXM_F5_TABLE_XS;
	if(!(s.T > 0) || !(s.salt > 0) || !(box > 0)) return -1;
	std::memset(&P, 0, sizeof(P));
	for(int t = 0; t < 2; t++) {
		P.f1_a[t] = f1a[t];
		P.f1_r0[t] = f1r0[t];
		P.f1_blow[t] = f1bl[t];
		P.f1_bhigh[t] = f1bh[t];
		P.f1_rlow[t] = f1rl[t];
		P.f1_rhigh[t] = f1rh[t];
		P.f1_rclow[t] = f1rcl[t];
		P.f1_rchigh[t] = f1rch[t];
		P.f2_k[t] = f2k[t];
		P.f2_r0[t] = f2r0[t];
		P.f2_rc[t] = f2rc[t];
		P.f2_blow[t] = f2bl[t];
		P.f2_bhigh[t] = f2bh[t];
		P.f2_rlow[t] = f2rl[t];
		P.f2_rhigh[t] = f2rh[t];
		P.f2_rclow[t] = f2rcl[t];
		P.f2_rchigh[t] = f2rch[t];
	}
	for(int i = 0; i < OXM_N_F4; i++) {
		P.f4_a[i] = f4a[i];
		P.f4_b[i] = f4b[i];
		P.f4_t0[i] = f4t0[i];
		P.f4_ts[i] = f4ts[i];
		P.f4_tc[i] = f4tc[i];
	}
	P.f4_sa = OXM_CXST_THETA1_SA;
	P.f4_sb = OXM_CXST_THETA1_SB;
	// support of each f4 in cos(theta): |theta - t0| < tc, widened by 1e-5 in the cosine (far
	// more than the FP32 error of an acos); open on a side that reaches 0 or pi
	const double pi = 3.141592653589793;
	for(int i = 0; i < OXM_N_F4; i++) {
		const double lo_t = (double) f4t0[i] - (double) f4tc[i], hi_t = (double) f4t0[i] + (double) f4tc[i];
		P.f4_chi[i] = lo_t <= 0.0 ? 2.0 : std::cos(lo_t) + 1e-5;
		P.f4_clo[i] = hi_t >= pi ? -2.0 : std::cos(hi_t) - 1e-5;
	}
	// the oxDNA2 pure-harmonic coaxial theta1 term adds for theta >= sb
	P.f4_clo[OXM_F4_CX_T1] = -2.0;
	P.f4_chi[OXM_F4_CX_T1] = std::fmax((double) P.f4_chi[OXM_F4_CX_T1], std::cos((double) OXM_CXST_THETA1_SB) + 1e-5);
	for(int i = 0; i < 4; i++) {
		P.f5_a[i] = f5a[i];
		P.f5_b[i] = f5b[i];
		P.f5_xc[i] = f5xc[i];
		P.f5_xs[i] = f5xs[i];
	}

	const double T = s.T;
	// exponent in float arithmetic on the float constants, exp in double
	const double st_x = 1 - std::exp((double) (-(f1rc[1] - f1r0[1]) * f1a[1]));
	const double hb_x = 1 - std::exp((double) (-(f1rc[0] - f1r0[0]) * f1a[0]));
	const double st_shift = st_x * st_x, hb_shift = hb_x * hb_x;
	const bool oxdna2_avg = s.average && !s.reference_cuda_eps;
	for(int i = 0; i < 5; i++) {
		for(int j = 0; j < 5; j++) {
			P.f1_eps[1][i][j] = oxdna2_avg ? OXM_STCK_BASE_EPS_OXDNA2 + OXM_STCK_FACT_EPS_OXDNA2 * T
										   : OXM_STCK_BASE_EPS_OXDNA + OXM_STCK_FACT_EPS_OXDNA * T;
			P.f1_eps[0][i][j] = oxdna2_avg ? OXM_HYDR_EPS_OXDNA2 : OXM_HYDR_EPS_OXDNA;
		}
	}
	if(!s.average) {
		const float fe = (float) s.seq_stck_fact_eps;
		float last = 0.f;
		for(int i = 0; i < 4; i++) {
			for(int j = 0; j < 4; j++) {
				last = (float) s.seq_stck[i][j];
				P.f1_eps[1][i][j] = last * (1.0 - fe + (T * 9.0 * fe));
			}
		}
		// entries of the dummy base keep the last value read when the file has none of them
		for(int i = 0; i < 5; i++)
			for(int j = 0; j < 5; j++)
				if(i == 4 || j == 4) P.f1_eps[1][i][j] = last * (1.0 - fe + (T * 9.0 * fe));
		const float at = (float) s.seq_hydr_at, gc = (float) s.seq_hydr_gc;
		P.f1_eps[0][0][3] = P.f1_eps[0][3][0] = at;
		P.f1_eps[0][1][2] = P.f1_eps[0][2][1] = gc;
	}
	for(int i = 0; i < 5; i++) {
		for(int j = 0; j < 5; j++) {
			P.f1_shift[1][i][j] = P.f1_eps[1][i][j] * st_shift;
			P.f1_shift[0][i][j] = P.f1_eps[0][i][j] * hb_shift;
		}
	}
	P.hb_multiplier = s.hb_multiplier;
	P.fene_r0 = OXM_FENE_R0_OXDNA2;

	P.use_mbf = s.use_mbf ? 1 : 0;
	if(s.use_mbf) {
		if(!(s.mbf_fmax > 0) || s.mbf_finf < 0) return -1;
		P.mbf_fmax = s.mbf_fmax;
		P.mbf_finf = s.mbf_finf;
		P.mbf_xmax = (-OXM_FENE_EPS + std::sqrt(OXM_FENE_EPS * OXM_FENE_EPS + 4.f * s.mbf_fmax * s.mbf_fmax * OXM_FENE_DELTA2)) /
				(2.f * s.mbf_fmax);
		P.mbf_fene_xmax = -(OXM_FENE_EPS / 2.f) * std::log(1.f - P.mbf_xmax * P.mbf_xmax / OXM_FENE_DELTA2);
		P.mbf_long_xmax = (P.mbf_fmax - P.mbf_finf) * P.mbf_xmax * std::log(P.mbf_xmax) + P.mbf_finf * P.mbf_xmax;
	}

	P.dh_half_charged_ends = s.dh_half_charged_ends ? 1 : 0;
	P.dh_prefactor = s.dh_strength;
	const double salt = (double) (float) s.salt;
	const double lambda_rhigh = s.dh_lambda * std::sqrt(T / 0.1f) / std::sqrt(salt);
	P.dh_rhigh = 3.0 * lambda_rhigh;
	const double lambda = s.dh_lambda * std::sqrt(T / 0.1) / std::sqrt(salt);
	P.dh_minus_kappa = -1.0 / lambda;
	const double x = P.dh_rhigh, q = P.dh_prefactor, l = lambda;
	P.dh_b = -(std::exp(-x / l) * q * q * (x + l) * (x + l)) / (-4. * x * x * x * l * l * q);
	P.dh_rc = x * (q * x + 3. * q * l) / (q * (x + l));

	const double rcutback = 2 * std::sqrt((double) ((OXM_POS_MM_BACK1) * (OXM_POS_MM_BACK1) + (OXM_POS_MM_BACK2) * (OXM_POS_MM_BACK2))) + OXM_EXCL_RC1;
	const double rcutbase = 2 * std::fabs(OXM_POS_BASE) + OXM_HYDR_RCHIGH;
	rcut = std::fmax(rcutback, rcutbase);
	const double debyecut = 2.0 * std::sqrt((double) (OXM_POS_MM_BACK1 * OXM_POS_MM_BACK1 + OXM_POS_MM_BACK2 * OXM_POS_MM_BACK2)) + P.dh_rc;
	if(debyecut > rcut) rcut = debyecut;
	P.rcut2 = rcut * rcut;
	P.box_hi = box;
	P.box_lo = 0.0;
	P.inv_box = 1.0 / box;
	P.pos_base_over_stack = (double) OXM_POS_BASE / (double) OXM_POS_STACK;
	return 0;
}

// FP32 copy of a table; the box side is split into a float and the float of the remainder
inline void to_float(const DNA2Table<double> &d, double box, DNA2Table<float> &f) {
	const double *src = reinterpret_cast<const double *>(&d);
	float *dst = reinterpret_cast<float *>(&f);
	// every member before the int fields is a double / float, in the same order
	const size_t nreal = offsetof(DNA2Table<double>, dh_half_charged_ends) / sizeof(double);
	for(size_t k = 0; k < nreal; k++) dst[k] = (float) src[k];
	f.dh_half_charged_ends = d.dh_half_charged_ends;
	f.use_mbf = d.use_mbf;
	f.box_hi = (float) box;
	f.box_lo = (float) (box - (double) f.box_hi);
	f.inv_box = (float) (1.0 / (double) f.box_hi);
}

// pair-distance bounds of the force kernel's term lists: a term can only act within these
// distances (model constants), widened by twice the skin so that a list built now stays complete
// until the next rebuild.  ev: centre-centre (excluded volume), base: base-base (hydrogen bonding,
// cross stacking), stk: stack-stack (coaxial stacking); evs: the excluded volume's four site
// pairs, of which one must be within its bound for a pair to enter the excluded-volume list.
// Squared, FP32.
struct TermRadii {
	float ev2, base2, stk2;
	float evs2[3];  // site pairs of the excluded volume: backbone-backbone, base-base, backbone-base
};

inline TermRadii term_radii(double skin) {
	const double back = std::sqrt((double) OXM_POS_MM_BACK1 * OXM_POS_MM_BACK1 + (double) OXM_POS_MM_BACK2 * OXM_POS_MM_BACK2);
	const double base = OXM_POS_BASE;
	double ev = OXM_EXCL_RC1 + 2 * back;                     // back-back
	ev = std::fmax(ev, (double) OXM_EXCL_RC2 + 2 * base);     // base-base
	ev = std::fmax(ev, (double) OXM_EXCL_RC3 + base + back);  // base-back
	const double hb = std::fmax((double) OXM_HYDR_RCHIGH, (double) OXM_CRST_RCHIGH);
	const double margin = 1e-3;
	TermRadii t;
	t.ev2 = (float) ((ev + 2 * skin + margin) * (ev + 2 * skin + margin));
	t.base2 = (float) ((hb + 2 * skin + margin) * (hb + 2 * skin + margin));
	t.stk2 = (float) (((double) OXM_CXST_RCHIGH + 2 * skin + margin) * ((double) OXM_CXST_RCHIGH + 2 * skin + margin));
	const double rc[3] = {OXM_EXCL_RC1, OXM_EXCL_RC2, std::fmax((double) OXM_EXCL_RC3, (double) OXM_EXCL_RC4)};
	for(int k = 0; k < 3; k++) t.evs2[k] = (float) ((rc[k] + 2 * skin + margin) * (rc[k] + 2 * skin + margin));
	return t;
}

// cells per side, CUDASimpleVerletList::_compute_N_cells_side
// (src/CUDA/Lists/CUDASimpleVerletList.cu:96-110), with the min-3 clamp applied last
inline int cells_per_side(int N, float L, float rverlet, bool auto_opt) {
	const float V3 = L * L * L;
	const float max_factor = (float) std::pow(2. * N / V3, 1. / 3.);
	const float min_cell = std::sqrt(rverlet * rverlet);
	int n = (int) (std::floor((double) L / (double) min_cell) + 0.1);
	if(auto_opt && n > std::ceil(max_factor * L)) n = (int) std::ceil(max_factor * L);
	if(n < 3) n = 3;
	return n;
}

}  // namespace oxgb
