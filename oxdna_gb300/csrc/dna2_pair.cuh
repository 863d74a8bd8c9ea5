// oxDNA2 pair physics for the GPU kernels, templated on the arithmetic type R (float for the
// production mixed-precision path, double for the FP64 parity path).
//
// The formulation is the reference CPU one (src/Interactions/DNAInteraction.cpp and
// src/Interactions/DNA2Interaction.cpp, DNA2_nomesh): every angular factor f4 is evaluated
// from the cosine of its angle, and its derivative enters as f4'(theta)/sin(theta) times
// un-normalised directions.  That form stays well conditioned in FP32 near aligned vectors,
// where the reference CUDA kernel's acos + normalised-cross form
// (src/CUDA/Interactions/CUDA_DNA.cuh:138-174,232-725) loses accuracy.  Only the forces and
// torques acting on one particle of a pair are formed for non-bonded pairs (the full
// neighbour list visits every pair from both ends); bonded pairs can return either side.
#pragma once

#include "dna2_model.h"
#include "oxgb_vec.cuh"
#include "split.cuh"

namespace oxgb {

// per-system parameter tables, filled on the host from the settings
template <typename R>
struct DNA2Table {
	R f1_eps[2][5][5], f1_shift[2][5][5];
	R f1_a[2], f1_r0[2], f1_blow[2], f1_bhigh[2], f1_rlow[2], f1_rhigh[2], f1_rclow[2], f1_rchigh[2];
	R f2_k[2], f2_r0[2], f2_rc[2], f2_blow[2], f2_bhigh[2], f2_rlow[2], f2_rhigh[2], f2_rclow[2], f2_rchigh[2];
	R f4_a[13], f4_b[13], f4_t0[13], f4_ts[13], f4_tc[13];
	R f4_sa, f4_sb;
	// support of f4 type i in cos(theta), slightly widened: outside (f4_clo, f4_chi) the factor
	// and its derivative are exactly zero, which a pair can be told from without an acos
	R f4_clo[13], f4_chi[13];
	R f5_a[4], f5_b[4], f5_xc[4], f5_xs[4];
	R hb_multiplier;
	R dh_prefactor, dh_rhigh, dh_rc, dh_b, dh_minus_kappa;
	R mbf_fmax, mbf_finf, mbf_xmax, mbf_fene_xmax, mbf_long_xmax;
	R fene_r0, rcut2;
	R box_hi, box_lo;  // box side as an unevaluated sum hi + lo (exact FP64 value)
	R inv_box;         // about 1 / box_hi: picks the periodic image (an integer; see LoadMixed::sep)
	R pos_base_over_stack;
	int dh_half_charged_ends, use_mbf, pad0, pad1;
};

// one nucleotide: lab-frame axes and interaction-site offsets from its centre
template <typename R>
struct Nuc {
	v3<R> a1, a2, a3, back, stack, base;
	int type, btype;
	bool is_end;
};

// grooved sites (src/Particles/DNANucleotide.cpp:66-82).  The reference forms the base site as
// stack * (POS_BASE / POS_STACK); the FP64 path keeps that, the FP32 path uses a1 * POS_BASE
// (the same value with one rounding instead of two).
template <typename R>
OXGB_HD void make_sites(const DNA2Table<R> &P, Nuc<R> &n) {
	n.back = n.a1 * R(OXM_POS_MM_BACK1) + n.a2 * R(OXM_POS_MM_BACK2);
	n.stack = n.a1 * R(OXM_POS_STACK);
	n.base = (sizeof(R) == 4) ? n.a1 * R(OXM_POS_BASE) : n.stack * P.pos_base_over_stack;
}

// centre-centre separation of a pair as an unevaluated sum hi + lo: the FP32 path carries the
// low part so that the stiff site-site vectors keep ~ulp accuracy; the other paths have lo = 0
template <typename R>
struct Sep {
	v3<R> hi, lo;
	OXGB_HD v3<R> plain() const { return hi + lo; }
};

// a * b - c * d from error-free products (Kahan's algorithm: within 1.5 ulp of the exact value)
template <typename R>
OXGB_HD R diff_of_products(R a, R b, R c, R d) {
	const R w = c * d;
	const R e = m_fma(-c, d, w);
	const R f = m_fma(a, b, -w);
	return f + e;
}

// (hi + lo) x b, the hi part with accurate 2x2 differences
template <typename R>
OXGB_HD v3<R> cross_accurate(const Sep<R> &a, const v3<R> &b) {
	const v3<R> h{diff_of_products(a.hi.y, b.z, a.hi.z, b.y), diff_of_products(a.hi.z, b.x, a.hi.x, b.z),
			diff_of_products(a.hi.x, b.y, a.hi.y, b.x)};
	return h + cross(a.lo, b);
}

template <typename R>
OXGB_HD void two_sum(R a, R b, R &s, R &e) {
	s = a + b;
	const R bb = s - a;
	e = (a - (s - bb)) + (b - bb);
}

// site-site vector r + qs - ps.  In FP32 the three-term sum is compensated (TwoSum on the site
// difference and on its sum with the separation), which removes the rounding of the ~1-long
// separation that otherwise dominates the error of the stiff radial terms (Morse minima of
// hydrogen bonding and stacking, FENE); in FP64 it is the reference's plain sum.
template <typename R>
OXGB_HD v3<R> site_vec(const Sep<R> &s, v3<R> qs, v3<R> ps) {
	if(sizeof(R) != 4) return (s.hi + qs) - ps;
	v3<R> d;
	R oh, ol, t, e;
	two_sum(qs.x, -ps.x, oh, ol);
	two_sum(s.hi.x, oh, t, e);
	d.x = t + ((e + ol) + s.lo.x);
	two_sum(qs.y, -ps.y, oh, ol);
	two_sum(s.hi.y, oh, t, e);
	d.y = t + ((e + ol) + s.lo.y);
	two_sum(qs.z, -ps.z, oh, ol);
	two_sum(s.hi.z, oh, t, e);
	d.z = t + ((e + ol) + s.lo.z);
	return d;
}

// energy-term slots, in the reference's split order
enum { T_FENE = 0, T_BEXC, T_STCK, T_NEXC, T_HB, T_CRST, T_CXST, T_DH, N_TERMS };

template <typename R>
struct PairOut {
	v3<R> F, T;  // force and lab-frame torque on the particle
	R E, Ehb;    // pair energy (all terms) and its hydrogen-bonding part
	R split[N_TERMS];
};

template <typename R, bool SPLIT>
OXGB_HD void add_e(PairOut<R> &o, int term, R e) {
	o.E += e;
	if(SPLIT) o.split[term] += e;
}

// ---------------------------------------------------------------- radial and angular factors

// r - c of a distance r + rl (rl: the remainder of the distance's FP32 rounding, 0 in FP64) and a
// model constant c.  The constants are FP32 literals of the reference (src/model.h), so for r
// within a factor of two of c the difference r - c is exact and only rl's rounding remains:
// the stiff radial factors (force slopes up to ~140) then see their argument to ~1e-10
// instead of the ~4e-8 of an FP32 distance.
template <typename R>
OXGB_HD R rdiff(R r, R c, R rl) {
	return (r - c) + rl;
}

// Morse f1 and its derivative (DNAInteraction.cpp:1239-1276); rl: see rdiff
template <typename R>
OXGB_HD void f1_both(const DNA2Table<R> &P, R r, int t, int i, int j, R &f, R &fd, R rl = R(0)) {
	f = R(0);
	fd = R(0);
	if(r < P.f1_rchigh[t]) {
		const R eps = P.f1_eps[t][i][j];
		if(r > P.f1_rhigh[t]) {
			const R d = rdiff(r, P.f1_rchigh[t], rl);
			f = eps * P.f1_bhigh[t] * d * d;
			fd = eps * (R(2) * P.f1_bhigh[t] * d);
		}
		else if(r > P.f1_rlow[t]) {
			// FP32: 1 - exp(-y) through expm1, exact near the well bottom where it cancels
			const R y = -rdiff(r, P.f1_r0[t], rl) * P.f1_a[t];
			const R x = m_exp(y);
			const R tmp = (sizeof(R) == 4) ? -m_expm1(y) : R(1) - x;
			f = eps * tmp * tmp - P.f1_shift[t][i][j];
			fd = eps * (R(2) * tmp * x * P.f1_a[t]);
		}
		else if(r > P.f1_rclow[t]) {
			const R d = rdiff(r, P.f1_rclow[t], rl);
			f = eps * P.f1_blow[t] * d * d;
			fd = eps * (R(2) * P.f1_blow[t] * d);
		}
	}
}

// harmonic f2 and its derivative (DNAInteraction.cpp:1278-1310); rl: see rdiff
template <typename R>
OXGB_HD void f2_both(const DNA2Table<R> &P, R r, int t, R &f, R &fd, R rl = R(0)) {
	f = R(0);
	fd = R(0);
	if(r < P.f2_rchigh[t]) {
		if(r > P.f2_rhigh[t]) {
			const R d = rdiff(r, P.f2_rchigh[t], rl);
			f = P.f2_k[t] * P.f2_bhigh[t] * d * d;
			fd = R(2) * P.f2_k[t] * P.f2_bhigh[t] * d;
		}
		else if(r > P.f2_rlow[t]) {
			const R d = rdiff(r, P.f2_r0[t], rl);
			f = (P.f2_k[t] / R(2)) * (d * d - (P.f2_rc[t] - P.f2_r0[t]) * (P.f2_rc[t] - P.f2_r0[t]));
			fd = P.f2_k[t] * d;
		}
		else if(r > P.f2_rclow[t]) {
			const R d = rdiff(r, P.f2_rclow[t], rl);
			f = P.f2_k[t] * P.f2_blow[t] * d * d;
			fd = R(2) * P.f2_k[t] * P.f2_blow[t] * d;
		}
	}
}

// |a x b|: the sine of the angle between the unit vectors a and b, for the FP32 path (0 in FP64,
// which takes the sine from the cosine)
template <typename R>
OXGB_HD R sin_between(const v3<R> &a, const v3<R> &b) {
	if(sizeof(R) != 4) return R(0);
	const v3<R> x = cross(a, b);
	return m_sqrt(dot(x, x));
}

// f4 of the angle whose cosine is c (and sine sn), and "f4D": minus f4'(theta)/sin(theta), the
// factor that multiplies the cosine's gradient (DNAInteraction.cpp:1312-1416,
// DNA2Interaction.cpp:308-352).  Set OXM_F4_CX_T1 adds the oxDNA2 pure-harmonic coaxial term.
// FP64 takes theta = acos(c) as the reference does.  FP32 takes theta = atan2(sn, c) with
// sn = |a x b|: the acos of a rounded cosine is off by d(cos) / sin(theta), ~2e-6 rad at
// theta = 0.1, where several modulations peak (theta0 = 0), which alone made force errors of
// 1e-5; atan2 of the cross product's norm is well conditioned at every angle.
template <typename R>
OXGB_HD void f4_both(const DNA2Table<R> &P, R c, R sn, int i, R &f, R &fd) {
	R t, s2, sint;
	if(sizeof(R) == 4) {
		t = m_atan2(sn, c);
		sint = sn;
		s2 = sn * sn;
	}
	else {
		c = m_max(R(-1), m_min(R(1), c));
		t = m_acos(c);
		s2 = m_fma(-c, c, R(1));  // sin^2(theta), with one rounding
		sint = m_sqrt(s2);
	}
	f = R(0);
	R dsin = R(0);
	R tt0 = t - P.f4_t0[i];
	R m = R(1);
	if(tt0 < R(0)) {
		tt0 = -tt0;
		m = R(-1);
	}
	if(tt0 < P.f4_tc[i]) {
		if(tt0 > P.f4_ts[i]) {
			f = P.f4_b[i] * (P.f4_tc[i] - tt0) * (P.f4_tc[i] - tt0);
			dsin = m * R(2) * P.f4_b[i] * (tt0 - P.f4_tc[i]) / sint;
		}
		else {
			f = R(1) - P.f4_a[i] * tt0 * tt0;
			dsin = (s2 > R(1e-8)) ? -m * R(2) * P.f4_a[i] * tt0 / sint : -m * R(2) * P.f4_a[i];
		}
	}
	if(i == OXM_F4_CX_T1) {
		const R h = t - P.f4_sb;
		if(h >= R(0)) {
			f += P.f4_sa * h * h;
			dsin += (s2 > R(1e-8)) ? R(2) * P.f4_sa * h / sint : R(2) * P.f4_sa;
		}
	}
	fd = -dsin;
}

// f4 of type i can be non-zero at cos(theta) = c
template <typename R>
OXGB_HD bool f4_may(const DNA2Table<R> &P, R c, int i) {
	return c > P.f4_clo[i] && c < P.f4_chi[i];
}

// f5 of cos(phi) and its derivative (DNAInteraction.cpp:1418-1450)
template <typename R>
OXGB_HD void f5_both(const DNA2Table<R> &P, R x, int t, R &f, R &fd) {
	f = R(0);
	fd = R(0);
	if(x > P.f5_xc[t]) {
		if(x < P.f5_xs[t]) {
			f = P.f5_b[t] * (P.f5_xc[t] - x) * (P.f5_xc[t] - x);
			fd = R(2) * P.f5_b[t] * (x - P.f5_xc[t]);
		}
		else if(x < R(0)) {
			f = R(1) - P.f5_a[t] * x * x;
			fd = R(-2) * P.f5_a[t] * x;
		}
		else f = R(1);
	}
}

// repulsive Lennard-Jones with quadratic smoothing; f = force on the second site
// (DNAInteraction.cpp:1182-1207)
template <typename R>
OXGB_HD R excl_vol(v3<R> r, R sigma, R rstar, R b, R rc, v3<R> &f) {
	const R rn = dot(r, r);
	f = v3<R>{R(0), R(0), R(0)};
	if(rn >= rc * rc) return R(0);
	if(rn > rstar * rstar) {
		const R rmod = m_sqrt(rn);
		const R rrc = rmod - rc;
		f = r * (-(R(2) * R(OXM_EXCL_EPS) * b * rrc / rmod));
		return R(OXM_EXCL_EPS) * b * rrc * rrc;
	}
	const R tmp = sigma * sigma / rn;
	const R lj = tmp * tmp * tmp;
	f = r * (-(R(24) * R(OXM_EXCL_EPS) * (lj - R(2) * lj * lj) / rn));
	return R(4) * R(OXM_EXCL_EPS) * (lj * lj - lj);
}

// ---------------------------------------------------------------- stiff excluded-volume contacts, FP32
//
// Inside its smoothing shell (rstar < r < rc) the excluded volume's force is 2 eps b (rc - r),
// with a slope 2 eps b of 1.6e4 (base-base), 6.8e3 and 3.6e3 per unit length.  There an FP32
// site distance (rounded to ~3e-8 at r ~ 0.33) or site offsets built from FP32-rounded axes
// (~2.4e-8) move the force by ~5e-4, far above the error of every other term.  The FP32 path
// therefore evaluates a site pair that the plain estimate puts inside rc (a few in a thousand
// listed pairs) once more: the site offsets carry the remainders of their FP32 rounding (from the
// FP64 quaternion, SiteLo), the site vector is a compensated sum kept as hi + lo, r^2 is a
// double-float, and rc - r = (rc^2 - r^2) / (rc + r), whose numerator is exact (r^2 and rc^2
// within a factor of 2; rc^2 a double-float constant).  The Lennard-Jones core (r < rstar) is
// well conditioned in relative terms and uses the refined site vector with r^2 rounded.

// remainders of a nucleotide's a1 and backbone offset (the base and stacking sites are
// multiples of a1): exact value = FP32 mirror + remainder, to ~2^-46
struct SiteLo {
	v3<float> a1, back;
};

// the FP64 and host paths refine nothing
struct NoRefine {
	static constexpr bool on = false;
	OXGB_HD SiteLo lo(int) const { return SiteLo{}; }
	template <int K>
	OXGB_HD float ev(const Sep<float> &, v3<float>, v3<float>, int, v3<float>, v3<float>, int, v3<float> &f) const {
		f = v3<float>{0.f, 0.f, 0.f};
		return 0.f;
	}
};

// the remainder of the site offset c a1 (c an FP32 constant: POS_BASE, POS_STACK) whose FP32
// value is hi = fl(c a1_hi), given a1's remainder a1l
OXGB_HD v3<float> multiple_lo(float c, v3<float> a1, v3<float> a1l, v3<float> hi) {
	return v3<float>{OXGB_FADD(OXGB_FMAF(c, a1.x, -hi.x), OXGB_FMUL(c, a1l.x)),
			OXGB_FADD(OXGB_FMAF(c, a1.y, -hi.y), OXGB_FMUL(c, a1l.y)), OXGB_FADD(OXGB_FMAF(c, a1.z, -hi.z), OXGB_FMUL(c, a1l.z))};
}

// a site of a nucleotide: its backbone (0) or base (1) site, the offset from the centre as hi +
// lo, from the FP32 offset `site` (the backbone offset, or fl(POS_BASE a1)), the FP32 axis a1
// and the remainders l
OXGB_HD void site_pair_of(v3<float> site, v3<float> a1, const SiteLo &l, int base, v3<float> &hi, v3<float> &lo) {
	hi = site;
	lo = base ? multiple_lo(float(OXM_POS_BASE), a1, l.a1, site) : l.back;
}

// the site-site vector sep + (qh + ql) - (ph + pl) as hi + lo (compensated sums)
OXGB_HD Sep<float> site_vec_lo(const Sep<float> &sep, v3<float> qh, v3<float> ql, v3<float> ph, v3<float> pl) {
	const float sh[3] = {sep.hi.x, sep.hi.y, sep.hi.z}, sl[3] = {sep.lo.x, sep.lo.y, sep.lo.z};
	const float qa[3] = {qh.x, qh.y, qh.z}, qb[3] = {ql.x, ql.y, ql.z}, pa[3] = {ph.x, ph.y, ph.z},
				pb[3] = {pl.x, pl.y, pl.z};
	float dh[3], dl[3];
#pragma unroll
	for(int k = 0; k < 3; k++) {
		const F2 o = two_sum(qa[k], -pa[k]);
		const float ol = OXGB_FADD(o.e, OXGB_FSUB(qb[k], pb[k]));
		const F2 t = two_sum(sh[k], o.s);
		const float l = OXGB_FADD(OXGB_FADD(t.e, ol), sl[k]);
		dh[k] = OXGB_FADD(t.s, l);
		dl[k] = OXGB_FSUB(l, OXGB_FSUB(dh[k], t.s));
	}
	return Sep<float>{v3<float>{dh[0], dh[1], dh[2]}, v3<float>{dl[0], dl[1], dl[2]}};
}

// |d|^2 of d = dh + dl as a double-float rn + rnl (error-free squares and sums; |dl|^2 dropped)
OXGB_HD void norm2_pair(const Sep<float> &d, float &rn, float &rnl) {
	const float dh[3] = {d.hi.x, d.hi.y, d.hi.z}, dl[3] = {d.lo.x, d.lo.y, d.lo.z};
	const float p0 = OXGB_FMUL(dh[0], dh[0]), p1 = OXGB_FMUL(dh[1], dh[1]), p2 = OXGB_FMUL(dh[2], dh[2]);
	const float e0 = OXGB_FMAF(dh[0], dh[0], -p0), e1 = OXGB_FMAF(dh[1], dh[1], -p1), e2 = OXGB_FMAF(dh[2], dh[2], -p2);
	const F2 s01 = two_sum(p0, p1);
	const F2 s012 = two_sum(s01.s, p2);
	const float cr = OXGB_FMAF(dh[0], dl[0], OXGB_FMAF(dh[1], dl[1], OXGB_FMUL(dh[2], dl[2])));
	const float lo = OXGB_FADD(OXGB_FADD(OXGB_FADD(s01.e, s012.e), OXGB_FADD(OXGB_FADD(e0, e1), e2)), OXGB_FMUL(2.f, cr));
	rn = OXGB_FADD(s012.s, lo);
	rnl = OXGB_FSUB(lo, OXGB_FSUB(rn, s012.s));
}

// the remainder r - rh of the distance r = |dh + dl| whose FP32 value is rh (within an ulp):
// (r^2 - rh^2) / (r + rh), with r^2 - rh^2 = fma(-rh, rh, rn) + rnl exact in its first term
OXGB_HD float dist_remainder(const Sep<float> &d, float rh) {
	float rn, rnl;
	norm2_pair(d, rn, rnl);
	return OXGB_FADD(OXGB_FMAF(-rh, rh, rn), rnl) / (2.f * rh);
}

// the excluded volume of site pair (ps of p, qs of q) from the refined site vector
// sep + (qh + ql) - (ph + pl); f = force on q's site; rc2h + rc2l = rc^2 (double-float)
OXGB_HD float excl_vol_refined(const Sep<float> &sep, v3<float> qh, v3<float> ql, v3<float> ph, v3<float> pl, float sigma,
		float rstar, float b, float rc, float rc2h, float rc2l, v3<float> &f) {
	const Sep<float> dd = site_vec_lo(sep, qh, ql, ph, pl);
	float rn, rnl;
	norm2_pair(dd, rn, rnl);
	const v3<float> d = dd.hi;
	f = v3<float>{0.f, 0.f, 0.f};
	if(rn > rc2h || (rn == rc2h && rnl >= rc2l)) return 0.f;
	if(rn > rstar * rstar) {
		const float rmod = m_sqrt(rn);
		const float rrc = OXGB_FADD(OXGB_FSUB(rn, rc2h), OXGB_FSUB(rnl, rc2l)) / (rmod + rc);  // r - rc
		f = d * (-(2.f * float(OXM_EXCL_EPS) * b * rrc / rmod));
		return float(OXM_EXCL_EPS) * b * rrc * rrc;
	}
	// the core's powers of r^-2 amplify a rounded r^2 some tenfold (forces there reach 10^3), so
	// this rarest branch takes r^2 = rn + rnl and the powers in FP64
	const double r2 = (double) rn + (double) rnl;
	const double tmp = (double) sigma * (double) sigma / r2;
	const double lj = tmp * tmp * tmp;
	const float fm = (float) (-(24.0 * (double) OXM_EXCL_EPS * (lj - 2.0 * lj * lj) / r2));
	f = v3<float>{(float) (fm * ((double) dd.hi.x + (double) dd.lo.x)), (float) (fm * ((double) dd.hi.y + (double) dd.lo.y)),
			(float) (fm * ((double) dd.hi.z + (double) dd.lo.z))};
	return (float) (4.0 * (double) OXM_EXCL_EPS * (lj * lj - lj));
}

// excluded-volume constants of one site pair: sigma, rstar, b, rc and rc^2 as a double-float
template <int K>
struct EVc;
template <>
struct EVc<1> {  // backbone-backbone
	static constexpr double S = OXM_EXCL_S1, R = OXM_EXCL_R1, B = OXM_EXCL_B1, RC = OXM_EXCL_RC1;
};
template <>
struct EVc<2> {  // base-base
	static constexpr double S = OXM_EXCL_S2, R = OXM_EXCL_R2, B = OXM_EXCL_B2, RC = OXM_EXCL_RC2;
};
template <>
struct EVc<3> {  // backbone (second) - base (first)
	static constexpr double S = OXM_EXCL_S3, R = OXM_EXCL_R3, B = OXM_EXCL_B3, RC = OXM_EXCL_RC3;
};
template <>
struct EVc<4> {  // base (second) - backbone (first)
	static constexpr double S = OXM_EXCL_S4, R = OXM_EXCL_R4, B = OXM_EXCL_B4, RC = OXM_EXCL_RC4;
};

// The refined evaluation of site pair K (site pbase of p, qbase of q: 1 base, 0 backbone), given
// the remainders of both nucleotides' offsets; f = force on q's site; plo (if given) receives
// the remainder of p's site offset (the lever arm of p's torque is ps + plo)
template <int K>
OXGB_HD float ev_refined(const Sep<float> &sep, v3<float> ps, v3<float> pa1, const SiteLo &pl_, int pbase, v3<float> qs,
		v3<float> qa1, const SiteLo &ql_, int qbase, v3<float> &f, v3<float> *plo = nullptr) {
	using C = EVc<K>;
	constexpr float rc2h = float(C::RC * C::RC);
	constexpr float rc2l = float(C::RC * C::RC - double(float(C::RC * C::RC)));
	v3<float> ph, pl, qh, ql;
	site_pair_of(ps, pa1, pl_, pbase, ph, pl);
	site_pair_of(qs, qa1, ql_, qbase, qh, ql);
	if(plo) *plo = pl;
	return excl_vol_refined(sep, qh, ql, ph, pl, float(C::S), float(C::R), float(C::B), float(C::RC), rc2h, rc2l, f);
}

// One excluded-volume site pair: site qbase of q against site pbase of p (1 base, 0 backbone),
// r = centre separation.  The plain evaluation, and in FP32 with a refining X the refined one
// (X::ev, kept out of line by the device refiner) for pairs inside the cutoff, with a relative
// margin well above the plain estimate's error.
template <int K, typename R, class X>
OXGB_HD R ev_site(const Sep<R> &sep, const v3<R> &r, const Nuc<R> &p, int pbase, const Nuc<R> &q, int qbase, const X &x,
		v3<R> &f) {
	using C = EVc<K>;
	const v3<R> ps = pbase ? p.base : p.back, qs = qbase ? q.base : q.back;
	const v3<R> d = r + qs - ps;
	R e = excl_vol(d, R(C::S), R(C::R), R(C::B), R(C::RC), f);
	if constexpr(X::on && sizeof(R) == 4) {
		if(dot(d, d) < R(C::RC * C::RC * 1.0001)) e = x.template ev<K>(sep, ps, p.a1, pbase, qs, q.a1, qbase, f);
	}
	return e;
}

// ---------------------------------------------------------------- non-bonded pair, p side

// The four site pairs of a non-bonded pair refined (FP32 engine path): adds the force and
// torque on p and returns the energy.  Site pairs outside their cutoff contribute nothing.
OXGB_HD float pair_ev_refined(const Sep<float> &sep, const Nuc<float> &p, const SiteLo &pl, const Nuc<float> &q,
		const SiteLo &ql, v3<float> &F, v3<float> &T) {
	// the torque's lever arm is p's site offset with its remainder: an FP32 arm alone is off by
	// ~2.4e-8, which the large forces of deep contacts would carry into the torque
	v3<float> f, lo;
	float e = ev_refined<2>(sep, p.base, p.a1, pl, 1, q.base, q.a1, ql, 1, f, &lo);
	F -= f;
	T -= cross(p.base, f) + cross(lo, f);
	e += ev_refined<4>(sep, p.back, p.a1, pl, 0, q.base, q.a1, ql, 1, f, &lo);
	F -= f;
	T -= cross(p.back, f) + cross(lo, f);
	e += ev_refined<3>(sep, p.base, p.a1, pl, 1, q.back, q.a1, ql, 0, f, &lo);
	F -= f;
	T -= cross(p.base, f) + cross(lo, f);
	e += ev_refined<1>(sep, p.back, p.a1, pl, 0, q.back, q.a1, ql, 0, f, &lo);
	F -= f;
	T -= cross(p.back, f) + cross(lo, f);
	return e;
}

// some site pair of (p, q) is inside its excluded-volume cutoff, by the plain FP32 estimate
// with a relative margin well above its error (FP32 engine path: only such pairs are evaluated,
// refined, by pair_ev_refined)
OXGB_HD bool ev_contact(const Nuc<float> &p, const Nuc<float> &q, const v3<float> r) {
	const v3<float> d2 = r + q.base - p.base, d4 = r + q.base - p.back, d3 = r + q.back - p.base, d1 = r + q.back - p.back;
	constexpr float m = 1.0001f;
	return dot(d2, d2) < float(EVc<2>::RC * EVc<2>::RC) * m || dot(d4, d4) < float(EVc<4>::RC * EVc<4>::RC) * m ||
			dot(d3, d3) < float(EVc<3>::RC * EVc<3>::RC) * m || dot(d1, d1) < float(EVc<1>::RC * EVc<1>::RC) * m;
}

// non-bonded excluded volume (DNAInteraction.cpp:707-777), plain
template <typename R, bool SPLIT>
OXGB_HD void pair_ev(const Nuc<R> &p, const Nuc<R> &q, const Sep<R> &sep, PairOut<R> &o) {
	const v3<R> r = sep.plain();
	v3<R> f;
	// excluded volume: base-base, back(p)-base(q), base(p)-back(q), back-back
	{
		R e = excl_vol(r + q.base - p.base, R(OXM_EXCL_S2), R(OXM_EXCL_R2), R(OXM_EXCL_B2), R(OXM_EXCL_RC2), f);
		o.F -= f;
		o.T -= cross(p.base, f);
		e += excl_vol(r + q.base - p.back, R(OXM_EXCL_S4), R(OXM_EXCL_R4), R(OXM_EXCL_B4), R(OXM_EXCL_RC4), f);
		o.F -= f;
		o.T -= cross(p.back, f);
		e += excl_vol(r + q.back - p.base, R(OXM_EXCL_S3), R(OXM_EXCL_R3), R(OXM_EXCL_B3), R(OXM_EXCL_RC3), f);
		o.F -= f;
		o.T -= cross(p.base, f);
		e += excl_vol(r + q.back - p.back, R(OXM_EXCL_S1), R(OXM_EXCL_R1), R(OXM_EXCL_B1), R(OXM_EXCL_RC1), f);
		o.F -= f;
		o.T -= cross(p.back, f);
		add_e<R, SPLIT>(o, T_NEXC, e);
	}
}

// The base-base vector of a pair and the cosines of its angles, shared by hydrogen bonding and
// cross stacking (DNAInteraction.cpp:779-1021), with which of the two can be non-zero: each
// needs its distance window and every angular factor inside its support (f4_may; else the term
// is exactly zero).
template <typename R>
struct BaseGeo {
	R rmod, c1, c2, c3, c4, c7, c8;
	v3<R> rd;
	bool hb, crst;
};

template <typename R>
OXGB_HD BaseGeo<R> base_geo(const DNA2Table<R> &P, const Nuc<R> &p, const Nuc<R> &q, const Sep<R> &sep) {
	BaseGeo<R> g;
	g.hb = g.crst = false;
	const v3<R> rhydro = site_vec(sep, q.base, p.base);
	const R rh2 = dot(rhydro, rhydro);
	const bool hb_range = p.btype + q.btype == 3 && R(OXM_HYDR_RCLOW) * R(OXM_HYDR_RCLOW) < rh2 &&
			rh2 < R(OXM_HYDR_RCHIGH) * R(OXM_HYDR_RCHIGH);
	const bool cr_range = R(OXM_CRST_RCLOW) * R(OXM_CRST_RCLOW) < rh2 && rh2 < R(OXM_CRST_RCHIGH) * R(OXM_CRST_RCHIGH);
	if(!hb_range && !cr_range) return g;
	g.rmod = m_sqrt(rh2);
	g.rd = rhydro * (R(1) / g.rmod);
	const v3<R> a1 = p.a1, a3 = p.a3, b1 = q.a1, b3 = q.a3;
	g.c1 = -dot(a1, b1), g.c2 = -dot(b1, g.rd), g.c3 = dot(a1, g.rd), g.c4 = dot(a3, b3), g.c7 = -dot(b3, g.rd), g.c8 = dot(a3, g.rd);
	g.hb = hb_range && R(OXM_HYDR_RCLOW) < g.rmod && g.rmod < R(OXM_HYDR_RCHIGH) && f4_may(P, g.c1, OXM_F4_HB_T1) &&
			f4_may(P, g.c2, OXM_F4_HB_T2) && f4_may(P, g.c3, OXM_F4_HB_T2) && f4_may(P, g.c4, OXM_F4_HB_T4) &&
			f4_may(P, g.c7, OXM_F4_HB_T7) && f4_may(P, g.c8, OXM_F4_HB_T7);
	// theta4, theta7, theta8 of cross stacking enter through f4(theta) + f4(pi - theta)
	g.crst = cr_range && R(OXM_CRST_RCLOW) < g.rmod && g.rmod < R(OXM_CRST_RCHIGH) && f4_may(P, g.c1, OXM_F4_CR_T1) &&
			f4_may(P, g.c2, OXM_F4_CR_T2) && f4_may(P, g.c3, OXM_F4_CR_T2) &&
			(f4_may(P, g.c4, OXM_F4_CR_T4) || f4_may(P, -g.c4, OXM_F4_CR_T4)) &&
			(f4_may(P, g.c7, OXM_F4_CR_T7) || f4_may(P, -g.c7, OXM_F4_CR_T7)) &&
			(f4_may(P, g.c8, OXM_F4_CR_T7) || f4_may(P, -g.c8, OXM_F4_CR_T7));
	return g;
}

// hydrogen bonding of a pair whose geometry admits it (g.hb)
template <typename R, bool SPLIT>
OXGB_HD void hb_term(const DNA2Table<R> &P, const Nuc<R> &p, const Nuc<R> &q, const BaseGeo<R> &g, PairOut<R> &o,
		R rl = R(0)) {
	const v3<R> a1 = p.a1, a3 = p.a3, b1 = q.a1, b3 = q.a3, rd = g.rd;
	const R rmod = g.rmod, c2 = g.c2, c3 = g.c3, c7 = g.c7, c8 = g.c8;
	const R hbm = (abs(q.btype) >= 300 && abs(p.btype) >= 300) ? P.hb_multiplier : R(1);
	R F1, F1D, g1, d1, g2, d2, g3, d3, g4, d4, g7, d7, g8, d8;
	f1_both(P, rmod, OXM_F1_HB, q.type, p.type, F1, F1D, rl);
	F1 *= hbm;
	F1D *= hbm;
	const R s1 = sin_between(a1, b1), s2 = sin_between(b1, rd), s3 = sin_between(a1, rd), s4 = sin_between(a3, b3),
			s7 = sin_between(b3, rd), s8 = sin_between(a3, rd);
	f4_both(P, g.c1, s1, OXM_F4_HB_T1, g1, d1);
	f4_both(P, c2, s2, OXM_F4_HB_T2, g2, d2);
	f4_both(P, c3, s3, OXM_F4_HB_T2, g3, d3);
	f4_both(P, g.c4, s4, OXM_F4_HB_T4, g4, d4);
	f4_both(P, c7, s7, OXM_F4_HB_T7, g7, d7);
	f4_both(P, c8, s8, OXM_F4_HB_T7, g8, d8);
	d3 = -d3;
	d4 = -d4;
	d8 = -d8;
	const R e = F1 * g1 * g2 * g3 * g4 * g7 * g8;
	if(e != R(0)) {
		add_e<R, SPLIT>(o, T_HB, e);
		o.Ehb += e;
		v3<R> force = rd * (-(F1D * g1 * g2 * g3 * g4 * g7 * g8));
		v3<R> tp = cross(a3, b3) * (F1 * g1 * g2 * g3 * d4 * g7 * g8);   // theta4: -= dir * (-..)
		tp += cross(a1, b1) * (F1 * d1 * g2 * g3 * g4 * g7 * g8);         // theta1
		force += (b1 + rd * c2) * (F1 * g1 * d2 * g3 * g4 * g7 * g8 / rmod);
		force += (a1 - rd * c3) * (F1 * g1 * g2 * d3 * g4 * g7 * g8 / rmod);
		tp += cross(rd, a1) * (-(F1 * g1 * g2 * d3 * g4 * g7 * g8));      // theta3
		force += (b3 + rd * c7) * (F1 * g1 * g2 * g3 * g4 * d7 * g8 / rmod);
		force += (a3 - rd * c8) * (F1 * g1 * g2 * g3 * g4 * g7 * d8 / rmod);
		tp += cross(rd, a3) * (-(F1 * g1 * g2 * g3 * g4 * g7 * d8));      // theta8
		o.F -= force;
		o.T += tp - cross(p.base, force);
	}
}

// cross stacking of a pair whose geometry admits it (g.crst)
template <typename R, bool SPLIT>
OXGB_HD void crst_term(const DNA2Table<R> &P, const Nuc<R> &p, const Nuc<R> &q, const BaseGeo<R> &g, PairOut<R> &o,
		R rl = R(0)) {
	const v3<R> a1 = p.a1, a3 = p.a3, b1 = q.a1, b3 = q.a3, rd = g.rd;
	const R rmod = g.rmod, c2 = g.c2, c3 = g.c3, c4 = g.c4, c7 = g.c7, c8 = g.c8;
	R F2, F2D, g1, d1, g2, d2, g3, d3, g4a, d4a, g4b, d4b, g7a, d7a, g7b, d7b, g8a, d8a, g8b, d8b;
	f2_both(P, rmod, OXM_F2_CRST, F2, F2D, rl);
	const R s1 = sin_between(a1, b1), s2 = sin_between(b1, rd), s3 = sin_between(a1, rd), s4 = sin_between(a3, b3),
			s7 = sin_between(b3, rd), s8 = sin_between(a3, rd);
	f4_both(P, g.c1, s1, OXM_F4_CR_T1, g1, d1);
	f4_both(P, c2, s2, OXM_F4_CR_T2, g2, d2);
	f4_both(P, c3, s3, OXM_F4_CR_T2, g3, d3);
	f4_both(P, c4, s4, OXM_F4_CR_T4, g4a, d4a);
	f4_both(P, -c4, s4, OXM_F4_CR_T4, g4b, d4b);
	f4_both(P, c7, s7, OXM_F4_CR_T7, g7a, d7a);
	f4_both(P, -c7, s7, OXM_F4_CR_T7, g7b, d7b);
	f4_both(P, c8, s8, OXM_F4_CR_T7, g8a, d8a);
	f4_both(P, -c8, s8, OXM_F4_CR_T7, g8b, d8b);
	const R g4 = g4a + g4b, g7 = g7a + g7b, g8 = g8a + g8b;
	d3 = -d3;
	const R d4 = -d4a + d4b, d7 = d7a - d7b, d8 = -d8a + d8b;
	const R e = F2 * g1 * g2 * g3 * g4 * g7 * g8;
	if(e != R(0)) {
		add_e<R, SPLIT>(o, T_CRST, e);
		v3<R> force = rd * (-(F2D * g1 * g2 * g3 * g4 * g7 * g8));
		v3<R> tp = cross(a1, b1) * (F2 * d1 * g2 * g3 * g4 * g7 * g8);
		force += (b1 + rd * c2) * (F2 * g1 * d2 * g3 * g4 * g7 * g8 / rmod);
		force += (a1 - rd * c3) * (F2 * g1 * g2 * d3 * g4 * g7 * g8 / rmod);
		tp += cross(rd, a1) * (-(F2 * g1 * g2 * d3 * g4 * g7 * g8));
		tp += cross(a3, b3) * (F2 * g1 * g2 * g3 * d4 * g7 * g8);
		force += (b3 + rd * c7) * (F2 * g1 * g2 * g3 * g4 * d7 * g8 / rmod);
		force += (a3 - rd * c8) * (F2 * g1 * g2 * g3 * g4 * g7 * d8 / rmod);
		tp += cross(rd, a3) * (-(F2 * g1 * g2 * g3 * g4 * g7 * d8));
		o.F -= force;
		o.T += tp - cross(p.base, force);
	}
}

// the remainder of the FP32 distance rh between the sites c a1 of p and q (c = POS_BASE for the
// base sites, POS_STACK for the stacking sites), from the remainders of their axes
OXGB_HD float site_dist_remainder(const Sep<float> &sep, const Nuc<float> &p, const SiteLo &pl, const Nuc<float> &q,
		const SiteLo &ql, bool stack, float rh) {
	const float c = stack ? float(OXM_POS_STACK) : float(OXM_POS_BASE);
	const v3<float> ps = stack ? p.stack : p.base, qs = stack ? q.stack : q.base;
	return dist_remainder(site_vec_lo(sep, qs, multiple_lo(c, q.a1, ql.a1, qs), ps, multiple_lo(c, p.a1, pl.a1, ps)), rh);
}

// hydrogen bonding and cross stacking, both on the base-base vector (DNAInteraction.cpp:779-1021)
template <typename R, bool SPLIT>
OXGB_HD void pair_base(const DNA2Table<R> &P, const Nuc<R> &p, const Nuc<R> &q, const Sep<R> &sep, PairOut<R> &o) {
	const BaseGeo<R> g = base_geo(P, p, q, sep);
	if(g.hb) hb_term<R, SPLIT>(P, p, q, g, o);
	if(g.crst) crst_term<R, SPLIT>(P, p, q, g, o);
}

// The stacking-site vector of a pair and its cosines, with whether coaxial stacking can be
// non-zero (distance window and every angular factor inside its support)
template <typename R>
struct StackGeo {
	R rmod, c1, c4, c5, c6;
	v3<R> rd;
	bool cxst;
};

template <typename R>
OXGB_HD StackGeo<R> stack_geo(const DNA2Table<R> &P, const Nuc<R> &p, const Nuc<R> &q, const Sep<R> &sep) {
	StackGeo<R> g;
	g.cxst = false;
	const v3<R> rstack = site_vec(sep, q.stack, p.stack);
	const R rs2 = dot(rstack, rstack);
	if(!(R(OXM_CXST_RCLOW) * R(OXM_CXST_RCLOW) < rs2 && rs2 < R(OXM_CXST_RCHIGH) * R(OXM_CXST_RCHIGH))) return g;
	g.rmod = m_sqrt(rs2);
	if(!(R(OXM_CXST_RCLOW) < g.rmod && g.rmod < R(OXM_CXST_RCHIGH))) return g;
	g.rd = rstack * (R(1) / g.rmod);
	g.c1 = -dot(p.a1, q.a1), g.c4 = dot(p.a3, q.a3), g.c5 = dot(p.a3, g.rd), g.c6 = -dot(q.a3, g.rd);
	g.cxst = f4_may(P, g.c1, OXM_F4_CX_T1) && f4_may(P, g.c4, OXM_F4_CX_T4) &&
			(f4_may(P, g.c5, OXM_F4_CX_T5) || f4_may(P, -g.c5, OXM_F4_CX_T5)) &&
			(f4_may(P, g.c6, OXM_F4_CX_T5) || f4_may(P, -g.c6, OXM_F4_CX_T5));
	return g;
}

// coaxial stacking, oxDNA2 form: no phi3 factor, pure-harmonic theta1 term
// (DNA2Interaction.cpp:214-306), of a pair whose geometry admits it (g.cxst)
template <typename R, bool SPLIT>
OXGB_HD void cxst_term(const DNA2Table<R> &P, const Nuc<R> &p, const Nuc<R> &q, const StackGeo<R> &g, PairOut<R> &o,
		R rl = R(0)) {
	const v3<R> a1 = p.a1, a3 = p.a3, b1 = q.a1, b3 = q.a3, rd = g.rd;
	const R rmod = g.rmod, c5 = g.c5, c6 = g.c6;
	R F2, F2D, g1, d1, g4, d4, g5a, d5a, g5b, d5b, g6a, d6a, g6b, d6b;
	f2_both(P, rmod, OXM_F2_CXST, F2, F2D, rl);
	const R s1 = sin_between(p.a1, q.a1), s4 = sin_between(p.a3, q.a3), s5 = sin_between(p.a3, g.rd),
			s6 = sin_between(q.a3, g.rd);
	f4_both(P, g.c1, s1, OXM_F4_CX_T1, g1, d1);
	f4_both(P, g.c4, s4, OXM_F4_CX_T4, g4, d4);
	f4_both(P, c5, s5, OXM_F4_CX_T5, g5a, d5a);
	f4_both(P, -c5, s5, OXM_F4_CX_T5, g5b, d5b);
	f4_both(P, c6, s6, OXM_F4_CX_T5, g6a, d6a);
	f4_both(P, -c6, s6, OXM_F4_CX_T5, g6b, d6b);
	const R g5 = g5a + g5b, g6 = g6a + g6b;
	d4 = -d4;
	const R d5 = -d5a + d5b, d6 = d6a - d6b;
	const R e = F2 * g1 * g4 * g5 * g6;
	if(e != R(0)) {
		add_e<R, SPLIT>(o, T_CXST, e);
		v3<R> force = rd * (-(F2D * g1 * g4 * g5 * g6));
		v3<R> tp = cross(a1, b1) * (F2 * d1 * g4 * g5 * g6);
		tp += cross(a3, b3) * (F2 * g1 * d4 * g5 * g6);
		const R f5 = F2 * g1 * g4 * d5 * g6;
		force += (a3 - rd * c5) * (f5 / rmod);
		tp -= cross(rd, a3) * f5;
		const R f6 = F2 * g1 * g4 * g5 * d6;
		force += (b3 + rd * c6) * (f6 / rmod);
		o.F -= force;
		o.T += tp - cross(p.stack, force);
	}
}

// coaxial stacking of a pair
template <typename R, bool SPLIT>
OXGB_HD void pair_stack(const DNA2Table<R> &P, const Nuc<R> &p, const Nuc<R> &q, const Sep<R> &sep, PairOut<R> &o) {
	const StackGeo<R> g = stack_geo(P, p, q, sep);
	if(g.cxst) cxst_term<R, SPLIT>(P, p, q, g, o);
}

// Debye-Hueckel between backbone sites rback = back site of q - back site of p, halved charges at
// strand ends (DNA2Interaction.cpp:157-212): the force on p and the energy; false outside the
// cutoff
template <typename R>
OXGB_HD bool dh_sites(const DNA2Table<R> &P, const v3<R> &rback, bool p_end, bool q_end, v3<R> &f, R &e) {
	const R rb2 = dot(rback, rback);
	if(!(rb2 < P.dh_rc * P.dh_rc)) return false;
	const R rmod = m_sqrt(rb2);
	if(!(rmod < P.dh_rc)) return false;
	R cut = R(1);
	if(P.dh_half_charged_ends && p_end) cut *= R(0.5);
	if(P.dh_half_charged_ends && q_end) cut *= R(0.5);
	const v3<R> rd = rback * (R(1) / rmod);
	R en, fm;
	if(rmod < P.dh_rhigh) {
		const R ex = m_exp(P.dh_minus_kappa * rmod);
		en = ex * (P.dh_prefactor / rmod);
		fm = -(P.dh_prefactor * ex) * (P.dh_minus_kappa / rmod - R(1) / (rmod * rmod));
	}
	else {
		en = P.dh_b * (rmod - P.dh_rc) * (rmod - P.dh_rc);
		fm = -(R(2) * P.dh_b * (rmod - P.dh_rc));
	}
	f = rd * (-(fm * cut));
	e = en * cut;
	return true;
}

// Debye-Hueckel of a pair from its centre separation r.  Reads only p.back, q.back and the
// strand-end flags.
template <typename R, bool SPLIT>
OXGB_HD void pair_dh(const DNA2Table<R> &P, const Nuc<R> &p, const Nuc<R> &q, const v3<R> r, PairOut<R> &o) {
	v3<R> f;
	R e;
	if(dh_sites(P, r + q.back - p.back, p.is_end, q.is_end, f, e)) {
		add_e<R, SPLIT>(o, T_DH, e);
		o.F += f;
		o.T += cross(p.back, f);
	}
}

template <typename R, bool SPLIT>
OXGB_HD void nonbonded_p(const DNA2Table<R> &P, const Nuc<R> &p, const Nuc<R> &q, const Sep<R> &sep, PairOut<R> &o) {
	const v3<R> r = sep.plain();
	if(dot(r, r) >= P.rcut2) return;
	pair_ev<R, SPLIT>(p, q, sep, o);
	pair_base<R, SPLIT>(P, p, q, sep, o);
	pair_stack<R, SPLIT>(P, p, q, sep, o);
	pair_dh<R, SPLIT>(P, p, q, r, o);
}

// ---------------------------------------------------------------- bonded pair

// p is the nucleotide whose 3' neighbour is q, r = q.centre - p.centre (no periodic image).
// Backbone FENE (with the optional max_backbone_force log tail), bonded excluded volume and
// stacking (DNAInteraction.cpp:415-705), evaluated once for both nucleotides: f is the force on
// q (-f acts on p), tp / tq the lab-frame torques on p / q.  Returns false if the backbone bond
// left the FENE range.
template <typename R>
struct BondOut {
	v3<R> f, tp, tq;
	R E;
	R split[3];  // FENE, bonded excluded volume, stacking
};

template <typename R, class X = NoRefine>
OXGB_HD bool bonded_both(const DNA2Table<R> &P, const Nuc<R> &p, const Nuc<R> &q, const Sep<R> &sep, BondOut<R> &b,
		const X &xr = X{}) {
	const v3<R> r = sep.plain();
	bool ok = true;
	b.f = b.tp = b.tq = v3<R>{R(0), R(0), R(0)};
	b.E = R(0);
	// refined FP32 path: the remainders of both nucleotides' site offsets, for the distances of
	// the stiff radial factors (FENE, stacking Morse)
	SiteLo lp{}, lq{};
	if constexpr(X::on && sizeof(R) == 4) {
		lp = xr.lo(0);
		lq = xr.lo(1);
	}
	// FENE
	{
		const v3<R> rback = site_vec(sep, q.back, p.back);
		const R rmod = m_sqrt(dot(rback, rback));
		R rl = R(0);
		if constexpr(X::on && sizeof(R) == 4) rl = dist_remainder(site_vec_lo(sep, q.back, lq.back, p.back, lp.back), rmod);
		const R x = rdiff(rmod, P.fene_r0, rl);
		v3<R> force;
		R e;
		if(P.use_mbf && m_fabs(x) > P.mbf_xmax) {
			const R ax = m_fabs(x);
			e = (P.mbf_fmax - P.mbf_finf) * P.mbf_xmax * m_log(ax) + P.mbf_finf * ax - P.mbf_long_xmax + P.mbf_fene_xmax;
			force = rback * (-m_copysign(R(1), x) * ((P.mbf_fmax - P.mbf_finf) * P.mbf_xmax / ax + P.mbf_finf) / rmod);
		}
		else if(m_fabs(x) >= R(OXM_FENE_DELTA)) {
			ok = false;
			e = R(0);
			force = v3<R>{R(0), R(0), R(0)};
		}
		else if(sizeof(R) == 4) {
			// FP32: Delta^2 - x^2 as (Delta - x)(Delta + x), exact to an ulp where a stretched
			// bond makes the difference of squares cancel (Delta - x is exact there)
			const R dd = (R(OXM_FENE_DELTA) - x) * (R(OXM_FENE_DELTA) + x);
			e = -(R(OXM_FENE_EPS) / R(2)) * m_log(dd / R(OXM_FENE_DELTA2));
			force = rback * (-(R(OXM_FENE_EPS) * x / dd) / rmod);
		}
		else {
			e = -(R(OXM_FENE_EPS) / R(2)) * m_log(R(1) - x * x / R(OXM_FENE_DELTA2));
			force = rback * (-(R(OXM_FENE_EPS) * x / (R(OXM_FENE_DELTA2) - x * x)) / rmod);
		}
		b.split[0] = e;
		b.f += force;
		b.tp -= cross(p.back, force);
		b.tq += cross(q.back, force);
	}
	// bonded excluded volume: base-base, base(p)-back(q), back(p)-base(q)
	{
		v3<R> f;
		R e = ev_site<2>(sep, r, p, 1, q, 1, xr, f);
		b.f += f;
		b.tp -= cross(p.base, f);
		b.tq += cross(q.base, f);
		e += ev_site<3>(sep, r, p, 1, q, 0, xr, f);
		b.f += f;
		b.tp -= cross(p.base, f);
		b.tq += cross(q.back, f);
		e += ev_site<4>(sep, r, p, 0, q, 1, xr, f);
		b.f += f;
		b.tp -= cross(p.back, f);
		b.tq += cross(q.base, f);
		b.split[1] = e;
	}
	// stacking
	b.split[2] = R(0);
	{
		const v3<R> a1 = p.a1, a2 = p.a2, a3 = p.a3, b1 = q.a1, b2 = q.a2, b3 = q.a3;
		const v3<R> rbackref = r + b1 * R(OXM_POS_BACK) - a1 * R(OXM_POS_BACK);
		const R rbr = m_sqrt(dot(rbackref, rbackref));
		const v3<R> rstack = site_vec(sep, q.stack, p.stack);
		const R rsm = m_sqrt(dot(rstack, rstack));
		R rl = R(0);
		if constexpr(X::on && sizeof(R) == 4) rl = site_dist_remainder(sep, p, lp, q, lq, true, rsm);
		const v3<R> rd = rstack * (R(1) / rsm);
		const R c4 = dot(a3, b3), c5 = dot(a3, rd), c6 = -dot(b3, rd);
		const R cp1 = dot(a2, rbackref) / rbr, cp2 = dot(b2, rbackref) / rbr;
		R F1, F1D, g4, d4, g5, d5, g6, d6, h1, h1d, h2, h2d;
		f1_both(P, rsm, OXM_F1_ST, q.type, p.type, F1, F1D, rl);
		const R s4 = sin_between(a3, b3), s5 = sin_between(a3, rd), s6 = sin_between(b3, rd);
		f4_both(P, c4, s4, OXM_F4_ST_T4, g4, d4);
		f4_both(P, -c5, s5, OXM_F4_ST_T5, g5, d5);
		f4_both(P, c6, s6, OXM_F4_ST_T5, g6, d6);
		f5_both(P, cp1, OXM_F5_PHI1, h1, h1d);
		f5_both(P, cp2, OXM_F5_PHI2, h2, h2d);
		d4 = -d4;
		d5 = -d5;
		d6 = -d6;
		const R e = F1 * g4 * g5 * g6 * h1 * h2;
		b.split[2] = e;
		if(e != R(0)) {
			const R gam = R(OXM_POS_STACK) - R(OXM_POS_BACK);
			const R rbr3 = rbr * rbr * rbr;
			v3<R> force = rd * (-(F1D * g4 * g5 * g6 * h1 * h2));
			force -= (a3 - rd * c5) * (F1 * g4 * d5 * g6 * h1 * h2 / rsm);
			force -= (b3 + rd * c6) * (F1 * g4 * g5 * d6 * h1 * h2 / rsm);

			const R ra2 = dot(rd, a2), ra1 = dot(rd, a1), rb1 = dot(rd, b1), a2b1 = dot(a2, b1);
			const R par1 = rsm * ra2 - a2b1 * gam;
			const R dc1dr = (rsm * rsm * ra2 - ra2 * rbr * rbr - rsm * (a2b1 + ra2 * (-ra1 + rb1)) * gam + a2b1 * (-ra1 + rb1) * gam * gam) / rbr3;
			const R dc1dra1 = rsm * gam * par1 / rbr3;
			const R dc1dra2 = -rsm / rbr;
			const R dc1drb1 = -rsm * gam * par1 / rbr3;
			const R dc1da1b1 = -gam * gam * par1 / rbr3;
			const R dc1da2b1 = gam / rbr;
			const R fp1 = -F1 * g4 * g5 * g6 * h1d * h2;
			force -= (rd * dc1dr + ((a2 - rd * ra2) * dc1dra2 + (a1 - rd * ra1) * dc1dra1 + (b1 - rd * rb1) * dc1drb1) * (R(1) / rsm)) * fp1;

			const R sb2 = dot(rd, b2), sb1 = dot(rd, b1), sa1 = dot(rd, a1), b2a1 = dot(b2, a1);
			const R par2 = rsm * sb2 + b2a1 * gam;
			const R dc2dr = (par2 * (rsm + (sa1 - sb1) * gam) - sb2 * rbr * rbr) / rbr3;
			const R dc2dra1 = -rsm * gam * (rsm * sb2 + b2a1 * gam) / rbr3;
			const R dc2dra2 = -rsm / rbr;
			const R dc2drb1 = rsm * gam * par2 / rbr3;
			const R dc2da1b1 = -gam * gam * par2 / rbr3;
			const R dc2da2b1 = -gam / rbr;
			const R fp2 = -F1 * g4 * g5 * g6 * h1 * h2d;
			force -= (rd * dc2dr + ((b2 - rd * sb2) * dc2dra2 + (b1 - rd * sb1) * dc2dra1 + (a1 - rd * sa1) * dc2drb1) * (R(1) / rsm)) * fp2;

			b.f += force;
			const v3<R> t4dir = cross(b3, a3);
			const R tm4 = F1 * d4 * g5 * g6 * h1 * h2;
			const v3<R> pure1 = cross(a2, b1) * (fp1 * dc1da2b1) + cross(a1, b1) * (fp1 * dc1da1b1);
			const v3<R> pure2 = cross(a1, b2) * (fp2 * dc2da2b1) + cross(a1, b1) * (fp2 * dc2da1b1);
			v3<R> tq = cross(q.stack, force) + t4dir * tm4;
			tq += cross(rd, b3) * (F1 * g4 * g5 * d6 * h1 * h2);
			tq += cross(rd, b1) * (fp1 * dc1drb1) + pure1;
			tq += cross(rd, b2) * (fp2 * dc2dra2) + cross(rd, b1) * (fp2 * dc2dra1) + pure2;
			b.tq += tq;
			v3<R> tp = -cross(p.stack, force) - t4dir * tm4;
			tp -= cross(rd, a3) * (-(F1 * g4 * d5 * g6 * h1 * h2));
			tp += cross(rd, a2) * (fp1 * dc1dra2) + cross(rd, a1) * (fp1 * dc1dra1) - pure1;
			tp += cross(rd, a1) * (fp2 * dc2drb1) - pure2;
			b.tp += tp;
		}
	}
	b.E = b.split[0] + b.split[1] + b.split[2];
	return ok;
}

// one side of a bonded pair: QSIDE selects q (force +f, torque tq) or p (force -f, torque tp)
template <typename R, bool SPLIT, bool QSIDE>
OXGB_HD bool bonded(const DNA2Table<R> &P, const Nuc<R> &p, const Nuc<R> &q, const Sep<R> &sep, PairOut<R> &o) {
	BondOut<R> b;
	const bool ok = bonded_both(P, p, q, sep, b);
	if(QSIDE) {
		o.F += b.f;
		o.T += b.tq;
	}
	else {
		o.F -= b.f;
		o.T += b.tp;
	}
	add_e<R, SPLIT>(o, T_FENE, b.split[0]);
	add_e<R, SPLIT>(o, T_BEXC, b.split[1]);
	add_e<R, SPLIT>(o, T_STCK, b.split[2]);
	return ok;
}

}  // namespace oxgb
