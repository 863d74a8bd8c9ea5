/*
 * ORACLE (test infrastructure only) -- CPU FP64 restatement of the reference oxDNA2 MD hot
 * path.  See dna2_oracle.h for what may use it.  Every function names the reference code it
 * restates.  The force field follows the reference CPU class DNA2Interaction_nomesh (exact
 * f4 through acos, no lookup meshes): src/Interactions/DNAInteraction.cpp and
 * src/Interactions/DNA2Interaction.cpp.  Compiled with -ffp-contract=off so that no
 * multiply-add is fused behind the source's back.
 */
#include "dna2_oracle.h"
#include "../oxdna_gb300/csrc/dna2_model.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SQR(x) ((x) * (x))

typedef struct {
	double x, y, z;
} vec;

static inline vec V(double x, double y, double z) {
	vec r = {x, y, z};
	return r;
}
static inline vec add(vec a, vec b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline vec sub(vec a, vec b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline vec mul(vec a, double s) { return V(a.x * s, a.y * s, a.z * s); }
static inline vec neg(vec a) { return V(-a.x, -a.y, -a.z); }
static inline double dot(vec a, vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline vec cross(vec a, vec b) { return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline double mod(vec a) { return sqrt(dot(a, a)); }
static inline vec load(const double *a, int i) { return V(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }

/* ---------------------------------------------------------------- parameters */

/* DNAInteraction::DNAInteraction + init + DNA2Interaction::DNA2Interaction + get_settings + init
 * (src/Interactions/DNAInteraction.cpp:12-213,290-380; src/Interactions/DNA2Interaction.cpp:5-21,62-155) */
int oxo_params_init(const oxo_settings *s, oxo_params *p) {
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
	memset(p, 0, sizeof(*p));
	p->T = s->T;
	for(int t = 0; t < 2; t++) {
		p->f1_a[t] = f1a[t]; p->f1_rc[t] = f1rc[t]; p->f1_r0[t] = f1r0[t]; p->f1_blow[t] = f1bl[t];
		p->f1_bhigh[t] = f1bh[t]; p->f1_rlow[t] = f1rl[t]; p->f1_rhigh[t] = f1rh[t]; p->f1_rclow[t] = f1rcl[t];
		p->f1_rchigh[t] = f1rch[t];
		p->f2_k[t] = f2k[t]; p->f2_rc[t] = f2rc[t]; p->f2_r0[t] = f2r0[t]; p->f2_blow[t] = f2bl[t];
		p->f2_rlow[t] = f2rl[t]; p->f2_rclow[t] = f2rcl[t]; p->f2_bhigh[t] = f2bh[t]; p->f2_rhigh[t] = f2rh[t];
		p->f2_rchigh[t] = f2rch[t];
	}
	for(int i = 0; i < 13; i++) {
		p->f4_a[i] = f4a[i]; p->f4_b[i] = f4b[i]; p->f4_t0[i] = f4t0[i]; p->f4_ts[i] = f4ts[i]; p->f4_tc[i] = f4tc[i];
	}
	p->f4_sa = OXM_CXST_THETA1_SA;
	p->f4_sb = OXM_CXST_THETA1_SB;
	for(int i = 0; i < 4; i++) {
		p->f5_a[i] = f5a[i]; p->f5_b[i] = f5b[i]; p->f5_xc[i] = f5xc[i]; p->f5_xs[i] = f5xs[i];
	}

	const double T = s->T;
	/* the exponent is float arithmetic on the float model constants, exp() is double */
	const double st_shift = SQR(1 - exp(-(f1rc[1] - f1r0[1]) * f1a[1]));
	const double hb_shift = SQR(1 - exp(-(f1rc[0] - f1r0[0]) * f1a[0]));
	/* oxDNA1 defaults for every base pair (DNAInteraction.cpp:313-324) */
	for(int i = 0; i < 5; i++) {
		for(int j = 0; j < 5; j++) {
			p->f1_eps[1][i][j] = OXM_STCK_BASE_EPS_OXDNA + OXM_STCK_FACT_EPS_OXDNA * T;
			p->f1_shift[1][i][j] = p->f1_eps[1][i][j] * st_shift;
			p->f1_eps[0][i][j] = OXM_HYDR_EPS_OXDNA;
			p->f1_shift[0][i][j] = p->f1_eps[0][i][j] * hb_shift;
		}
	}
	if(s->average) {
		/* oxDNA2 average-sequence well depths (DNA2Interaction.cpp:111-123) */
		for(int i = 0; i < 5; i++) {
			for(int j = 0; j < 5; j++) {
				p->f1_eps[1][i][j] = OXM_STCK_BASE_EPS_OXDNA2 + OXM_STCK_FACT_EPS_OXDNA2 * T;
				p->f1_shift[1][i][j] = p->f1_eps[1][i][j] * st_shift;
				p->f1_eps[0][i][j] = OXM_HYDR_EPS_OXDNA2;
				p->f1_shift[0][i][j] = p->f1_eps[0][i][j] * hb_shift;
			}
		}
	}
	else {
		/* sequence dependence (DNAInteraction.cpp:329-379): the file values are read as
		 * floats; dummy-base entries reuse the last value read when the file lacks them */
		const float fe = (float) s->seq_stck_fact_eps;
		float last = 0.f;
		for(int i = 0; i < 4; i++) {
			for(int j = 0; j < 4; j++) {
				last = (float) s->seq_stck[i][j];
				p->f1_eps[1][i][j] = last * (1.0 - fe + (T * 9.0 * fe));
				p->f1_shift[1][i][j] = p->f1_eps[1][i][j] * st_shift;
			}
		}
		for(int i = 0; i < 5; i++) {
			for(int j = 0; j < 5; j++) {
				if(i == 4 || j == 4) {
					p->f1_eps[1][i][j] = last * (1.0 - fe + (T * 9.0 * fe));
					p->f1_shift[1][i][j] = p->f1_eps[1][i][j] * st_shift;
				}
			}
		}
		const float at = (float) s->seq_hydr_at, gc = (float) s->seq_hydr_gc;
		p->f1_eps[0][0][3] = p->f1_eps[0][3][0] = at;
		p->f1_shift[0][0][3] = p->f1_shift[0][3][0] = p->f1_eps[0][0][3] * hb_shift;
		p->f1_eps[0][1][2] = p->f1_eps[0][2][1] = gc;
		p->f1_shift[0][1][2] = p->f1_shift[0][2][1] = p->f1_eps[0][1][2] * hb_shift;
	}
	p->hb_multiplier = s->hb_multiplier;
	p->fene_r0 = OXM_FENE_R0_OXDNA2;

	/* max_backbone_force (DNAInteraction.cpp:271-287) */
	p->use_mbf = s->use_mbf;
	if(s->use_mbf) {
		if(s->mbf_fmax < 0. || s->mbf_finf < 0.) return -2;
		p->mbf_fmax = s->mbf_fmax;
		p->mbf_finf = s->mbf_finf;
		p->mbf_xmax = (-OXM_FENE_EPS + sqrt(OXM_FENE_EPS * OXM_FENE_EPS + 4.f * p->mbf_fmax * p->mbf_fmax * OXM_FENE_DELTA2)) /
				(2.f * p->mbf_fmax);
	}

	/* Debye-Hueckel (DNA2Interaction.cpp:62-81 get_settings, 125-155 init); RHIGH is set in
	 * get_settings with T / 0.1f and kept, lambda is recomputed in init with T / 0.1 */
	p->dh_half_charged_ends = s->dh_half_charged_ends;
	p->dh_prefactor = s->dh_strength;
	const double lambda_settings = s->dh_lambda * sqrt(T / 0.1f) / sqrt((double) (float) s->salt);
	p->dh_rhigh = 3.0 * lambda_settings;
	const double lambda = s->dh_lambda * sqrt(T / 0.1) / sqrt((double) (float) s->salt);
	p->dh_lambda = lambda;
	p->dh_minus_kappa = -1.0 / lambda;
	const double x = p->dh_rhigh, q = p->dh_prefactor, l = lambda;
	p->dh_b = -(exp(-x / l) * q * q * (x + l) * (x + l)) / (-4. * x * x * x * l * l * q);
	p->dh_rc = x * (q * x + 3. * q * l) / (q * (x + l));

	/* cutoff: DNAInteraction::init (:291-303) then the Debye-Hueckel extension (DNA2 :136-148) */
	const double rcutback = 2 * sqrt((OXM_POS_MM_BACK1) * (OXM_POS_MM_BACK1) + (OXM_POS_MM_BACK2) * (OXM_POS_MM_BACK2)) + OXM_EXCL_RC1;
	const double rcutbase = 2 * fabs(OXM_POS_BASE) + OXM_HYDR_RCHIGH;
	p->rcut = fmax(rcutback, rcutbase);
	const double debyecut = 2.0 * sqrt(SQR(OXM_POS_MM_BACK1) + SQR(OXM_POS_MM_BACK2)) + p->dh_rc;
	if(debyecut > p->rcut) p->rcut = debyecut;
	return 0;
}

/* ---------------------------------------------------------------- radial / angular functions */

/* DNAInteraction::_f1 / _f1D (src/Interactions/DNAInteraction.cpp:1239-1276) */
static double f1(const oxo_params *P, double r, int t, int n3, int n5) {
	double val = 0.;
	if(r < P->f1_rchigh[t]) {
		if(r > P->f1_rhigh[t]) val = P->f1_eps[t][n3][n5] * P->f1_bhigh[t] * SQR(r - P->f1_rchigh[t]);
		else if(r > P->f1_rlow[t]) {
			double tmp = 1 - exp(-(r - P->f1_r0[t]) * P->f1_a[t]);
			val = P->f1_eps[t][n3][n5] * SQR(tmp) - P->f1_shift[t][n3][n5];
		}
		else if(r > P->f1_rclow[t]) val = P->f1_eps[t][n3][n5] * P->f1_blow[t] * SQR(r - P->f1_rclow[t]);
	}
	return val;
}

static double f1D(const oxo_params *P, double r, int t, int n3, int n5) {
	double val = 0.;
	if(r < P->f1_rchigh[t]) {
		if(r > P->f1_rhigh[t]) val = 2 * P->f1_bhigh[t] * (r - P->f1_rchigh[t]);
		else if(r > P->f1_rlow[t]) {
			double tmp = exp(-(r - P->f1_r0[t]) * P->f1_a[t]);
			val = 2 * (1 - tmp) * tmp * P->f1_a[t];
		}
		else if(r > P->f1_rclow[t]) val = 2 * P->f1_blow[t] * (r - P->f1_rclow[t]);
	}
	return P->f1_eps[t][n3][n5] * val;
}

/* DNAInteraction::_f2 / _f2D (:1278-1310) */
static double f2(const oxo_params *P, double r, int t) {
	double val = 0.;
	if(r < P->f2_rchigh[t]) {
		if(r > P->f2_rhigh[t]) val = P->f2_k[t] * P->f2_bhigh[t] * SQR(r - P->f2_rchigh[t]);
		else if(r > P->f2_rlow[t]) val = (P->f2_k[t] / 2.) * (SQR(r - P->f2_r0[t]) - SQR(P->f2_rc[t] - P->f2_r0[t]));
		else if(r > P->f2_rclow[t]) val = P->f2_k[t] * P->f2_blow[t] * SQR(r - P->f2_rclow[t]);
	}
	return val;
}

static double f2D(const oxo_params *P, double r, int t) {
	double val = 0.;
	if(r < P->f2_rchigh[t]) {
		if(r > P->f2_rhigh[t]) val = 2. * P->f2_k[t] * P->f2_bhigh[t] * (r - P->f2_rchigh[t]);
		else if(r > P->f2_rlow[t]) val = P->f2_k[t] * (r - P->f2_r0[t]);
		else if(r > P->f2_rclow[t]) val = 2. * P->f2_k[t] * P->f2_blow[t] * (r - P->f2_rclow[t]);
	}
	return val;
}

/* DNAInteraction::_f4 and _f4Dsin (:1356-1416) */
static double f4(const oxo_params *P, double t, int i) {
	double val = 0.;
	t -= P->f4_t0[i];
	if(t < 0) t *= -1;
	if(t < P->f4_tc[i]) {
		if(t > P->f4_ts[i]) val = P->f4_b[i] * SQR(P->f4_tc[i] - t);
		else val = 1. - P->f4_a[i] * SQR(t);
	}
	return val;
}

static double f4Dsin(const oxo_params *P, double t, int i) {
	double val = 0., m = 1.;
	double tt0 = t - P->f4_t0[i];
	if(tt0 < 0) {
		tt0 *= -1;
		m = -1.;
	}
	if(tt0 < P->f4_tc[i]) {
		double sint = sin(t);
		if(tt0 > P->f4_ts[i]) val = m * 2 * P->f4_b[i] * (tt0 - P->f4_tc[i]) / sint;
		else {
			if(SQR(sint) > 1e-8) val = -m * 2 * P->f4_a[i] * tt0 / sint;
			else val = -m * 2 * P->f4_a[i];
		}
	}
	return val;
}

/* DNA2Interaction::_f4_pure_harmonic / _f4Dsin_pure_harmonic (src/Interactions/DNA2Interaction.cpp:326-352) */
static double f4_harm(const oxo_params *P, double t) {
	t -= P->f4_sb;
	return (t < 0) ? 0. : P->f4_sa * SQR(t);
}

static double f4Dsin_harm(const oxo_params *P, double t) {
	double tt0 = t - P->f4_sb;
	if(tt0 < 0) return 0.;
	double sint = sin(t);
	return (SQR(sint) > 1e-8) ? 2 * P->f4_sa * tt0 / sint : 2 * P->f4_sa;
}

static double safe_acos(double x) { return acos(fmax(-1.0, fmin(1.0, x))); }

/* DNA2Interaction_nomesh::_custom_f4 / _custom_f4D (src/Interactions/DNA2Interaction.h:121-152):
 * DNAInteraction::_fakef4/_fakef4D (DNAInteraction.cpp:1312-1330) for every set but the
 * coaxial theta1, which uses DNA2Interaction::_fakef4_cxst_t1/_fakef4D_cxst_t1 (DNA2:308-324) */
static double cf4(const oxo_params *P, double cost, int i) {
	if(i != OXM_F4_CX_T1) return f4(P, safe_acos(cost), i);
	if(cost * cost > 1) cost = copysign(1, cost);
	double t = acos(cost);
	return f4(P, t, i) + f4_harm(P, t);
}

static double cf4D(const oxo_params *P, double cost, int i) {
	if(i != OXM_F4_CX_T1) return -f4Dsin(P, safe_acos(cost), i);
	if(cost * cost > 1) cost = copysign(1, cost);
	double t = acos(cost);
	return -f4Dsin(P, t, i) - f4Dsin_harm(P, t);
}

/* DNAInteraction::_f5 / _f5D (:1418-1450) */
static double f5(const oxo_params *P, double f, int t) {
	double val = 0.;
	if(f > P->f5_xc[t]) {
		if(f < P->f5_xs[t]) val = P->f5_b[t] * SQR(P->f5_xc[t] - f);
		else if(f < 0) val = 1. - P->f5_a[t] * SQR(f);
		else val = 1.;
	}
	return val;
}

static double f5D(const oxo_params *P, double f, int t) {
	double val = 0.;
	if(f > P->f5_xc[t]) {
		if(f < P->f5_xs[t]) val = 2 * P->f5_b[t] * (f - P->f5_xc[t]);
		else if(f < 0) val = -2. * P->f5_a[t] * f;
	}
	return val;
}

/* DNAInteraction::_repulsive_lj (:1182-1207); *force is the force on q */
static double repulsive_lj(vec r, vec *force, double sigma, double rstar, double b, double rc) {
	double rnorm = SQR(r.x) + SQR(r.y) + SQR(r.z);
	double energy = 0.;
	*force = V(0., 0., 0.);
	if(rnorm < SQR(rc)) {
		if(rnorm > SQR(rstar)) {
			double rmod = sqrt(rnorm);
			double rrc = rmod - rc;
			energy = OXM_EXCL_EPS * b * SQR(rrc);
			*force = mul(neg(r), 2 * OXM_EXCL_EPS * b * rrc / rmod);
		}
		else {
			double tmp = SQR(sigma) / rnorm;
			double lj_part = tmp * tmp * tmp;
			energy = 4 * OXM_EXCL_EPS * (SQR(lj_part) - lj_part);
			*force = mul(neg(r), 24 * OXM_EXCL_EPS * (lj_part - 2 * SQR(lj_part)) / rnorm);
		}
	}
	if(energy == 0.) *force = V(0., 0., 0.);
	return energy;
}

/* ---------------------------------------------------------------- per-particle context */

typedef struct {
	vec pos, a1, a2, a3, back, stack, base;
	int type, btype, n3, n5;
} nuc;

typedef struct {
	double *F, *T; /* accumulators: lab-frame force, LAB-frame torque (rotated at the end) */
	double *E_split, *E_part;
	int err;
} acc;

static inline void add_force(acc *A, int i, vec f) {
	A->F[3 * i] += f.x;
	A->F[3 * i + 1] += f.y;
	A->F[3 * i + 2] += f.z;
}

/* the reference adds p->orientationT * torque per term; rotations are linear, so the oracle
 * keeps lab-frame sums and rotates once (differences are rounding only) */
static inline void add_torque(acc *A, int i, vec t) {
	A->T[3 * i] += t.x;
	A->T[3 * i + 1] += t.y;
	A->T[3 * i + 2] += t.z;
}

static inline void add_energy(acc *A, int term, int p, int q, double e) {
	A->E_split[term] += e;
	A->E_part[p] += e;
	A->E_part[q] += e;
}

/* DNANucleotide::set_positions, grooved (src/Particles/DNANucleotide.cpp:66-82) */
static void make_nuc(nuc *n, const double *pos, const double *a1, const double *a2, const double *a3, int i) {
	n->pos = load(pos, i);
	n->a1 = load(a1, i);
	n->a2 = load(a2, i);
	n->a3 = load(a3, i);
	n->back = add(mul(n->a1, (double) OXM_POS_MM_BACK1), mul(n->a2, (double) OXM_POS_MM_BACK2));
	n->stack = mul(n->a1, (double) OXM_POS_STACK);
	n->base = mul(n->stack, (double) OXM_POS_BASE / (double) OXM_POS_STACK);
}

/* ---------------------------------------------------------------- bonded terms */

/* p is the nucleotide whose 3' neighbour is q; r = q.pos - p.pos (no periodic image).
 * DNAInteraction::_backbone (:415-466), _bonded_excluded_volume (:468-528), _stacking (:530-705) */
static void bonded_pair(const oxo_params *P, const nuc *p, const nuc *q, int ip, int iq, vec r, acc *A) {
	/* FENE */
	vec rback = add(r, sub(q->back, p->back));
	double rbackmod = mod(rback);
	double rbackr0 = rbackmod - P->fene_r0;
	vec force;
	double energy;
	if(P->use_mbf && fabs(rbackr0) > P->mbf_xmax) {
		double fene_xmax = -(OXM_FENE_EPS / 2.f) * log(1.f - SQR(P->mbf_xmax) / OXM_FENE_DELTA2);
		double long_xmax = (P->mbf_fmax - P->mbf_finf) * P->mbf_xmax * log(P->mbf_xmax) + P->mbf_finf * P->mbf_xmax;
		energy = (P->mbf_fmax - P->mbf_finf) * P->mbf_xmax * log(fabs(rbackr0)) + P->mbf_finf * fabs(rbackr0) - long_xmax + fene_xmax;
		force = mul(rback, -copysign(1.f, rbackr0) * ((P->mbf_fmax - P->mbf_finf) * P->mbf_xmax / fabs(rbackr0) + P->mbf_finf) / rbackmod);
	}
	else {
		if(fabs(rbackr0) > OXM_FENE_DELTA - DBL_EPSILON) {
			A->err = -1;
			energy = 1.e12;
			add_energy(A, OXO_FENE, ip, iq, energy);
			return;
		}
		energy = -(OXM_FENE_EPS / 2.f) * log(1.f - SQR(rbackr0) / OXM_FENE_DELTA2);
		force = mul(rback, -(OXM_FENE_EPS * rbackr0 / (OXM_FENE_DELTA2 - SQR(rbackr0))) / rbackmod);
	}
	add_energy(A, OXO_FENE, ip, iq, energy);
	add_force(A, ip, neg(force));
	add_force(A, iq, force);
	add_torque(A, ip, neg(cross(p->back, force)));
	add_torque(A, iq, cross(q->back, force));

	/* bonded excluded volume: base-base, p-base/q-back, p-back/q-base */
	const struct {
		const vec *ps, *qs;
		double s, rs, b, rc;
	} ev[3] = {{&p->base, &q->base, OXM_EXCL_S2, OXM_EXCL_R2, OXM_EXCL_B2, OXM_EXCL_RC2},
			{&p->base, &q->back, OXM_EXCL_S3, OXM_EXCL_R3, OXM_EXCL_B3, OXM_EXCL_RC3},
			{&p->back, &q->base, OXM_EXCL_S4, OXM_EXCL_R4, OXM_EXCL_B4, OXM_EXCL_RC4}};
	for(int k = 0; k < 3; k++) {
		vec rc = add(r, sub(*ev[k].qs, *ev[k].ps));
		double e = repulsive_lj(rc, &force, ev[k].s, ev[k].rs, ev[k].b, ev[k].rc);
		add_energy(A, OXO_BEXC, ip, iq, e);
		add_force(A, ip, neg(force));
		add_force(A, iq, force);
		add_torque(A, ip, neg(cross(*ev[k].ps, force)));
		add_torque(A, iq, cross(*ev[k].qs, force));
	}

	/* stacking */
	const vec a1 = p->a1, a2 = p->a2, a3 = p->a3, b1 = q->a1, b2 = q->a2, b3 = q->a3;
	vec rbackref = add(r, sub(mul(b1, (double) OXM_POS_BACK), mul(a1, (double) OXM_POS_BACK)));
	double rbackrefmod = mod(rbackref);
	vec rstack = add(r, sub(q->stack, p->stack));
	double rstackmod = mod(rstack);
	vec rstackdir = mul(rstack, 1. / rstackmod);
	double cost4 = dot(a3, b3);
	double cost5 = dot(a3, rstackdir);
	double cost6 = -dot(b3, rstackdir);
	double cosphi1 = dot(a2, rbackref) / rbackrefmod;
	double cosphi2 = dot(b2, rbackref) / rbackrefmod;
	double F1 = f1(P, rstackmod, OXM_F1_ST, q->type, p->type);
	double f4t4 = cf4(P, cost4, OXM_F4_ST_T4);
	double f4t5 = cf4(P, -cost5, OXM_F4_ST_T5);
	double f4t6 = cf4(P, cost6, OXM_F4_ST_T5);
	double f5phi1 = f5(P, cosphi1, OXM_F5_PHI1);
	double f5phi2 = f5(P, cosphi2, OXM_F5_PHI2);
	energy = F1 * f4t4 * f4t5 * f4t6 * f5phi1 * f5phi2;
	add_energy(A, OXO_STCK, ip, iq, energy);
	if(energy == 0.) return;

	vec tp = V(0, 0, 0), tq = V(0, 0, 0);
	double F1D = f1D(P, rstackmod, OXM_F1_ST, q->type, p->type);
	double f4t4Dsin = -cf4D(P, cost4, OXM_F4_ST_T4);
	double f4t5Dsin = -cf4D(P, -cost5, OXM_F4_ST_T5);
	double f4t6Dsin = -cf4D(P, cost6, OXM_F4_ST_T5);
	double f5phi1D = f5D(P, cosphi1, OXM_F5_PHI1);
	double f5phi2D = f5D(P, cosphi2, OXM_F5_PHI2);

	force = mul(neg(rstackdir), F1D * f4t4 * f4t5 * f4t6 * f5phi1 * f5phi2);
	force = add(force, mul(neg(sub(a3, mul(rstackdir, cost5))), F1 * f4t4 * f4t5Dsin * f4t6 * f5phi1 * f5phi2 / rstackmod));
	force = add(force, mul(neg(add(b3, mul(rstackdir, cost6))), F1 * f4t4 * f4t5 * f4t6Dsin * f5phi1 * f5phi2 / rstackmod));

	const double gamma = OXM_POS_STACK - OXM_POS_BACK;
	double rbrc = rbackrefmod * rbackrefmod * rbackrefmod;
	double ra2 = dot(rstackdir, a2), ra1 = dot(rstackdir, a1), rb1 = dot(rstackdir, b1), a2b1 = dot(a2, b1);
	double par = rstackmod * ra2 - a2b1 * gamma;
	double dc1dr = (SQR(rstackmod) * ra2 - ra2 * SQR(rbackrefmod) - rstackmod * (a2b1 + ra2 * (-ra1 + rb1)) * gamma +
			a2b1 * (-ra1 + rb1) * SQR(gamma)) / rbrc;
	double dc1dra1 = rstackmod * gamma * par / rbrc;
	double dc1dra2 = -rstackmod / rbackrefmod;
	double dc1drb1 = -rstackmod * gamma * par / rbrc;
	double dc1da1b1 = -SQR(gamma) * par / rbrc;
	double dc1da2b1 = gamma / rbackrefmod;
	double fp1 = -F1 * f4t4 * f4t5 * f4t6 * f5phi1D * f5phi2;
	vec g = add(add(mul(sub(a2, mul(rstackdir, ra2)), dc1dra2), mul(sub(a1, mul(rstackdir, ra1)), dc1dra1)),
			mul(sub(b1, mul(rstackdir, rb1)), dc1drb1));
	force = add(force, mul(neg(add(mul(rstackdir, dc1dr), mul(g, 1. / rstackmod))), fp1));

	double rb2 = dot(rstackdir, b2), rb1b = dot(rstackdir, b1), ra1b = dot(rstackdir, a1), b2a1 = dot(b2, a1);
	double par2 = rstackmod * rb2 + b2a1 * gamma;
	double dc2dr = (par2 * (rstackmod + (ra1b - rb1b) * gamma) - rb2 * SQR(rbackrefmod)) / rbrc;
	double dc2dra1 = -rstackmod * gamma * (rstackmod * rb2 + b2a1 * gamma) / rbrc;
	double dc2dra2 = -rstackmod / rbackrefmod;
	double dc2drb1 = rstackmod * gamma * par2 / rbrc;
	double dc2da1b1 = -SQR(gamma) * par2 / rbrc;
	double dc2da2b1 = -gamma / rbackrefmod;
	double fp2 = -F1 * f4t4 * f4t5 * f4t6 * f5phi1 * f5phi2D;
	vec g2 = add(add(mul(sub(b2, mul(rstackdir, rb2)), dc2dra2), mul(sub(b1, mul(rstackdir, rb1b)), dc2dra1)),
			mul(sub(a1, mul(rstackdir, ra1b)), dc2drb1));
	force = add(force, mul(add(mul(rstackdir, dc2dr), mul(g2, 1. / rstackmod)), -fp2));

	add_force(A, ip, neg(force));
	add_force(A, iq, force);
	tp = sub(tp, cross(p->stack, force));
	tq = add(tq, cross(q->stack, force));

	vec t4dir = cross(b3, a3);
	double tm = F1 * f4t4Dsin * f4t5 * f4t6 * f5phi1 * f5phi2;
	tp = sub(tp, mul(t4dir, tm));
	tq = add(tq, mul(t4dir, tm));
	vec t5dir = cross(rstackdir, a3);
	tm = -F1 * f4t4 * f4t5Dsin * f4t6 * f5phi1 * f5phi2;
	tp = sub(tp, mul(t5dir, tm));
	vec t6dir = cross(rstackdir, b3);
	tm = F1 * f4t4 * f4t5 * f4t6Dsin * f5phi1 * f5phi2;
	tq = add(tq, mul(t6dir, tm));

	tp = add(tp, add(mul(cross(rstackdir, a2), fp1 * dc1dra2), mul(cross(rstackdir, a1), fp1 * dc1dra1)));
	tq = add(tq, mul(cross(rstackdir, b1), fp1 * dc1drb1));
	vec pure = add(mul(cross(a2, b1), fp1 * dc1da2b1), mul(cross(a1, b1), fp1 * dc1da1b1));
	tp = sub(tp, pure);
	tq = add(tq, pure);

	tp = add(tp, mul(cross(rstackdir, a1), fp2 * dc2drb1));
	tq = add(tq, add(mul(cross(rstackdir, b2), fp2 * dc2dra2), mul(cross(rstackdir, b1), fp2 * dc2dra1)));
	pure = add(mul(cross(a1, b2), fp2 * dc2da2b1), mul(cross(a1, b1), fp2 * dc2da1b1));
	tp = sub(tp, pure);
	tq = add(tq, pure);

	add_torque(A, ip, tp);
	add_torque(A, iq, tq);
}

/* ---------------------------------------------------------------- non-bonded terms */

/* DNA2Interaction::pair_interaction_nonbonded (src/Interactions/DNA2Interaction.cpp:42-60) with
 * _nonbonded_excluded_volume (DNAInteraction.cpp:707-777), _hydrogen_bonding (:779-902),
 * _cross_stacking (:904-1021), DNA2 _coaxial_stacking (DNA2Interaction.cpp:214-306) and
 * _debye_huckel (DNA2Interaction.cpp:157-212); r = minimum image of q.pos - p.pos */
static void nonbonded_pair(const oxo_params *P, const nuc *p, const nuc *q, int ip, int iq, vec r, acc *A) {
	if(dot(r, r) >= SQR(P->rcut)) return;
	if(p->n3 == iq || p->n5 == iq) return;

	vec force, tp, tq;
	const vec a1 = p->a1, a3 = p->a3, b1 = q->a1, b3 = q->a3;

	/* excluded volume: base-base, p-back/q-base, p-base/q-back, back-back */
	const struct {
		const vec *ps, *qs;
		double s, rs, b, rc;
	} ev[4] = {{&p->base, &q->base, OXM_EXCL_S2, OXM_EXCL_R2, OXM_EXCL_B2, OXM_EXCL_RC2},
			{&p->back, &q->base, OXM_EXCL_S4, OXM_EXCL_R4, OXM_EXCL_B4, OXM_EXCL_RC4},
			{&p->base, &q->back, OXM_EXCL_S3, OXM_EXCL_R3, OXM_EXCL_B3, OXM_EXCL_RC3},
			{&p->back, &q->back, OXM_EXCL_S1, OXM_EXCL_R1, OXM_EXCL_B1, OXM_EXCL_RC1}};
	tp = V(0, 0, 0);
	tq = V(0, 0, 0);
	for(int k = 0; k < 4; k++) {
		vec rc = add(r, sub(*ev[k].qs, *ev[k].ps));
		double e = repulsive_lj(rc, &force, ev[k].s, ev[k].rs, ev[k].b, ev[k].rc);
		add_energy(A, OXO_NEXC, ip, iq, e);
		tp = sub(tp, cross(*ev[k].ps, force));
		tq = add(tq, cross(*ev[k].qs, force));
		add_force(A, ip, neg(force));
		add_force(A, iq, force);
	}
	add_torque(A, ip, tp);
	add_torque(A, iq, tq);

	/* hydrogen bonding */
	vec rhydro = add(r, sub(q->base, p->base));
	double rhydromod = mod(rhydro);
	int is_pair = (q->btype + p->btype == 3);
	double hb_multi = (abs(q->btype) >= 300 && abs(p->btype) >= 300) ? P->hb_multiplier : 1.f;
	if(is_pair && OXM_HYDR_RCLOW < rhydromod && rhydromod < OXM_HYDR_RCHIGH) {
		vec rhydrodir = mul(rhydro, 1. / rhydromod);
		double cost1 = -dot(a1, b1), cost2 = -dot(b1, rhydrodir), cost3 = dot(a1, rhydrodir);
		double cost4 = dot(a3, b3), cost7 = -dot(b3, rhydrodir), cost8 = dot(a3, rhydrodir);
		double F1 = hb_multi * f1(P, rhydromod, OXM_F1_HB, q->type, p->type);
		double f4t1 = cf4(P, cost1, OXM_F4_HB_T1), f4t2 = cf4(P, cost2, OXM_F4_HB_T2), f4t3 = cf4(P, cost3, OXM_F4_HB_T2);
		double f4t4 = cf4(P, cost4, OXM_F4_HB_T4), f4t7 = cf4(P, cost7, OXM_F4_HB_T7), f4t8 = cf4(P, cost8, OXM_F4_HB_T7);
		double energy = F1 * f4t1 * f4t2 * f4t3 * f4t4 * f4t7 * f4t8;
		add_energy(A, OXO_HB, ip, iq, energy);
		if(energy != 0.) {
			tp = V(0, 0, 0);
			tq = V(0, 0, 0);
			double F1D = hb_multi * f1D(P, rhydromod, OXM_F1_HB, q->type, p->type);
			double d1 = cf4D(P, cost1, OXM_F4_HB_T1), d2 = cf4D(P, cost2, OXM_F4_HB_T2), d3 = -cf4D(P, cost3, OXM_F4_HB_T2);
			double d4 = -cf4D(P, cost4, OXM_F4_HB_T4), d7 = cf4D(P, cost7, OXM_F4_HB_T7), d8 = -cf4D(P, cost8, OXM_F4_HB_T7);
			force = mul(neg(rhydrodir), F1D * f4t1 * f4t2 * f4t3 * f4t4 * f4t7 * f4t8);
			vec dir = cross(a3, b3);
			double tm = -F1 * f4t1 * f4t2 * f4t3 * d4 * f4t7 * f4t8;
			tp = sub(tp, mul(dir, tm));
			tq = add(tq, mul(dir, tm));
			dir = cross(a1, b1);
			tm = -F1 * d1 * f4t2 * f4t3 * f4t4 * f4t7 * f4t8;
			tp = sub(tp, mul(dir, tm));
			tq = add(tq, mul(dir, tm));
			double fact = F1 * f4t1 * d2 * f4t3 * f4t4 * f4t7 * f4t8;
			force = add(force, mul(add(b1, mul(rhydrodir, cost2)), fact / rhydromod));
			tq = add(tq, mul(neg(cross(rhydrodir, b1)), fact));
			force = add(force, mul(sub(a1, mul(rhydrodir, cost3)), F1 * f4t1 * f4t2 * d3 * f4t4 * f4t7 * f4t8 / rhydromod));
			tm = -F1 * f4t1 * f4t2 * d3 * f4t4 * f4t7 * f4t8;
			tp = add(tp, mul(cross(rhydrodir, a1), tm));
			force = add(force, mul(add(b3, mul(rhydrodir, cost7)), F1 * f4t1 * f4t2 * f4t3 * f4t4 * d7 * f4t8 / rhydromod));
			tm = -F1 * f4t1 * f4t2 * f4t3 * f4t4 * d7 * f4t8;
			tq = add(tq, mul(cross(rhydrodir, b3), tm));
			force = add(force, mul(sub(a3, mul(rhydrodir, cost8)), F1 * f4t1 * f4t2 * f4t3 * f4t4 * f4t7 * d8 / rhydromod));
			tm = -F1 * f4t1 * f4t2 * f4t3 * f4t4 * f4t7 * d8;
			tp = add(tp, mul(cross(rhydrodir, a3), tm));
			add_force(A, ip, neg(force));
			add_force(A, iq, force);
			tp = sub(tp, cross(p->base, force));
			tq = add(tq, cross(q->base, force));
			add_torque(A, ip, tp);
			add_torque(A, iq, tq);
		}
	}

	/* cross stacking */
	vec rcs = rhydro;
	double rcsmod = rhydromod;
	if(OXM_CRST_RCLOW < rcsmod && rcsmod < OXM_CRST_RCHIGH) {
		vec rcsdir = mul(rcs, 1. / rcsmod);
		double cost1 = -dot(a1, b1), cost2 = -dot(b1, rcsdir), cost3 = dot(a1, rcsdir);
		double cost4 = dot(a3, b3), cost7 = -dot(b3, rcsdir), cost8 = dot(a3, rcsdir);
		double F2 = f2(P, rcsmod, OXM_F2_CRST);
		double f4t1 = cf4(P, cost1, OXM_F4_CR_T1), f4t2 = cf4(P, cost2, OXM_F4_CR_T2), f4t3 = cf4(P, cost3, OXM_F4_CR_T2);
		double f4t4 = cf4(P, cost4, OXM_F4_CR_T4) + cf4(P, -cost4, OXM_F4_CR_T4);
		double f4t7 = cf4(P, cost7, OXM_F4_CR_T7) + cf4(P, -cost7, OXM_F4_CR_T7);
		double f4t8 = cf4(P, cost8, OXM_F4_CR_T7) + cf4(P, -cost8, OXM_F4_CR_T7);
		double energy = F2 * f4t1 * f4t2 * f4t3 * f4t4 * f4t7 * f4t8;
		add_energy(A, OXO_CRST, ip, iq, energy);
		if(energy != 0.) {
			tp = V(0, 0, 0);
			tq = V(0, 0, 0);
			double F2D = f2D(P, rcsmod, OXM_F2_CRST);
			double d1 = cf4D(P, cost1, OXM_F4_CR_T1), d2 = cf4D(P, cost2, OXM_F4_CR_T2), d3 = -cf4D(P, cost3, OXM_F4_CR_T2);
			double d4 = -cf4D(P, cost4, OXM_F4_CR_T4) + cf4D(P, -cost4, OXM_F4_CR_T4);
			double d7 = cf4D(P, cost7, OXM_F4_CR_T7) - cf4D(P, -cost7, OXM_F4_CR_T7);
			double d8 = -cf4D(P, cost8, OXM_F4_CR_T7) + cf4D(P, -cost8, OXM_F4_CR_T7);
			force = mul(neg(rcsdir), F2D * f4t1 * f4t2 * f4t3 * f4t4 * f4t7 * f4t8);
			vec dir = cross(a1, b1);
			double tm = -F2 * d1 * f4t2 * f4t3 * f4t4 * f4t7 * f4t8;
			tp = sub(tp, mul(dir, tm));
			tq = add(tq, mul(dir, tm));
			force = add(force, mul(add(b1, mul(rcsdir, cost2)), F2 * f4t1 * d2 * f4t3 * f4t4 * f4t7 * f4t8 / rcsmod));
			tm = -F2 * f4t1 * d2 * f4t3 * f4t4 * f4t7 * f4t8;
			tq = add(tq, mul(cross(rcsdir, b1), tm));
			force = add(force, mul(sub(a1, mul(rcsdir, cost3)), F2 * f4t1 * f4t2 * d3 * f4t4 * f4t7 * f4t8 / rcsmod));
			tm = -F2 * f4t1 * f4t2 * d3 * f4t4 * f4t7 * f4t8;
			tp = add(tp, mul(cross(rcsdir, a1), tm));
			dir = cross(a3, b3);
			tm = -F2 * f4t1 * f4t2 * f4t3 * d4 * f4t7 * f4t8;
			tp = sub(tp, mul(dir, tm));
			tq = add(tq, mul(dir, tm));
			force = add(force, mul(add(b3, mul(rcsdir, cost7)), F2 * f4t1 * f4t2 * f4t3 * f4t4 * d7 * f4t8 / rcsmod));
			tm = -F2 * f4t1 * f4t2 * f4t3 * f4t4 * d7 * f4t8;
			tq = add(tq, mul(cross(rcsdir, b3), tm));
			force = add(force, mul(sub(a3, mul(rcsdir, cost8)), F2 * f4t1 * f4t2 * f4t3 * f4t4 * f4t7 * d8 / rcsmod));
			tm = -F2 * f4t1 * f4t2 * f4t3 * f4t4 * f4t7 * d8;
			tp = add(tp, mul(cross(rcsdir, a3), tm));
			add_force(A, ip, neg(force));
			add_force(A, iq, force);
			tp = sub(tp, cross(p->base, force));
			tq = add(tq, cross(q->base, force));
			add_torque(A, ip, tp);
			add_torque(A, iq, tq);
		}
	}

	/* coaxial stacking (oxDNA2 form, no phi3 term) */
	vec rstack = add(r, sub(q->stack, p->stack));
	double rstackmod = mod(rstack);
	if(OXM_CXST_RCLOW < rstackmod && rstackmod < OXM_CXST_RCHIGH) {
		vec rstackdir = mul(rstack, 1. / rstackmod);
		double cost1 = -dot(a1, b1), cost4 = dot(a3, b3), cost5 = dot(a3, rstackdir), cost6 = -dot(b3, rstackdir);
		double F2 = f2(P, rstackmod, OXM_F2_CXST);
		double f4t1 = cf4(P, cost1, OXM_F4_CX_T1), f4t4 = cf4(P, cost4, OXM_F4_CX_T4);
		double f4t5 = cf4(P, cost5, OXM_F4_CX_T5) + cf4(P, -cost5, OXM_F4_CX_T5);
		double f4t6 = cf4(P, cost6, OXM_F4_CX_T5) + cf4(P, -cost6, OXM_F4_CX_T5);
		double energy = F2 * f4t1 * f4t4 * f4t5 * f4t6;
		add_energy(A, OXO_CXST, ip, iq, energy);
		if(energy != 0.) {
			tp = V(0, 0, 0);
			tq = V(0, 0, 0);
			double F2D = f2D(P, rstackmod, OXM_F2_CXST);
			double d1 = cf4D(P, cost1, OXM_F4_CX_T1), d4 = -cf4D(P, cost4, OXM_F4_CX_T4);
			double d5 = -cf4D(P, cost5, OXM_F4_CX_T5) + cf4D(P, -cost5, OXM_F4_CX_T5);
			double d6 = cf4D(P, cost6, OXM_F4_CX_T5) - cf4D(P, -cost6, OXM_F4_CX_T5);
			force = mul(neg(rstackdir), F2D * f4t1 * f4t4 * f4t5 * f4t6);
			vec dir = cross(a1, b1);
			double tm = -F2 * d1 * f4t4 * f4t5 * f4t6;
			tp = sub(tp, mul(dir, tm));
			tq = add(tq, mul(dir, tm));
			dir = cross(a3, b3);
			tm = -F2 * f4t1 * d4 * f4t5 * f4t6;
			tp = sub(tp, mul(dir, tm));
			tq = add(tq, mul(dir, tm));
			double fact = F2 * f4t1 * f4t4 * d5 * f4t6;
			force = add(force, mul(mul(sub(a3, mul(rstackdir, cost5)), fact), 1. / rstackmod));
			tp = sub(tp, mul(cross(rstackdir, a3), fact));
			fact = F2 * f4t1 * f4t4 * f4t5 * d6;
			force = add(force, mul(add(b3, mul(rstackdir, cost6)), fact / rstackmod));
			tq = add(tq, mul(neg(cross(rstackdir, b3)), fact));
			add_force(A, ip, neg(force));
			add_force(A, iq, force);
			tp = sub(tp, cross(p->stack, force));
			tq = add(tq, cross(q->stack, force));
			add_torque(A, ip, tp);
			add_torque(A, iq, tq);
		}
	}

	/* Debye-Hueckel */
	double cut_factor = 1.0f;
	if(P->dh_half_charged_ends && (p->n3 < 0 || p->n5 < 0)) cut_factor *= 0.5f;
	if(P->dh_half_charged_ends && (q->n3 < 0 || q->n5 < 0)) cut_factor *= 0.5f;
	vec rback = add(r, sub(q->back, p->back));
	double rbackmod = mod(rback);
	if(rbackmod < P->dh_rc) {
		double energy;
		vec rbackdir = mul(rback, 1. / rbackmod);
		if(rbackmod < P->dh_rhigh) {
			energy = exp(rbackmod * P->dh_minus_kappa) * (P->dh_prefactor / rbackmod);
			force = mul(rbackdir, -1.0f * (P->dh_prefactor * exp(P->dh_minus_kappa * rbackmod)) *
					(P->dh_minus_kappa / rbackmod - 1.0f / SQR(rbackmod)));
		}
		else {
			energy = P->dh_b * SQR(rbackmod - P->dh_rc);
			force = mul(neg(rbackdir), 2.0f * P->dh_b * (rbackmod - P->dh_rc));
		}
		energy *= cut_factor;
		force = mul(force, cut_factor);
		add_energy(A, OXO_DH, ip, iq, energy);
		add_force(A, ip, neg(force));
		add_force(A, iq, force);
		add_torque(A, ip, neg(cross(p->back, force)));
		add_torque(A, iq, cross(q->back, force));
	}
}

/* ---------------------------------------------------------------- pair search (FP64) */

static inline double min_image1(double d, double L) { return d - rint(d / L) * L; }

long oxo_pairs_within(int N, const double *pos, double L, double rc, int *pairs, long max_pairs) {
	long count = 0;
	const double rc2 = rc * rc;
	int n = (int) floor(L / rc);
	if(n < 3) {
		for(int i = 0; i < N; i++) {
			for(int j = 0; j < i; j++) {
				double dx = min_image1(pos[3 * j] - pos[3 * i], L), dy = min_image1(pos[3 * j + 1] - pos[3 * i + 1], L),
						dz = min_image1(pos[3 * j + 2] - pos[3 * i + 2], L);
				if(dx * dx + dy * dy + dz * dz < rc2) {
					if(count < max_pairs) {
						pairs[2 * count] = i;
						pairs[2 * count + 1] = j;
					}
					count++;
				}
			}
		}
		return count;
	}
	const long nc = (long) n * n * n;
	int *head = (int *) malloc(sizeof(int) * nc), *next = (int *) malloc(sizeof(int) * N), *cid = (int *) malloc(sizeof(int) * 3 * N);
	for(long c = 0; c < nc; c++) head[c] = -1;
	for(int i = 0; i < N; i++) {
		int c3[3];
		for(int d = 0; d < 3; d++) {
			double s = pos[3 * i + d] / L;
			int k = (int) ((s - floor(s)) * n);
			if(k >= n) k = n - 1;
			if(k < 0) k = 0;
			c3[d] = k;
			cid[3 * i + d] = k;
		}
		long c = ((long) c3[2] * n + c3[1]) * n + c3[0];
		next[i] = head[c];
		head[c] = i;
	}
	for(int i = 0; i < N; i++) {
		for(int dz = -1; dz <= 1; dz++)
			for(int dy = -1; dy <= 1; dy++)
				for(int dx = -1; dx <= 1; dx++) {
					int cx = (cid[3 * i] + dx + n) % n, cy = (cid[3 * i + 1] + dy + n) % n, cz = (cid[3 * i + 2] + dz + n) % n;
					for(int j = head[((long) cz * n + cy) * n + cx]; j >= 0; j = next[j]) {
						if(j >= i) continue;
						double ddx = min_image1(pos[3 * j] - pos[3 * i], L), ddy = min_image1(pos[3 * j + 1] - pos[3 * i + 1], L),
								ddz = min_image1(pos[3 * j + 2] - pos[3 * i + 2], L);
						if(ddx * ddx + ddy * ddy + ddz * ddz < rc2) {
							if(count < max_pairs) {
								pairs[2 * count] = i;
								pairs[2 * count + 1] = j;
							}
							count++;
						}
					}
				}
	}
	free(head);
	free(next);
	free(cid);
	return count;
}

/* ---------------------------------------------------------------- FFS order parameters */

/* The per-pair order-parameter quantities of the reference's FFS backend, as its CUDA kernels
 * define them (src/CUDA/Interactions/CUDA_DNA.cuh:910-1067): for the pair (op1[k], op2[k]), with
 * the centre separation taken at its minimum image and the base sites at POS_BASE a1,
 *   mode 0 (hb_op_precalc):      the hydrogen-bonding energy f1 f4(t1) f4(t2) f4(t3) f4(t4)
 *                                f4(t7) f4(t8) of the pair (0 unless the bases are complementary
 *                                and the base-base distance is inside (RCLOW, RCHIGH)); unlike
 *                                the force field's own term it carries no hb_multiplier;
 *   mode 1 (near_hb_op_precalc): 1 if at least six of the seven factors are "on" (f1 < 0, each
 *                                f4 > 0), else 0;
 *   mode 2 (dist_op_precalc):    the base-base distance |r + b1 POS_BASE - a1 POS_BASE|.
 * FP64; out[k] receives the value. */
void oxo_order_params(const oxo_params *P, const double *pos, const double *a1v, const double *a3v, const int *type,
		const int *btype, double L, const int *op1, const int *op2, int n, int mode, double *out) {
	for(int k = 0; k < n; k++) {
		const int i = op1[k], j = op2[k];
		vec r = sub(load(pos, j), load(pos, i));
		r = V(min_image1(r.x, L), min_image1(r.y, L), min_image1(r.z, L));
		const vec a1 = load(a1v, i), a3 = load(a3v, i), b1 = load(a1v, j), b3 = load(a3v, j);
		const vec rb = add(r, sub(mul(b1, (double) OXM_POS_BASE), mul(a1, (double) OXM_POS_BASE)));
		const double r2 = dot(rb, rb);
		if(mode == 2) {
			out[k] = sqrt(r2);
			continue;
		}
		double e = 0., near = 0.;
		if(btype[i] + btype[j] == 3 && SQR(OXM_HYDR_RCLOW) < r2 && r2 < SQR(OXM_HYDR_RCHIGH)) {
			const double rmod = sqrt(r2);
			const vec rd = mul(rb, 1. / rmod);
			const double F1 = f1(P, rmod, OXM_F1_HB, type[i], type[j]);
			const double g[6] = {cf4(P, -dot(a1, b1), OXM_F4_HB_T1), cf4(P, -dot(b1, rd), OXM_F4_HB_T2),
					cf4(P, dot(a1, rd), OXM_F4_HB_T2), cf4(P, dot(a3, b3), OXM_F4_HB_T4), cf4(P, -dot(rd, b3), OXM_F4_HB_T7),
					cf4(P, dot(rd, a3), OXM_F4_HB_T7)};
			e = F1;
			int on = F1 < 0;
			for(int m = 0; m < 6; m++) {
				e *= g[m];
				on += g[m] > 0;
			}
			near = on >= 6;
		}
		out[k] = mode == 0 ? e : near;
	}
}

/* ---------------------------------------------------------------- full force evaluation */

int oxo_forces(const oxo_params *P, int N, const double *pos, const double *a1, const double *a2, const double *a3,
		const int *n3, const int *n5, const int *type, const int *btype, double L, const int *pairs, int npairs,
		double *F, double *T, double *E_split, double *E_part, int nthreads) {
	nuc *nucs = (nuc *) malloc(sizeof(nuc) * (N > 0 ? N : 1));
	for(int i = 0; i < N; i++) {
		make_nuc(&nucs[i], pos, a1, a2, a3, i);
		nucs[i].type = type[i];
		nucs[i].btype = btype[i];
		nucs[i].n3 = n3[i];
		nucs[i].n5 = n5[i];
	}
	int *own_pairs = NULL;
	long np = npairs;
	if(npairs < 0) {
		long cap = 64L * N + 1024;
		own_pairs = (int *) malloc(sizeof(int) * 2 * cap);
		np = oxo_pairs_within(N, pos, L, P->rcut, own_pairs, cap);
		if(np > cap) {
			free(own_pairs);
			own_pairs = (int *) malloc(sizeof(int) * 2 * np);
			oxo_pairs_within(N, pos, L, P->rcut, own_pairs, np);
		}
		pairs = own_pairs;
	}

	int nt = 1;
#ifdef _OPENMP
	nt = nthreads > 0 ? nthreads : 1;
#endif
	/* per-thread accumulators keep the half-pair loop free of races */
	double *buf = (double *) calloc((size_t) nt * (7 * (size_t) N + OXO_NTERMS), sizeof(double));
	int err = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt) reduction(min : err)
#endif
	{
		int tid = 0;
#ifdef _OPENMP
		tid = omp_get_thread_num();
#endif
		double *base = buf + (size_t) tid * (7 * (size_t) N + OXO_NTERMS);
		acc A = {base, base + 3 * (size_t) N, base + 6 * (size_t) N, base + 6 * (size_t) N + OXO_NTERMS, 0};
		/* bonded pairs, each once, from the particle whose 3' neighbour is the other */
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
		for(int i = 0; i < N; i++) {
			int q = n3[i];
			if(q >= 0) {
				vec r = sub(nucs[q].pos, nucs[i].pos);
				bonded_pair(P, &nucs[i], &nucs[q], i, q, r, &A);
			}
		}
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
		for(long k = 0; k < np; k++) {
			int i = pairs[2 * k], j = pairs[2 * k + 1];
			int hi = i > j ? i : j, lo = i > j ? j : i;
			vec d = sub(nucs[lo].pos, nucs[hi].pos);
			vec r = V(min_image1(d.x, L), min_image1(d.y, L), min_image1(d.z, L));
			nonbonded_pair(P, &nucs[hi], &nucs[lo], hi, lo, r, &A);
		}
		err = A.err;
	}
	for(int i = 0; i < 3 * N; i++) F[i] = T[i] = 0.;
	for(int t = 0; t < OXO_NTERMS; t++) E_split[t] = 0.;
	for(int i = 0; i < N; i++) E_part[i] = 0.;
	for(int t = 0; t < nt; t++) {
		double *base = buf + (size_t) t * (7 * (size_t) N + OXO_NTERMS);
		for(int i = 0; i < 3 * N; i++) {
			F[i] += base[i];
			T[i] += base[3 * (size_t) N + i];
		}
		for(int k = 0; k < OXO_NTERMS; k++) E_split[k] += base[6 * (size_t) N + k];
		for(int i = 0; i < N; i++) E_part[i] += base[6 * (size_t) N + OXO_NTERMS + i];
	}
	/* lab -> body frame: T_body = (a1.T, a2.T, a3.T) */
	for(int i = 0; i < N; i++) {
		vec t = load(T, i);
		T[3 * i] = dot(nucs[i].a1, t);
		T[3 * i + 1] = dot(nucs[i].a2, t);
		T[3 * i + 2] = dot(nucs[i].a3, t);
	}
	free(buf);
	free(nucs);
	free(own_pairs);
	return err;
}

/* ---------------------------------------------------------------- FP32 Verlet list restatement */

/* CUDASimpleVerletList::_compute_N_cells_side (src/CUDA/Lists/CUDASimpleVerletList.cu:96-110);
 * the min-3 clamp is applied after the density cap (as src/Lists/Cells.cpp:50-60 does) */
static void cells_side(int N, float L, float rverlet, int auto_opt, int *n_side) {
	float V3 = L * L * L;
	float max_factor = (float) pow(2. * N / V3, 1. / 3.);
	float min_cell = sqrtf(rverlet * rverlet);
	int n = (int) (floor((double) L / (double) min_cell) + 0.1);
	if(auto_opt && n > ceilf(max_factor * L)) n = (int) ceilf(max_factor * L);
	if(n < 3) n = 3;
	*n_side = n;
}

/* CUDABox::compute_cell_index (src/CUDA/cuda_utils/CUDABox.h:62-68) with IEEE division */
static inline int cell_coord(float x, float L, int n) {
	float s = x / L;
	return (int) (((s - floorf(s)) * (1.f - FLT_EPSILON)) * (float) n);
}

/* CUDABox::minimum_image + sqr_minimum_image (CUDABox.h:42-60), with the fused multiply-adds the
 * GPU list kernel issues explicitly */
static inline float sqr_min_image_f32(const float *pi, const float *pj, float L) {
	float dx = pj[0] - pi[0], dy = pj[1] - pi[1], dz = pj[2] - pi[2];
	dx = fmaf(-rintf(dx / L), L, dx);
	dy = fmaf(-rintf(dy / L), L, dy);
	dz = fmaf(-rintf(dz / L), L, dz);
	return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}

static int cmp_int(const void *a, const void *b) { return (*(const int *) a) - (*(const int *) b); }

int oxo_verlet_f32(int N, const float *pos4, float L, float rverlet, const int *n3, const int *n5, int auto_opt,
		int *n_cells_side, int *cell, int *nnb, int *nb, int max_nb) {
	int n;
	cells_side(N, L, rverlet, auto_opt, &n);
	*n_cells_side = n;
	const float rv2 = rverlet * rverlet;
	long nc = (long) n * n * n;
	int *head = (int *) malloc(sizeof(int) * nc), *next = (int *) malloc(sizeof(int) * (N > 0 ? N : 1));
	for(long c = 0; c < nc; c++) head[c] = -1;
	for(int i = N - 1; i >= 0; i--) {
		int cx = cell_coord(pos4[4 * i], L, n), cy = cell_coord(pos4[4 * i + 1], L, n), cz = cell_coord(pos4[4 * i + 2], L, n);
		long c = ((long) cz * n + cy) * n + cx;
		cell[i] = (int) c;
		next[i] = head[c];
		head[c] = i;
	}
	int overflow = 0;
	for(int i = 0; i < N; i++) {
		int cx = cell_coord(pos4[4 * i], L, n), cy = cell_coord(pos4[4 * i + 1], L, n), cz = cell_coord(pos4[4 * i + 2], L, n);
		int cnt = 0;
		for(int dz = -1; dz <= 1; dz++)
			for(int dy = -1; dy <= 1; dy++)
				for(int dx = -1; dx <= 1; dx++) {
					long c = (((long) ((cz + dz + n) % n)) * n + (cy + dy + n) % n) * n + (cx + dx + n) % n;
					for(int j = head[c]; j >= 0; j = next[j]) {
						if(j == i || n3[i] == j || n5[i] == j) continue;
						if(sqr_min_image_f32(pos4 + 4 * i, pos4 + 4 * j, L) < rv2) {
							if(cnt < max_nb) nb[(long) i * max_nb + cnt] = j;
							cnt++;
						}
					}
				}
		if(cnt > max_nb) overflow = 1;
		nnb[i] = cnt;
		qsort(nb + (long) i * max_nb, cnt < max_nb ? cnt : max_nb, sizeof(int), cmp_int);
	}
	free(head);
	free(next);
	return overflow ? -1 : 0;
}

/* ---------------------------------------------------------------- random numbers */

/* Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC11 2011): 10 rounds of the published round
 * function with the published multipliers and Weyl key increments */
void oxo_philox(unsigned int k0, unsigned int k1, unsigned int c0, unsigned int c1, unsigned int c2, unsigned int c3,
		unsigned int out[4]) {
	const unsigned int M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
	for(int r = 0; r < 10; r++) {
		unsigned long long p0 = (unsigned long long) M0 * c0, p1 = (unsigned long long) M1 * c2;
		unsigned int hi0 = (unsigned int) (p0 >> 32), lo0 = (unsigned int) p0;
		unsigned int hi1 = (unsigned int) (p1 >> 32), lo1 = (unsigned int) p1;
		unsigned int n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
		c0 = n0;
		c1 = n1;
		c2 = n2;
		c3 = n3;
		k0 += W0;
		k1 += W1;
	}
	out[0] = c0;
	out[1] = c1;
	out[2] = c2;
	out[3] = c3;
}

/* uniform in (0, 1] */
static inline double u01(unsigned int x) { return ((double) x + 1.0) * (1.0 / 4294967296.0); }

static inline void box_muller(unsigned int ua, unsigned int ub, double *g0, double *g1) {
	double r = sqrt(-2.0 * log(u01(ua)));
	double phi = 6.283185307179586 * u01(ub);
	*g0 = r * cos(phi);
	*g1 = r * sin(phi);
}

/* stream tags (third counter word); the step index fills the first two words */
#define OXO_RNG_BROWNIAN 0x42524f57u
#define OXO_RNG_BUSSI 0x42555353u

/* Brownian draws of particle i at step s: two Philox blocks (8 uniforms): test_t, test_r, six
 * normals (v.x v.y v.z L.x L.y L.z) */
static void brownian_draws(unsigned long long seed, long long s, int i, double *ut, double *ur, double g[6]) {
	unsigned int o0[4], o1[4];
	unsigned int k0 = (unsigned int) seed, k1 = (unsigned int) (seed >> 32);
	unsigned int s0 = (unsigned int) s, s1 = (unsigned int) ((unsigned long long) s >> 32);
	oxo_philox(k0, k1, s0, s1, OXO_RNG_BROWNIAN, (unsigned int) (2 * i), o0);
	oxo_philox(k0, k1, s0, s1, OXO_RNG_BROWNIAN, (unsigned int) (2 * i + 1), o1);
	*ut = u01(o0[0]);
	*ur = u01(o0[1]);
	box_muller(o0[2], o0[3], &g[0], &g[1]);
	box_muller(o1[0], o1[1], &g[2], &g[3]);
	box_muller(o1[2], o1[3], &g[4], &g[5]);
}

/* sequential uniform stream for the Bussi kinetic-energy update at step s, channel c */
typedef struct {
	unsigned int k0, k1, s0, s1, c, blk, idx;
	unsigned int buf[4];
} oxo_stream;

static void stream_init(oxo_stream *st, unsigned long long seed, long long s, unsigned int channel) {
	st->k0 = (unsigned int) seed;
	st->k1 = (unsigned int) (seed >> 32);
	st->s0 = (unsigned int) s;
	st->s1 = (unsigned int) ((unsigned long long) s >> 32);
	st->c = OXO_RNG_BUSSI ^ channel;
	st->blk = 0;
	st->idx = 4;
}

static double stream_u01(oxo_stream *st) {
	if(st->idx == 4) {
		oxo_philox(st->k0, st->k1, st->s0, st->s1, st->c, st->blk++, st->buf);
		st->idx = 0;
	}
	return u01(st->buf[st->idx++]);
}

static double stream_gauss(oxo_stream *st) {
	double u1 = stream_u01(st), u2 = stream_u01(st);
	return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

/* gamma deviate of integer order ia (Numerical Recipes gamdev, the algorithm the reference's
 * BussiThermostat::_gamdev uses, src/Backends/Thermostats/BussiThermostat.cpp:130-155) */
static double gamdev(oxo_stream *st, int ia) {
	double x;
	if(ia < 6) {
		x = 1.0;
		for(int j = 1; j <= ia; j++) x *= stream_u01(st);
		return -log(x);
	}
	double am = ia - 1, s = sqrt(2.0 * am + 1.0), e, y, v1, v2;
	do {
		do {
			do {
				v1 = stream_u01(st);
				v2 = 2.0 * stream_u01(st) - 1.0;
			} while(v1 * v1 + v2 * v2 > 1.0);
			y = v2 / v1;
			x = s * y + am;
		} while(x <= 0.0);
		e = (1.0 + y * y) * exp(am * log(x / am) - s * y);
	} while(stream_u01(st) > e);
	return x;
}

/* sum of nn squared normals (BussiThermostat::_sum_noises, :105-128) */
static double sum_noises(oxo_stream *st, int nn) {
	if(nn == 0) return 0.0;
	if(nn == 1) {
		double rr = stream_gauss(st);
		return rr * rr;
	}
	if(nn % 2 == 0) return 2.0 * gamdev(st, nn / 2);
	double rr = stream_gauss(st);
	return 2.0 * gamdev(st, (nn - 1) / 2) + rr * rr;
}

/* BussiThermostat::_update_K (:44-52) */
static void bussi_update_K(oxo_stream *st, double *K, int dof, double T, double c) {
	double K_target = 0.5 * dof * T;
	double rr = stream_gauss(st);
	double dK = (1.0 - c) * (K_target * (sum_noises(st, dof - 1) + rr * rr) / dof - *K) +
			2.0 * rr * sqrt(*K * K_target / dof * (1.0 - c) * c);
	*K += dK;
}

/* ---------------------------------------------------------------- integrator */

void oxo_quat_to_frame(const double *q, double *a1, double *a2, double *a3) {
	double x = q[0], y = q[1], z = q[2], w = q[3];
	double sqx = x * x, sqy = y * y, sqz = z * z, sqw = w * w;
	a1[0] = sqx - sqy - sqz + sqw;
	a1[1] = 2 * (x * y + z * w);
	a1[2] = 2 * (x * z - y * w);
	a2[0] = 2 * (x * y - z * w);
	a2[1] = -sqx + sqy - sqz + sqw;
	a2[2] = 2 * (y * z + x * w);
	a3[0] = 2 * (x * z + y * w);
	a3[1] = 2 * (y * z - x * w);
	a3[2] = -sqx - sqy + sqz + sqw;
}

static void compute_all(const oxo_params *P, int N, const double *pos, const double *quat, const int *n3, const int *n5,
		const int *type, const int *btype, double L, double *F, double *T, double *E_split, double *a1, double *a2, double *a3,
		double *E_part, int nthreads, int *err) {
	for(int i = 0; i < N; i++) oxo_quat_to_frame(quat + 4 * i, a1 + 3 * i, a2 + 3 * i, a3 + 3 * i);
	int e = oxo_forces(P, N, pos, a1, a2, a3, n3, n5, type, btype, L, NULL, -1, F, T, E_split, E_part, nthreads);
	if(e) *err = e;
}

int oxo_md_run(const oxo_params *P, oxo_md *md, int N, double *pos, double *quat, double *vel, double *Lm,
		const int *n3, const int *n5, const int *type, const int *btype, double L, double *F, double *T,
		long long step0, int nsteps, double *E_split, int nthreads) {
	const double dt = md->dt;
	double *a1 = (double *) malloc(sizeof(double) * 3 * N), *a2 = (double *) malloc(sizeof(double) * 3 * N),
			*a3 = (double *) malloc(sizeof(double) * 3 * N), *Ep = (double *) malloc(sizeof(double) * N);
	int err = 0;
	for(int k = 0; k < nsteps; k++) {
		long long s = step0 + k;
		/* first step: CUDA_mixed.cuh:23-69 in FP64 */
		for(int i = 0; i < N; i++) {
			for(int d = 0; d < 3; d++) {
				vel[3 * i + d] += F[3 * i + d] * dt * 0.5;
				pos[3 * i + d] += vel[3 * i + d] * dt;
				Lm[3 * i + d] += T[3 * i + d] * dt * 0.5;
			}
			double lx = Lm[3 * i], ly = Lm[3 * i + 1], lz = Lm[3 * i + 2];
			double norm = sqrt(lx * lx + ly * ly + lz * lz);
			if(norm > 0.) {
				double ux = lx / norm, uy = ly / norm, uz = lz / norm;
				double half = 0.5 * dt * norm, sh = sin(half), ch = cos(half);
				double rx = ux * sh, ry = uy * sh, rz = uz * sh, rw = ch;
				double *q = quat + 4 * i;
				double qx = q[0], qy = q[1], qz = q[2], qw = q[3];
				/* q <- q * r (CUDA_lr_common.cuh:63-71 quat_multiply) */
				q[3] = qw * rw - qx * rx - qy * ry - qz * rz;
				q[0] = qw * rx + qx * rw + qy * rz - qz * ry;
				q[1] = qw * ry - qx * rz + qy * rw + qz * rx;
				q[2] = qw * rz + qx * ry - qy * rx + qz * rw;
			}
		}
		compute_all(P, N, pos, quat, n3, n5, type, btype, L, F, T, E_split, a1, a2, a3, Ep, nthreads, &err);
		/* second step: CUDA_mixed.cuh:71-93 */
		for(int i = 0; i < 3 * N; i++) {
			vel[i] += F[i] * dt * 0.5;
			Lm[i] += T[i] * dt * 0.5;
		}
		/* thermostat (MD_CUDABackend::_thermalize, applied when step % newtonian_steps == 0) */
		if(md->thermostat != 0 && md->newtonian_steps > 0 && s % md->newtonian_steps == 0) {
			const double resc = sqrt(P->T);
			if(md->thermostat == 1) {
				/* CUDABrownianThermostat.cu:15-51 / BrownianThermostat::apply */
				for(int i = 0; i < N; i++) {
					double ut, ur, g[6];
					brownian_draws(md->seed, s, i, &ut, &ur, g);
					if(ut < md->pt) {
						vel[3 * i] = g[0] * resc;
						vel[3 * i + 1] = g[1] * resc;
						vel[3 * i + 2] = g[2] * resc;
					}
					if(ur < md->pr) {
						Lm[3 * i] = g[3] * resc;
						Lm[3 * i + 1] = g[4] * resc;
						Lm[3 * i + 2] = g[5] * resc;
					}
				}
			}
			else if(md->thermostat == 2) {
				/* CUDABussiThermostat::apply_cuda (CUDABussiThermostat.cu:97-122) in FP64 */
				double vc[3] = {0, 0, 0}, Kt = 0, Kr = 0;
				for(int i = 0; i < N; i++)
					for(int d = 0; d < 3; d++) vc[d] += vel[3 * i + d];
				for(int d = 0; d < 3; d++) vc[d] /= N;
				for(int i = 0; i < N; i++) {
					for(int d = 0; d < 3; d++) {
						double vr = vel[3 * i + d] - vc[d];
						Kt += 0.5 * vr * vr;
						Kr += 0.5 * Lm[3 * i + d] * Lm[3 * i + d];
					}
				}
				double c = exp(-md->newtonian_steps / md->bussi_tau);
				oxo_stream st;
				stream_init(&st, md->seed, s, 0u);
				bussi_update_K(&st, &md->bussi_K_t, 3 * (N - 1), P->T, c);
				stream_init(&st, md->seed, s, 1u);
				bussi_update_K(&st, &md->bussi_K_r, 3 * N, P->T, c);
				double ft = sqrt(md->bussi_K_t / Kt), fr = sqrt(md->bussi_K_r / Kr);
				for(int i = 0; i < N; i++) {
					for(int d = 0; d < 3; d++) {
						vel[3 * i + d] = (vel[3 * i + d] - vc[d]) * ft + vc[d];
						Lm[3 * i + d] *= fr;
					}
				}
			}
		}
	}
	free(a1);
	free(a2);
	free(a3);
	free(Ep);
	return err;
}
