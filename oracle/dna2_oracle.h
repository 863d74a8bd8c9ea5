/*
 * ORACLE (test infrastructure only).  CPU FP64 restatement of the reference oxDNA2
 * physics on the GPU MD hot path: the DNA2_nomesh force field, the cell-binned Verlet
 * pair search of the CUDA list, and the velocity-Verlet integrator with its thermostats.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library,
 * and only as the checker.  The product (oxdna_gb300/) never links, loads or calls it.
 * Parity pin: tests/test_oracle_pin.py checks it against the reference's own golden split
 * energies (test/DNA/FORCE_FIELD/{AVG_SEQ,SEQ_DEP}/reference.dat) and against full-precision
 * forces, torques and energies printed by the reference CPU code built from its sources
 * (oracle/ref/, fixtures in tests/golden/).
 */
#ifndef OXGB_DNA2_ORACLE_H
#define OXGB_DNA2_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* user-facing settings, the same keys the reference reads
 * (src/Interactions/DNAInteraction.cpp:216-298, src/Interactions/DNA2Interaction.cpp:62-99) */
typedef struct oxo_settings {
	double T;                 /* temperature, simulation units (1 = 3000 K) */
	double salt;              /* salt_concentration, molar */
	int average;              /* use_average_seq */
	double seq_stck[4][4];    /* STCK_X_Y of the sequence-dependence file (X, Y in A G C T order) */
	double seq_stck_fact_eps; /* STCK_FACT_EPS */
	double seq_hydr_at;       /* HYDR_A_T */
	double seq_hydr_gc;       /* HYDR_G_C */
	double hb_multiplier;     /* hb_multiplier (btype >= 300 pairs) */
	int dh_half_charged_ends; /* dh_half_charged_ends */
	double dh_lambda;         /* dh_lambda */
	double dh_strength;       /* dh_strength */
	int use_mbf;              /* max_backbone_force given */
	double mbf_fmax;          /* max_backbone_force */
	double mbf_finf;          /* max_backbone_force_far */
} oxo_settings;

/* derived parameter tables, as DNAInteraction::init + DNA2Interaction::init leave them */
typedef struct oxo_params {
	double T;
	double f1_eps[2][5][5], f1_shift[2][5][5];
	double f1_a[2], f1_rc[2], f1_r0[2], f1_blow[2], f1_bhigh[2], f1_rlow[2], f1_rhigh[2], f1_rclow[2], f1_rchigh[2];
	double f2_k[2], f2_rc[2], f2_r0[2], f2_blow[2], f2_rlow[2], f2_rclow[2], f2_bhigh[2], f2_rhigh[2], f2_rchigh[2];
	double f4_a[13], f4_b[13], f4_t0[13], f4_ts[13], f4_tc[13], f4_sa, f4_sb;
	double f5_a[4], f5_b[4], f5_xc[4], f5_xs[4];
	double hb_multiplier;
	int dh_half_charged_ends;
	double dh_prefactor, dh_rhigh, dh_rc, dh_b, dh_minus_kappa, dh_lambda;
	int use_mbf;
	double mbf_fmax, mbf_finf, mbf_xmax;
	double fene_r0;
	double rcut;              /* interaction cutoff (centre-centre) */
} oxo_params;

/* the 8 energy terms, in the reference's split order */
enum { OXO_FENE = 0, OXO_BEXC, OXO_STCK, OXO_NEXC, OXO_HB, OXO_CRST, OXO_CXST, OXO_DH, OXO_NTERMS };

int oxo_params_init(const oxo_settings *s, oxo_params *p);

/*
 * One full force evaluation.  Positions pos[3N]; body frames a1, a2, a3 [3N] (lab
 * components of the body axes); n3, n5 bonded neighbours (-1 if none); type (0..4 base
 * code), btype (base type used for pairing).  Cubic periodic box of side L.
 * Non-bonded pairs: if npairs >= 0, the unordered pairs listed in pairs[2*npairs];
 * if npairs < 0 the oracle finds every pair within rcut itself (cell search).
 * Outputs: F[3N] lab-frame forces, T[3N] body-frame torques, E_split[8] system energy per
 * term, E_part[N] per-particle energy with every pair term counted on both particles.
 * Returns 0, or a negative code for an error (FENE bond outside its range: -1).
 */
int oxo_forces(const oxo_params *p, int N, const double *pos, const double *a1, const double *a2, const double *a3,
		const int *n3, const int *n5, const int *type, const int *btype, double L, const int *pairs, int npairs,
		double *F, double *T, double *E_split, double *E_part, int nthreads);

/*
 * Every unordered pair (i > j) whose minimum-image centre distance is below rc, found by
 * an FP64 cell search; bonded pairs included.  Writes at most max_pairs pairs, returns
 * the total count (callers retry with a larger buffer when it exceeds max_pairs).
 */
long oxo_pairs_within(int N, const double *pos, double L, double rc, int *pairs, long max_pairs);

/* FFS order-parameter quantities of pairs (op1[k], op2[k]): mode 0 hydrogen-bonding energy, 1
 * nearly-bonded flag, 2 base-base distance (CUDA_DNA.cuh:910-1067) */
void oxo_order_params(const oxo_params *P, const double *pos, const double *a1, const double *a3, const int *type,
		const int *btype, double L, const int *op1, const int *op2, int n, int mode, double *out);

/*
 * FP32 restatement of the GPU Verlet-list build: cell of every particle and the full
 * neighbour set, with the cell count rules of CUDASimpleVerletList::_compute_N_cells_side
 * (src/CUDA/Lists/CUDASimpleVerletList.cu:96-110) and the fp32 geometry of
 * src/CUDA/cuda_utils/CUDABox.h:42-75 and src/CUDA/Lists/CUDA_simple_verlet.cuh:23-82
 * (IEEE division, explicit fused multiply-adds in the order the GPU kernel uses).
 * pos4[4N] float (x, y, z, unused).  Outputs cell[N], nnb[N], nb[N*max_nb] (row-major,
 * neighbours of i sorted ascending).  Returns 0, or -1 when a row overflows max_nb.
 */
int oxo_verlet_f32(int N, const float *pos4, float L, float rverlet, const int *n3, const int *n5, int auto_opt,
		int *n_cells_side, int *cell, int *nnb, int *nb, int max_nb);

/* ---------------- integrator ---------------- */

/* counter-based Philox-4x32-10 stream: 4 uniforms in (0, 1] per (key, counter) */
void oxo_philox(unsigned int key0, unsigned int key1, unsigned int c0, unsigned int c1, unsigned int c2, unsigned int c3,
		unsigned int out[4]);

typedef struct oxo_md {
	double dt;
	int thermostat;           /* 0 none, 1 brownian ("john"), 2 bussi */
	int newtonian_steps;
	double pt, pr;            /* brownian probabilities */
	double bussi_tau;         /* steps */
	double bussi_K_t, bussi_K_r; /* bussi running kinetic energies (state) */
	unsigned long long seed;
	double verlet_skin;
} oxo_md;

/*
 * nsteps velocity-Verlet steps in FP64, with the step order of MD_CUDABackend::sim_step
 * (src/CUDA/Backends/MD_CUDABackend.cu:567-619): first half kick + drift + rotation, forces,
 * second half kick, thermostat.  The quaternion update is that of
 * src/CUDA/Backends/CUDA_mixed.cuh:8-21 (q <- q * (sin(theta/2) L^, cos(theta/2)),
 * theta = dt |L|, L and torques in the body frame).  State arrays are updated in place:
 * pos[3N], quat[4N] (x, y, z, w), vel[3N], L[3N]; F[3N], T[3N] must hold the forces of
 * the current state on entry and hold those of the final state on exit.  step0 is the
 * index of the first step (thermostat schedule and random stream use it).
 */
int oxo_md_run(const oxo_params *p, oxo_md *md, int N, double *pos, double *quat, double *vel, double *Lmom,
		const int *n3, const int *n5, const int *type, const int *btype, double L, double *F, double *T,
		long long step0, int nsteps, double *E_split, int nthreads);

void oxo_quat_to_frame(const double *q, double *a1, double *a2, double *a3);

#ifdef __cplusplus
}
#endif

#endif
