/*
 * oxgb -- GB300-native oxDNA2 molecular-dynamics hot path, C ABI.
 *
 * One shared library (liboxgb.so) exports three layers, each the replacement for one of the
 * reference's plugin surfaces on the GPU MD path (backend = CUDA, interaction_type = DNA2,
 * CUDA_list = verlet):
 *
 *   oxgb_dna2_*   the interaction: oxDNA2 forces, torques and energies on device buffers in
 *                 the reference's device layout (CUDABaseInteraction,
 *                 src/CUDA/Interactions/CUDABaseInteraction.h:20-64);
 *   oxgb_verlet_* the cell-binned Verlet list (CUDABaseList, src/CUDA/Lists/CUDABaseList.h:25-62);
 *   oxgb_md_*     the MD backend with its integrator and thermostats on host buffers
 *                 (MD_CUDABackend / CUDAMixedBackend, src/CUDA/Backends/MD_CUDABackend.h:29-93,
 *                 and CUDABaseThermostat, src/CUDA/Thermostats/CUDABaseThermostat.h:26-49),
 *                 including batches of independent systems.
 *
 * Conventions: every function returns an oxgb_status (0 = success); oxgb_last_error() gives
 * the message of the last failure on the calling thread.  Lengths are in oxDNA simulation
 * units, temperatures in simulation units (1 = 3000 K), quaternions are (x, y, z, w) with the
 * body axes a1, a2, a3 as the columns of their rotation matrix, forces are in the lab frame and
 * torques in the body frame (the reference's conventions).  Device pointers are passed as
 * void * and streams as void * (a cudaStream_t, NULL for the legacy default stream).  A handle
 * may be used by one host thread at a time.  Nothing in this header depends on PyTorch.
 */
#ifndef OXGB_H
#define OXGB_H

#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum oxgb_status {
	OXGB_OK = 0,
	OXGB_E_INVALID = 1,        /* bad argument or call order */
	OXGB_E_CUDA = 2,           /* a CUDA runtime call failed */
	OXGB_E_FENE = 3,           /* a backbone bond left the FENE range */
	OXGB_E_NEIGH_OVERFLOW = 4, /* a neighbour row exceeded its capacity */
	OXGB_E_NONFINITE = 5,      /* non-finite or huge coordinates (an exploded simulation) */
	OXGB_E_NOMEM = 6
} oxgb_status;

/* model settings: the input keys read by DNAInteraction::get_settings and
 * DNA2Interaction::get_settings (src/Interactions/DNAInteraction.cpp:216-288,
 * src/Interactions/DNA2Interaction.cpp:62-99) */
typedef struct oxgb_dna2_settings {
	double T;                   /* T, simulation units */
	double salt;                /* salt_concentration (M) */
	int average;                /* use_average_seq */
	double seq_stck[4][4];      /* STCK_X_Y of seq_dep_file, X and Y in A G C T order */
	double seq_stck_fact_eps;   /* STCK_FACT_EPS */
	double seq_hydr_at;         /* HYDR_A_T */
	double seq_hydr_gc;         /* HYDR_G_C */
	double hb_multiplier;       /* hb_multiplier */
	int dh_half_charged_ends;   /* dh_half_charged_ends */
	double dh_lambda;           /* dh_lambda */
	double dh_strength;         /* dh_strength */
	int use_mbf;                /* max_backbone_force given */
	double mbf_fmax;            /* max_backbone_force */
	double mbf_finf;            /* max_backbone_force_far */
	int reference_cuda_eps;     /* 1: average-sequence well depths of the reference CUDA
	                               backend (oxDNA1 values, CUDADNAInteraction.cu:61-64);
	                               0 (default): the oxDNA2 values of the CPU DNA2 class */
} oxgb_dna2_settings;

/* fills *s with the reference defaults for the given temperature and salt */
void oxgb_dna2_default_settings(oxgb_dna2_settings *s, double T, double salt);

/* version string of the library */
const char *oxgb_version(void);
/* message of the last failure on this thread */
const char *oxgb_last_error(void);

/* ------------------------------------------------------------------ interaction layer */

typedef struct oxgb_dna2 oxgb_dna2;

/* CUDADNAInteraction::get_settings + cuda_init (src/CUDA/Interactions/CUDADNAInteraction.cu:28-154):
 * derives the parameter tables and uploads them to the current device */
int oxgb_dna2_create(const oxgb_dna2_settings *s, oxgb_dna2 **out);
/* CUDABaseInteraction::get_cuda_rcut: the interaction cutoff (Debye-Hueckel extended) */
int oxgb_dna2_get_rcut(const oxgb_dna2 *h, double *rcut);
/* CUDADNAInteraction::_on_T_update (CUDADNAInteraction.cu:156-158): new temperature */
int oxgb_dna2_set_temperature(oxgb_dna2 *h, double T);
/*
 * CUDADNAInteraction::compute_forces (src/CUDA/Interactions/CUDADNAInteraction.cu:165-203) on
 * the reference's device layout: d_poss float4 (x, y, z, w = int bits btype << 22 | index),
 * d_orientations float4 quaternions, d_bonds int2 (n3, n5; -1 for none), the neighbour matrix
 * with element k of nucleotide i at d_matrix_neighs[i * stride_i + k * stride_k] (the reference's
 * column-major CUDASimpleVerletList layout is stride_i = 1, stride_k = N) and counts in
 * d_number_neighs.  d_forces / d_torques (float4) arrive initialised by the caller (zeros or
 * external forces) and are accumulated into: force in the lab frame with w += energy, torque
 * in the body frame with w = hydrogen-bonding energy, exactly as the reference kernel leaves
 * them.  box is the cubic box side.  Asynchronous on `stream`.
 */
int oxgb_dna2_compute_forces(oxgb_dna2 *h, int N, double box, const void *d_poss, const void *d_orientations,
		void *d_forces, void *d_torques, const void *d_bonds, const int *d_matrix_neighs, const int *d_number_neighs,
		int max_neigh, long long stride_i, long long stride_k, void *stream);
/*
 * The FFS order-parameter kernels of CUDADNAInteraction (_hb_op_precalc, _near_hb_op_precalc,
 * _dist_op_precalc: src/CUDA/Interactions/CUDADNAInteraction.cu:205-218, kernels in
 * src/CUDA/Interactions/CUDA_DNA.cuh:910-1067) on the same device layout as compute_forces, for
 * the n_pairs pairs (d_op_pairs1[k], d_op_pairs2[k]):
 *   hb_op_precalc       d_hb_energies[k] = the pair's hydrogen-bonding energy (f1 times the six
 *                       f4 factors; no hb_multiplier, as the reference kernel);
 *   near_hb_op_precalc  d_nearly_bonded[k] (one byte, C bool) = at least six of those seven
 *                       factors are on (f1 < 0, each f4 > 0);
 *   dist_op_precalc     d_op_dists[k] = the distance between the two base sites.
 * Centre separations at the minimum image of the cubic box of side box.  Asynchronous on stream.
 */
int oxgb_dna2_hb_op_precalc(oxgb_dna2 *h, double box, const void *d_poss, const void *d_orientations,
		const int *d_op_pairs1, const int *d_op_pairs2, int n_pairs, float *d_hb_energies, void *stream);
int oxgb_dna2_near_hb_op_precalc(oxgb_dna2 *h, double box, const void *d_poss, const void *d_orientations,
		const int *d_op_pairs1, const int *d_op_pairs2, int n_pairs, bool *d_nearly_bonded, void *stream);
int oxgb_dna2_dist_op_precalc(oxgb_dna2 *h, double box, const void *d_poss, const void *d_orientations,
		const int *d_op_pairs1, const int *d_op_pairs2, int n_pairs, float *d_op_dists, void *stream);
int oxgb_dna2_destroy(oxgb_dna2 *h);

/* ------------------------------------------------------------------ Verlet list layer */

typedef struct oxgb_verlet oxgb_verlet;

/*
 * CUDASimpleVerletList::get_settings + init (src/CUDA/Lists/CUDASimpleVerletList.cu:44-52,
 * 165-202): rcut is the interaction cutoff, skin the verlet_skin, the cells per side follow
 * _compute_N_cells_side (cells_auto_optimisation), max_neigh bounds each neighbour row.
 */
int oxgb_verlet_create(int N, double box, double rcut, double skin, int cells_auto_optimisation, int max_neigh,
		oxgb_verlet **out);
/*
 * CUDASimpleVerletList::update (CUDASimpleVerletList.cu:231-289): rebuilds cells and neighbour
 * rows from d_poss (float4, reference layout), writes d_list_poss, excludes bonded pairs of
 * d_bonds.  Rows are column-major like the reference's d_matrix_neighs (element k of i at
 * k * N + i, src/CUDA/Lists/CUDABaseList.h:13).  Asynchronous; an overflow is reported by
 * oxgb_verlet_status after the stream is synchronised.
 */
int oxgb_verlet_update(oxgb_verlet *h, const void *d_poss, void *d_list_poss, const void *d_bonds, void *stream);
/*
 * No counterpart in the reference.  The same list build as oxgb_verlet_update into caller-owned
 * d_matrix_neighs (column-major, int[max_neigh * N]), d_number_neighs (int[N]) and
 * d_list_poss, with no device allocation at all: the scratch (cells, segments, scan tiles,
 * status) is a fixed static device array of the library, so the call never runs
 * cudaMalloc/cudaFree (which synchronise the device and can fail under a caching allocator
 * that holds the free memory), and needs no handle with a lifetime.  Limits: N <=
 * OXGB_NOALLOC_MAX_N and at most OXGB_NOALLOC_MAX_CELLS cells; larger requests return
 * OXGB_E_INVALID before any launch.  The scratch is shared by all calls on a device: calls
 * that overlap in time race and must be serialised by the caller.  The first call on a device
 * looks the scratch up (and may load the module), so it should precede any stream capture.
 * Synchronises `stream` to read the status: OXGB_E_NEIGH_OVERFLOW if a row exceeded max_neigh.
 */
#define OXGB_NOALLOC_MAX_N 65536
#define OXGB_NOALLOC_MAX_CELLS 32768
int oxgb_verlet_build_noalloc(int N, double box, double rcut, double skin, int cells_auto_optimisation,
		const void *d_poss, void *d_list_poss, const void *d_bonds, int *d_matrix_neighs, int *d_number_neighs,
		int max_neigh, void *stream);
/* device pointers of the neighbour rows (int[N * max_neigh]) and counts (int[N]) */
int oxgb_verlet_buffers(oxgb_verlet *h, int **d_matrix_neighs, int **d_number_neighs, int *max_neigh, int *n_cells_side);
int oxgb_verlet_status(oxgb_verlet *h);
int oxgb_verlet_destroy(oxgb_verlet *h);

/* ------------------------------------------------------------------ MD backend layer */

typedef struct oxgb_md oxgb_md;

enum { OXGB_THERMOSTAT_NONE = 0, OXGB_THERMOSTAT_BROWNIAN = 1, OXGB_THERMOSTAT_BUSSI = 2 };
/* backend_precision (src/Backends/BackendFactory.cpp:50-86): mixed = FP32 forces with FP64
 * integration (the reference's default, MD_CUDAMixedBackend); double = FP64 throughout; float
 * = FP32 forces and FP32 integration (src/CUDA/Backends/CUDA_MD.cuh:11-60,556-578: kicks,
 * drift and rotation in FP32, the state FP32-representable) */
enum { OXGB_PRECISION_MIXED = 0, OXGB_PRECISION_DOUBLE = 1, OXGB_PRECISION_FLOAT = 2 };

/* MDBackend / thermostat input keys (src/Backends/MDBackend.cpp:25-90,
 * src/Backends/Thermostats/{Brownian,Bussi}Thermostat.cpp get_settings) */
typedef struct oxgb_md_settings {
	double dt;                  /* dt */
	double verlet_skin;         /* verlet_skin */
	int thermostat;             /* thermostat: none, john/brownian, bussi */
	int newtonian_steps;        /* newtonian_steps */
	double pt;                  /* pt (0: derived from diff_coeff) */
	double diff_coeff;          /* diff_coeff */
	double bussi_tau;           /* bussi_tau */
	uint64_t seed;              /* seed of the counter-based random stream */
	int precision;              /* backend_precision: OXGB_PRECISION_MIXED, _DOUBLE or _FLOAT */
	int cells_auto_optimisation;/* cells_auto_optimisation */
	int max_neigh;              /* neighbour-row capacity; 0 = sized from the first build */
	int steps_per_graph;        /* MD steps captured per CUDA graph launch (0 = 16) */
	int list_rebuild_node;      /* 0: the list rebuild is a device-side IF node of the step graph;
	                               1: the rebuild kernels are launched every step and return at once
	                               while the list is fresh (same results; kernel nodes profilable) */
	int sort_every;             /* CUDA_sort_every (CUDABaseBackend.cu:263-281): every sort_every-th
	                               list rebuild stores the nucleotides in cell order, on the device
	                               (0: never).  Forces, Brownian and NVE trajectories are bit-identical
	                               to an unsorted run; the state, forces and energies cross this
	                               interface in the caller's order.  Device buffers and the rows of
	                               oxgb_md_neighbours are in storage order (oxgb_md_storage_order). */
	int autotune;               /* 1: the first oxgb_md_set_state times every shape of the MD step's
	                               force kernels on that state and keeps the fastest (cached per size
	                               class for later engines); 0: the default shape.  Shapes change the
	                               work distribution, not the arithmetic of a pair.  The reference has
	                               no counterpart (a fixed 64 threads per block,
	                               src/CUDA/Backends/CUDABaseBackend.cu:244-261). */
	int use_edge;               /* use_edge (CUDABaseInteraction / CUDASimpleVerletList get_settings;
	                               kernels CUDA_DNA.cuh:727-830): 1 evaluates Debye-Hueckel and the
	                               excluded volume once per unordered pair, adding both nucleotides'
	                               shares with atomic adds (the summation order, and so the last bits of
	                               the forces, then vary from run to run; the shape is the default one);
	                               0 (default): each pair from both ends, a fixed order */
	int sort_order;             /* the storage order of sort_every: OXGB_SORT_HILBERT (default; the
	                               reference's key, CUDA_sort.cu:106-200): the cells of each system
	                               along a 3D Hilbert curve, nucleotides by caller's index within a
	                               cell; OXGB_SORT_CELLS: row-major cell order */
	int list_kernel;            /* OXGB_LIST_AUTO (default), _WARP, _THREAD or _GROUP4/8/16 (below) */
} oxgb_md_settings;
enum { OXGB_SORT_HILBERT = 0, OXGB_SORT_CELLS = 1 };
/* oxgb_md_settings.list_kernel: the neighbour-row kernel of the list build.  All give the same
 * rows entry for entry; which is faster depends on how many candidates a nucleotide's 27 cells hold
 * and on how many nucleotides a build covers.  AUTO: timed by the autotuner (md.autotune), else
 * WARP; WARP: a warp per nucleotide, lanes over the candidates; THREAD: a thread per nucleotide,
 * coalesced stores into the column-major rows; GROUP4 / GROUP8 / GROUP16: 4, 8 or 16 lanes per
 * nucleotide over its candidates */
enum { OXGB_LIST_AUTO = 0, OXGB_LIST_WARP = 1, OXGB_LIST_THREAD = 2, OXGB_LIST_GROUP4 = 3, OXGB_LIST_GROUP8 = 4,
	OXGB_LIST_GROUP16 = 5 };

void oxgb_md_default_settings(oxgb_md_settings *s);

/*
 * A batch of n_systems independent systems in one engine (n_systems = 1 for a plain run).
 * offsets[n_systems + 1] partitions the N = offsets[n_systems] nucleotides; system k has its own
 * cubic box box[k] and model settings dna[k] (temperature, salt, ...), hence its own cutoff,
 * cell grid, Verlet lists and thermostat, and its random stream uses the seed md->seed + k
 * (keyed by the index within the system, so a system evolves exactly as it would alone).  All
 * systems step together in the same kernels and graphs.  Bonds may not cross systems.
 * Allocates device memory on the current device.  MD_CUDABackend::get_settings + init
 * (MD_CUDABackend.cu:621-755).
 */
int oxgb_md_create(int n_systems, const int *offsets, const double *box, const oxgb_dna2_settings *dna,
		const oxgb_md_settings *md, oxgb_md **out);
/* topology: n3/n5 neighbour indices (global, -1 for none), pairing code btype, base type 0..4 */
int oxgb_md_set_topology(oxgb_md *h, const int *n3, const int *n5, const int *btype, const int *type);
/*
 * MD_CUDABackend::apply_changes_to_simulation_data (MD_CUDABackend.cu:231-313): uploads
 * positions pos[3N], quaternions quat[4N], velocities vel[3N] and angular momenta L[3N] (body
 * frame), rebuilds the Verlet lists and computes the forces of this state.
 */
int oxgb_md_set_state(oxgb_md *h, const double *pos, const double *quat, const double *vel, const double *L);
/* MD_CUDABackend::apply_simulation_data_changes (MD_CUDABackend.cu:315-394): downloads the state */
int oxgb_md_get_state(oxgb_md *h, double *pos, double *quat, double *vel, double *L);
/* nsteps calls of sim_step (MD_CUDABackend.cu:567-619), replayed as CUDA graphs; returns when
 * they are enqueued unless sync is set.  The step counter continues across calls. */
int oxgb_md_run(oxgb_md *h, int nsteps, int sync);
/* forces (lab, F[3N]), torques (body, T[3N]) and per-nucleotide energies (E[N], every pair term
 * counted on both nucleotides) of the current state, plus the per-system split into the 8 terms
 * of the reference's potential_energy observable (E_split[8 * n_systems]: FENE, bonded excluded
 * volume, stacking, non-bonded excluded volume, hydrogen bonding, cross stacking, coaxial
 * stacking, Debye-Hueckel).  Any output pointer may be NULL. */
int oxgb_md_compute_forces(oxgb_md *h, double *F, double *T, double *E, double *E_split);
/* forces and torques the dynamics uses (those of the last step, or of the last state upload)
 * and per-nucleotide energies of the current state; the download half of
 * apply_simulation_data_changes.  The MD steps compute forces and torques only: E is evaluated
 * on request from the current state and lists, in separate buffers, so asking for it never
 * changes a trajectory. */
int oxgb_md_get_forces(oxgb_md *h, double *F, double *T, double *E);
/* per-system potential energy (FP64 sum of the per-nucleotide energies / 2, evaluated on
 * request as for oxgb_md_get_forces) and the translational and rotational kinetic energies,
 * each double[n_systems] */
int oxgb_md_energies(oxgb_md *h, double *U, double *K_t, double *K_r);
/* new temperature of system k (parameter table, cutoff, thermostat; the Bussi running kinetic
 * energies scale with T; the lists are rebuilt) -- the replica-exchange hook.  Velocities are
 * left to the caller (a swap usually rescales them by sqrt(T_new / T_old)). */
int oxgb_md_set_temperature(oxgb_md *h, int k, double T);
/*
 * External forces, the CUDA backend's set_external_forces (src/CUDA/Backends/CUDA_MD.cuh:97-555,
 * records of src/CUDA/Forces/forces_defs.cuh) for the force types of src/Forces/
 * {ConstantRateForce,MutualTrap,MovingTrap,LowdimMovingTrap,RepulsionPlane,AttractionPlane,
 * RepulsiveSphere,RepulsiveSphereSmooth,LJWall,GenericCentralForce,RepulsionPlaneMoving,LJCone,
 * ConstantRateTorque,RepulsiveEllipsoid,COMForce,YukawaSphere,RepulsiveSphereMoving}.cpp.
 * Each record acts on one nucleotide (global index) and is evaluated at every force evaluation
 * from the FP64 positions, with `step` the MD step being computed (0 for a state just uploaded);
 * no torques, no energies (as in the reference).  dir is taken as given (the reference
 * normalises it when it reads the file).  With r the nucleotide's position:
 *   CONSTANT:          F += (F0 + rate step) dir, dir -> unit(dir - r) if flags & 1
 *   MUTUAL_TRAP:       d = r(ref) - r (minimum image if flags & 1), F += d (|d| - (r0 + rate step))
 *                      (stiff + stiff_rate step) / |d|
 *   MOVING_TRAP:       F += -stiff (r - (pos0 + rate step dir))
 *   LOWDIM_TRAP:       the same on the components whose flags bit (2: x, 4: y, 8: z) is set
 *   REPULSION_PLANE:   p = position + rate step, stopped at r0 (the end position) when rate != 0;
 *                      d = dir . r + p; F += -d stiff dir where d < 0
 *   ATTRACTION_PLANE:  d = dir . r + position; F += -d stiff dir where d < 0, else -stiff dir
 *   SPHERE:            d = minimum image of r - pos0 (the centre), R = r0 + rate step;
 *                      F += -stiff (1 - R / |d|) d where R < |d| < cutoff (r_ext)
 *   SPHERE_SMOOTH:     d = minimum image of r - pos0; where r0 <= |d| <= cutoff (r_ext):
 *                      F += -(stiff / 2) exp((|d| - p1) / sigma) d / |d| if |d| >= p1 (alpha),
 *                      else -(stiff |d| - (stiff / 2) exp(-(|d| - p1) / sigma)) d / |d|
 *                      (sigma: the smoothing length)
 *   LJ_WALL:           x = dir . r + position, y = x / sigma; where y <= cutoff:
 *                      F += 4 n stiff (2 y^-2n - y^-n) / x dir
 *   CENTRAL:           (generic_central_force, force_type = gravity) d = pos0 - r; unless |d| <
 *                      p1 (inner cut-off) or, p2 > 0, |d| > p2 (outer): F += F0 d / |d|
 *   REPULSION_PLANE_MOVING: x = (r - r(ref)) . dir; F += -stiff min(x, 0) dir (one record per
 *                      reference particle; the records of a nucleotide add up)
 *   LJ_CONE:           apex pos0, axis dir, half-angle p1 (alpha): with v = r - pos0, a = v . dir,
 *                      b = |a dir - v|, x = a sin(alpha) - b cos(alpha), y = x / sigma; where
 *                      y <= cutoff: F += 4 n stiff (2 y^-2n - y^-n) / x nrm, nrm = unit((a + b
 *                      tan(alpha)) dir - v)
 *   TWIST:             (twist) the trap pos0 rotated by F0 + rate step radians about the unit axis
 *                      dir through v1 (the centre): F += -stiff (r - trap) * v2 (the mask,
 *                      component-wise)
 *   ELLIPSOID:         d = minimum image of r - pos0 (the centre); unless sum (d_k / v2_k)^2 < 1
 *                      (inside r_2) and sum (d_k / v1_k)^2 > 1 (outside r_1): F += -stiff d / |d|
 *   COM:               (com) with c = centre of mass of group n (com_list, oxgb_md_set_force_groups)
 *                      and c' = that of group ref_particle (ref_list), d = c' - c: F += d (|d| -
 *                      (r0 + rate step)) stiff / (|d| n_com), one record per member of group n
 *   YUKAWA_SPHERE:     d = minimum image of r - pos0 (the centre), s = r0 (the radius) - |d|;
 *                      where s < cutoff: F += -d / |d| (F0 exp(-s / p2) (1 / (s p2) + 1 / s^2)),
 *                      F0 = debye_A, p2 = debye_length; where also s < p1 (the WCA cut-off):
 *                      F += -d / |d| 4 stiff n (2 w^2 - w) / s, w = (sigma / s)^6, n = WCA_n
 *   SPHERE_MOVING:     (repulsive_sphere_moving) centre v1 + (v2 - v1) clamp(step / p1, 0, 1)
 *                      (origin v1, target v2, p1 steps; the origin if p1 <= 0); d = minimum image
 *                      of r - centre, g = |d| - (r0 + rate step); where g < cutoff (r_ext) and
 *                      g < sqrt 2: A = 1 / max(g, 1e-9)^2, F += 8 stiff (2 A - 1) A / max(g,
 *                      1e-9) d / |d|
 */
enum {
	OXGB_FORCE_CONSTANT = 0,
	OXGB_FORCE_MUTUAL_TRAP = 1,
	OXGB_FORCE_MOVING_TRAP = 2,
	OXGB_FORCE_LOWDIM_TRAP = 3,
	OXGB_FORCE_REPULSION_PLANE = 4,
	OXGB_FORCE_ATTRACTION_PLANE = 5,
	OXGB_FORCE_SPHERE = 6,
	OXGB_FORCE_SPHERE_SMOOTH = 7,
	OXGB_FORCE_LJ_WALL = 8,
	OXGB_FORCE_CENTRAL = 9,
	OXGB_FORCE_REPULSION_PLANE_MOVING = 10,
	OXGB_FORCE_LJ_CONE = 11,
	OXGB_FORCE_TWIST = 12,
	OXGB_FORCE_ELLIPSOID = 13,
	OXGB_FORCE_COM = 14,
	OXGB_FORCE_YUKAWA_SPHERE = 15,
	OXGB_FORCE_SPHERE_MOVING = 16
};
typedef struct oxgb_ext_force {
	int type, particle, ref_particle, flags;
	double F0, rate, stiff, stiff_rate, r0, position;
	double dir[3], pos0[3];
	double sigma, cutoff, p1, p2; /* parameters of the sphere, wall, cone and central types */
	int n, pad;                   /* the Lennard-Jones exponent of LJ_WALL / LJ_CONE, the WCA
	                                 exponent of YUKAWA_SPHERE, the centre-of-mass group of COM */
	double v1[3], v2[3];          /* further vectors: TWIST centre and mask, ELLIPSOID r_1 and r_2,
	                                 SPHERE_MOVING origin and target */
} oxgb_ext_force;
/* replaces the engine's external forces by f[0 .. n-1] (n = 0 removes them) */
int oxgb_md_set_external_forces(oxgb_md *h, int n, const oxgb_ext_force *f);
/* the particle groups of COM records (COMForce's com_list / ref_list): group g holds the caller's
 * indices members[offsets[g] .. offsets[g + 1] - 1]; replaces the previous groups.  Call before
 * oxgb_md_set_external_forces; no counterpart in the reference, whose records hold the lists. */
int oxgb_md_set_force_groups(oxgb_md *h, int n_groups, const int *offsets, const int *members);
/* velocities and angular momenta of system k times f (after a temperature swap: f =
 * sqrt(T_new / T_old)); no counterpart in the reference's CUDA backend, which has no batches */
int oxgb_md_scale_momenta(oxgb_md *h, int k, double f);
/* neighbour rows of the last list build: counts nnb[N], rows nb[N * max_neigh] (row-major),
 * cell index of every nucleotide cell[N]; any pointer may be NULL */
int oxgb_md_neighbours(oxgb_md *h, int *nnb, int *nb, int max_neigh, int *cell, int *n_cells_side);
/* number of list rebuilds so far, current step counter, neighbour-row capacity */
int oxgb_md_info(oxgb_md *h, long long *n_rebuilds, long long *step, int *max_neigh);
/* id[k] = the caller's index of the nucleotide stored at slot k (the identity until a cell-order
 * sort, oxgb_md_settings.sort_every) */
int oxgb_md_storage_order(oxgb_md *h, int *id);
/* status bits raised by the kernels since the last call (and clears them): 0 = healthy */
int oxgb_md_status(oxgb_md *h);
/* the shape of the MD step's force kernels: nucleotides per pair-block warp queue, non-bonded
 * lanes per nucleotide, the register cap as resident blocks per SM, and (autotuned engines) the
 * measured launch time in microseconds (0 otherwise).  No counterpart in the reference. */
int oxgb_md_force_shape(oxgb_md *h, int *pair_npw, int *nb_lanes, int *nb_min_blocks, double *launch_us);
/* pins shape k (0 .. 5; 0 the default) of the MD step's force kernels, e.g. to repeat a tuned run
 * on another engine; the forces of the current state are recomputed with it.  No counterpart in
 * the reference. */
int oxgb_md_set_force_shape(oxgb_md *h, int k);
/* the shape table itself: shape k's nucleotides per pair-block warp queue, non-bonded lanes per
 * nucleotide and register cap (OXGB_E_INVALID past the last shape) */
int oxgb_force_shape_table(int k, int *pair_npw, int *nb_lanes, int *nb_min_blocks);
/* the neighbour-row kernel the engine's list builds use: OXGB_LIST_WARP, _THREAD or _GROUP4/8/16 */
int oxgb_md_list_kernel(oxgb_md *h, int *kernel);
/* device pointers (for zero-copy callers): FP64 positions, velocities, angular momenta and
 * quaternions (double4 each), FP32 forces and torques (float4; double4 in double precision) */
int oxgb_md_device_buffers(oxgb_md *h, void **pos, void **vel, void **L, void **quat, void **F, void **T);
/* the CUDA stream all of the engine's work runs on */
void *oxgb_md_stream(oxgb_md *h);
/* enqueues one force and energy evaluation of the current state and lists, device only, into
 * the engine's evaluation buffers (the forces the dynamics uses are left alone): the engine-side
 * equivalent of CUDABaseInteraction::compute_forces, used to time the kernels */
int oxgb_md_launch_forces(oxgb_md *h);

/* ------------------------------------------------------------------ diagnostics */

/* measures the FP32 FMA throughput of the current device (FLOP/s) with a register-resident
 * multiply-add chain, the denominator of the force kernel's roofline */
int oxgb_probe_fp32_peak(double *flops_per_s);
int oxgb_md_destroy(oxgb_md *h);

#ifdef __cplusplus
}
#endif

#endif
