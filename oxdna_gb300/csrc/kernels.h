// Internal interface between the C-ABI layer (api.cu) and the kernels.
#pragma once

#include <cuda_runtime.h>

#include "../../include/oxgb.h"
#include "dna2_pair.cuh"

// device status bits (OR-ed by kernels, read by the host between launches)
#define OXGB_ERR_FENE 1            /* a backbone bond left the FENE range */
#define OXGB_ERR_NEIGH_OVERFLOW 2  /* a neighbour row exceeded its capacity */
#define OXGB_ERR_NONFINITE 4       /* a non-finite or huge coordinate */
#define OXGB_ERR_CELL 8            /* cell index out of range */

namespace oxgb {

// Programmatic dependent launch.  A kernel launched with launch_after may start while the
// kernel before it on the stream is still running (once every block of that one has called
// pdl_trigger or finished); it calls pdl_wait before it reads anything the earlier kernel
// writes, and may do independent work first.  pdl_wait returns at once in a kernel launched
// the ordinary way.  Both are hardware waits: they end when the earlier grid completes.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_after(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = grid;
	cfg.blockDim = block;
	cfg.dynamicSmemBytes = smem;
	cfg.stream = s;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	at[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Thermostat and step bookkeeping of the MD engine.  The step number of a kernel is
// *step_base + step_offset: a graph of K steps bakes offsets 0..K-1 and advances the base by K
// at its end, so no kernel of a step changes the number the others read.  Velocity Verlet
// runs with a deferred second half kick: the forces of step s are computed at the end of step
// s, and the next first step (or the flush at the end of a run) completes v(s+1) = v + dt/2 F,
// applies the thermostat of step s to it, then makes its own half kick and drift.
#define OXGB_NO_STEP (-4611686018427387904LL)  // "no step" mark of open_step / bussi_stamp

// per-system thermostat parameters, sys_par[s * SP_STRIDE + k]
enum { SP_T = 0, SP_SQRTT, SP_PT, SP_PR, SP_1MC, SP_A, SP_B, SP_INVN, SP_STRIDE = 8 };

// Every engine handles a batch of independent systems packed one after the other (a plain run
// is a batch of one): nucleotide i belongs to system sys[i], whose nucleotides are
// sys_off[s] .. sys_off[s + 1] - 1.  The random streams are keyed by (system seed, step, index
// within the system), so a system evolves exactly as it would alone with that seed.
struct ThermoArgs {
	int N;                                 // nucleotides of all systems
	int n_systems;
	int thermostat;                        // 0 none, 1 brownian, 2 bussi
	int newtonian_steps;
	double dt;
	const int *sys, *sys_off;
	const double *sys_par;                 // [n_systems * SP_STRIDE]: T, sqrt T, pt, pr, and with
	                                       // c = exp(-newtonian_steps / tau): 1 - c, (1 - c) T / 2,
	                                       // sqrt(2 T (1 - c) c), 1 / N_s
	const unsigned long long *sys_seed;    // [n_systems]
	// Bussi: the kinetic sums run over chunks of up to 256 nucleotides of one system
	const int *chunk_sys, *chunk_first;    // [chunks]
	const int *sys_chunk0;                 // [n_systems + 1] first chunk of each system
	double *bussi_partials;                // [chunks * 16] per-chunk sums 0-4 of the half-kicked
	                                       // state (v, |v|^2, |L|^2); the force terms (F, v.F,
	                                       // |F|^2, L.T, |T|^2) go to bussi_fpart
	float4 *bussi_vf, *bussi_Lf;           // [N] half-kicked v and L rounded to FP32 (mixed precision)
	double *bussi_state;                   // [n_systems * 16]: K_t, K_r, factor_t, factor_r,
	                                       // vcom x y z, -, then the step's draws: sum_t, rr_t,
	                                       // sum_r, rr_r
	unsigned *bussi_done;                  // [n_systems] chunks arrived in this step's sums (0 between steps)
	unsigned *bussi_prep_done;             // the same for the sums of the half-kicked state
	double *bussi_tot;                     // [n_systems * 8] system totals of the half-kicked state
	float2 *bussi_fpart;                   // [chunks * 8] per-chunk force-term sums as float pairs
	long long *bussi_stamp;                // step of the last Bussi update (OXGB_NO_STEP: none)
	long long *open_step;                  // step whose second half kick is pending
	                                       // (OXGB_NO_STEP: none); null in force-only calls
	long long *step_base;                  // device step counter of the current graph
	int step_offset;
	const int *id;                         // [N] caller's index of the nucleotide at each slot
	                                       // (null: never sorted, slot = index); keys the draws
};

struct ForceArgs {
	int N;
	const float4 *pos_hi, *pos_lo;         // FP32 mirrors (w of pos_hi: btype<<22 | index, w of pos_lo: type)
	const float4 *fa1, *fa3;               // FP32 body axes a1, a3 (rounded once from FP64)
	const float4 *quat;                    // reference layout only: FP32 quaternions
	const double4_32a *posd, *quatd;          // FP64 state
	const int2 *bonds;                    // (n3, n5), -1 if none
	const int *nb, *nnb;                  // neighbour rows and counts
	const int *dh_nb, *dh_n;              // Debye-Hueckel rows (engine; null: the full rows)
	int max_nb;
	long long nb_stride_i, nb_stride_k;   // element (i, k) at nb[i * stride_i + k * stride_k]
	void *forces, *torques;               // float4 or double4_32a per particle
	const void *table;                    // DNA2Table<float> or DNA2Table<double>, one per system
	const int *sys;                       // [N] system of each nucleotide (null: one system)
	int tab_span;                         // most systems one block of the split kernels touches
	int *status;
	double *esplit;                       // [8 * n_systems] energies (split kernels only)
	// split path (engine layout): backbone-site offsets (w = strand-end flag), term lists
	// (column-major: element k of nucleotide i at [k * N + i]) and the per-bond buffers
	const float4 *fback;
	const float4 *fa1lo, *fbacklo;            // remainders of fa1 / fback (null: the FP32 sites unrefined)
	const int *ev_nb, *ev_n, *base_nb, *base_n, *stk_nb, *stk_n;
	int ev_cap, base_cap, stk_cap;            // capacities (an overflowed list is read up to them)
	void *bond_f, *bond_tp, *bond_tq;         // per bond owner p (q = n3[p]): f on q with w = energy, torques
	// base / stack pairs are evaluated once, by their lower nucleotide i (by caller's index), which writes slot k of i
	// and slot pos[k N + i] of its partner j: (force, E), (torque, E_hb) as two V4 per slot
	void *base_res, *stk_res;
	const int *base_pos, *stk_pos;            // see ListArgs
	const int *term_max;                      // [4] longest EV / base / stack list (slots past it are empty), full row
	// MD-step bookkeeping (engine layout): the bonded kernel marks the step's half kick pending
	ThermoArgs th;
	// external forces (oxgb_ext_force records grouped by nucleotide): ext_n nucleotides
	// ext_nuc[k] with records ext_off[k] .. ext_off[k + 1] - 1
	const void *ext_rec;
	const int *ext_nuc, *ext_off;
	int ext_n;
	const int *grp_off, *grp_mem;             // particle groups of COM records (caller's indices)
	float box;                                // cubic box of the (single-system) engine
	const float *sys_box;                     // per system (batches), or null
	// cell-order storage (null: never sorted): caller's index of each slot, which decides the
	// owner of a base / stack pair as in an unsorted run, and the slot of each caller's index
	// (external-force records name caller's indices)
	const int *id, *slot;
	// shape of the MD step's kernels (no energies; mixed / float engine): index into the
	// autotuner's shape table, 0 the default
	int shape;
	// use_edge: Debye-Hueckel and excluded volume evaluated once per unordered pair by the edge
	// blocks of the bonded/pair kernel, both nucleotides' shares added atomically into edge_acc
	// ([2 N] V4: force with w = energy, lab torque with w = hydrogen-bonding energy), which the
	// non-bonded kernel gathers and clears; 0 (default): both from each end of the full rows
	int edge;
	void *edge_acc;
};

cudaError_t launch_forces_reference_layout(const ForceArgs &a, cudaStream_t s);
// FFS order parameters of listed pairs on the reference layout (mode 0 hydrogen-bonding energy,
// 1 nearly-bonded flag, 2 base-base distance)
cudaError_t launch_order_params(int mode, const float4 *poss, const float4 *quat, const int *op1, const int *op2, int n,
		const void *table, float *val, bool *flag, cudaStream_t s);
// split path: bonded pairs (one thread per bond, both sides), then non-bonded terms (one
// thread per nucleotide, one loop per term list) with the bonded results gathered in its epilogue
// wait: an event the non-bonded kernel waits for, or null
// energy = false: forces and torques only (w of F and T left 0), what an MD step needs
cudaError_t launch_forces_split(const ForceArgs &a, bool dbl, bool split, bool energy, cudaStream_t s,
		cudaEvent_t wait = nullptr);
// blocks of the split non-bonded kernel for N nucleotides at `lanes` lanes per nucleotide
int nonbonded_blocks(int N, int lanes);
// shapes of the MD step's force kernels (mixed / float engine, ForceArgs::shape): how many, and
// shape k's nucleotides per pair-block warp queue, non-bonded lanes per nucleotide and register cap
int force_shape_count();
void force_shape_of(int k, int *npw, int *lanes, int *minb);
// lets the split kernels use `bytes` of dynamic shared memory (per-block system tables);
// nonzero if that is more than they may have
int set_forces_smem(bool dbl, size_t bytes);

struct ListArgs {
	int N;
	const float4 *pos;      // FP32 positions the list is built from (hi part)
	float box;
	float rverlet2;
	int n_side;             // cells per side
	const int2 *bonds;
	int *cell_of;           // [N]
	int *cell_count;        // [n_cells]
	int *cell_start;        // [n_cells + 1]
	int *cell_cursor;       // [n_cells]
	int *cell_list;         // [N] particles by cell, by caller's index within a cell
	int *cell_tmp;          // [N] scatter target before the ordering
	int *scan_part;         // [scan_tiles(n_cells) + 1]
	int *nb, *nnb;          // [N * max_nb], [N]
	int max_nb;
	float4 *list_pos;       // positions at this build
	int *status;
	int *flag;              // rebuild request, cleared by the build
	int check_flag;         // 1: every kernel exits at once unless *flag is set
	unsigned long long *rebuilds;  // counts builds (may be null)
	// term lists (null: full rows only).  A pair enters the excluded-volume list when its centres
	// are closer than ev_r, the base list when its base sites are closer than base_r, the stack
	// list when its stacking sites are closer than stk_r (all thresholds include twice the skin)
	const float4 *fa1, *fback;
	int *ev_nb, *ev_n, *base_nb, *base_n, *stk_nb, *stk_n;
	// for every base / stack entry (k, i) whose partner j is higher (i owns the pair): the
	// position of i in j's list, where the pair evaluation also writes j's result; -1 otherwise
	int *base_pos, *stk_pos;
	int ev_cap, base_cap, stk_cap;
	float ev_r2, base_r2, stk_r2;
	// the excluded-volume list keeps only pairs with a site pair within its cutoff plus twice the
	// skin (squared: backbone-backbone, base-base, backbone-base)
	float evs_r2[3];
	// Debye-Hueckel rows (null: none): the entries of the full rows whose backbone sites are
	// closer than sqrt(dh_r2) (the Debye-Hueckel cutoff plus twice the skin; per system in
	// sys_dh2 for a batch), column-major with the full rows' capacity
	int *dh_nb, *dh_n;
	float dh_r2;
	const float *sys_dh2;
	float4 *list_a1, *list_back;   // body axis a1 and backbone offset at this build
	int *term_max;          // [4] longest EV / base / stack list and full row of any build so far (may be null)
	int col_major;          // full rows column-major ([k * N + i]) instead of row-major
	// batch of systems (sys null: one system with the scalar geometry above).  System s has
	// its own box, cutoff and cell grid (sys_nside^3 cells from sys_cell0); only systems with
	// sys_stale set are rebuilt (their cells, segments and rows), the others keep theirs
	const int *sys, *sys_nside, *sys_cell0, *cell_sys;
	const float *sys_box, *sys_rv2;
	int *sys_stale;
	int n_systems;
	int n_cells_total;      // cells of all systems (0: n_side^3)
	// Cell-order storage (CUDA_sort_every; sort_every 0 or id null: off).  On every sort_every-th
	// build the nucleotides of the rebuilt systems move to the slots of their cell order (cell,
	// then caller's index) before the rows are built: the FP64 state, the mirrors, bonds
	// (renumbered) and id.  Segments are ordered and pairs owned by caller's index, so the rows
	// list the same partners in the same order as an unsorted build.
	int sort_every;
	int *id, *slot;         // [N] caller's index of each slot, and its inverse
	int *perm, *inv;        // [N] scratch: old slot of new slot k, new slot of old slot
	double4_32a *st[4];     // FP64 state: positions, velocities, angular momenta, quaternions
	float4 *mir[7];         // mirrors: pos_hi, pos_lo, fa1, fa3, fback, fa1lo, fbacklo (any may be null)
	int2 *bonds_rw;         // the bonds the rows exclude (the array of `bonds`)
	unsigned char *scratch; // [N * SORT_BYTES]
	// Hilbert order of the cells (null: row-major cell order): cell c of the global numbering is
	// the cell_hil[c]-th of its system's cells along a Hilbert curve (plus the system's first
	// cell); hcount / hstart / hcursor [n_cells + 1] are the counts and the exclusive scan in that
	// order.  hilbert_pass marks the argument copy that runs the scan kernels on them.
	const int *cell_hil;
	int *hcount, *hstart, *hcursor;
	int hilbert_pass;
	int list_kind;          // neighbour-row kernel: OXGB_LIST_WARP, _THREAD or _GROUP4/8/16
};

// bytes per nucleotide of the sort's staging buffer: 4 FP64 vectors, 7 FP32 vectors, bonds,
// id and cell
#define SORT_MIRRORS 7
#define SORT_BYTES (4 * 32 + SORT_MIRRORS * 16 + 8 + 4 + 4)

// full rebuild: cells (counting sort, deterministic order) then neighbour rows
cudaError_t launch_list_build(const ListArgs &a, cudaStream_t s);
// size of ListArgs::scan_part is scan_tiles(n_cells) + 1
int scan_tiles(int n_cells);

struct StepArgs {
	int N;
	double dt;
	double4_32a *pos, *vel, *angmom, *quat;   // FP64 state
	int f32;                               // backend_precision = float: FP32 integration, the state kept FP32-representable
	float4 *pos_hi, *pos_lo, *fa1, *fa3;  // FP32 mirrors written by the first step
	const void *forces, *torques;         // float4 (mixed) or double4_32a (double)
	const float4 *list_pos;
	float4 *fback;                         // backbone offset (w: strand-end flag), written with the mirrors
	float4 *fa1lo, *fbacklo;               // remainders of fa1 and fback (mixed / float engine; null: none)
	const int2 *bonds;
	const float4 *list_a1, *list_back;     // site data of the last list build (null: centres only)
	float skin2;
	int *flag;
	int *sys_stale;                        // [n_systems] per-system rebuild requests
	int *status;
	ThermoArgs th;
};

// first half of an MD step: completes a pending half kick and the previous step's thermostat,
// then half kick, drift, rotation, FP32 mirrors and the list-staleness flags
cudaError_t launch_first_step(const StepArgs &a, bool double_forces, cudaStream_t s);
// the Bussi draws of the current step, per system (they do not depend on the state: they run
// beside the step)
cudaError_t launch_bussi_noise(const StepArgs &a, cudaStream_t s);
// Bussi kinetic-energy sums of the half-kicked state (after the first step, beside the forces)
// and of the force terms with the per-system update (after the forces); n_chunks chunks of up to
// 256 nucleotides
cudaError_t launch_bussi_prep(const StepArgs &a, int n_chunks, bool double_forces, cudaStream_t s);
cudaError_t launch_bussi_reduce(const StepArgs &a, int n_chunks, bool double_forces, cudaStream_t s);
// id[k] = slot[k] = k: the caller's order (cell-order storage undone)
cudaError_t launch_identity_order(int *id, int *slot, int N, cudaStream_t s);
// end of a graph of K steps: the step base advances by K
cudaError_t launch_step_advance(const StepArgs &a, int K, cudaStream_t s);
// end of a run: completes the pending half kick and thermostat so the state is whole
cudaError_t launch_step_flush(const StepArgs &a, bool double_forces, cudaStream_t s);
// the caller's state arrays (3, 4, 3, 3 doubles per nucleotide, back to back) to and from the
// FP64 state; *bad receives the lowest nucleotide whose quaternion cannot be normalised (with
// check_only that is all that is written)
cudaError_t launch_unpack_state(const StepArgs &a, const double *in, int *bad, bool check_only, cudaStream_t s);
cudaError_t launch_pack_state(const StepArgs &a, double *out, cudaStream_t s);
cudaError_t launch_set_conditional(const int *flag, cudaGraphConditionalHandle h, cudaStream_t s);
// refresh the FP32 mirrors from the FP64 state (after a host upload)
cudaError_t launch_make_mirrors(const StepArgs &a, cudaStream_t s);
// velocities and angular momenta of nucleotides lo .. hi - 1 times f
cudaError_t launch_scale_momenta(const StepArgs &a, int lo, int hi, double f, cudaStream_t s);
// per-chunk FP64 sums of the potential energy (sum of F.w / 2) and the translational and
// rotational kinetic energies: out[chunk * 4 + {0, 1, 2}]
cudaError_t launch_system_sums(const StepArgs &a, int n_chunks, bool double_forces, double *out, cudaStream_t s);

}  // namespace oxgb
