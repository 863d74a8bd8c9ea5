// Link-time substitute for the reference's CUDADNAInteraction (declared in
// src/CUDA/Interactions/CUDADNAInteraction.h, which this file includes unchanged): a reference
// program linked with this object instead of src/CUDA/Interactions/CUDADNAInteraction.cu
// evaluates DNA / DNA2 forces with liboxgb (oxgb_dna2_compute_forces on the reference's own
// device buffers), selected by the reference's own keys -- backend = CUDA, interaction_type =
// DNA2 (or DNA) -- through its unmodified CUDAInteractionFactory
// (src/CUDA/Interactions/CUDAInteractionFactory.cu:31-53).
//
// The CPU side stays the reference's DNAInteraction (the class this one derives from): it reads
// the input keys and initialises the model; for interaction_type = DNA2 the DNA2 constants are
// taken as DNA2Interaction sets them (src/Interactions/DNA2Interaction.cpp:103-155: the oxDNA2
// stacking and hydrogen-bonding well depths, FENE r0, Debye-Hueckel).  The reference's own CUDA
// class keeps the oxDNA1 average-sequence well depths there (CUDADNAInteraction.cu:61-64); the
// input key gb300_reference_cuda_eps = true reproduces that choice.  The order-parameter
// helpers of the reference's FFS backend run liboxgb's kernels.
//
// Built by oracle/ref/Makefile (target cuda-gb300) against the reference headers; not part of
// liboxgb itself.

#include "CUDA/Interactions/CUDADNAInteraction.h"
#include "CUDA/Lists/CUDABaseList.h"
#include "Utilities/ConfigInfo.h"
#include "Utilities/oxDNAException.h"

#include "oxgb.h"

#include <map>
#include <string>

namespace {

void oxgb_check(int rc, const char *what) {
	if(rc != OXGB_OK) throw oxDNAException("%s failed: %s", what, oxgb_last_error());
}

double cubic_side() {
	const LR_vector L = CONFIG_INFO->box->box_sides();
	if(L.x != L.y || L.x != L.z) throw oxDNAException("the GB300 interaction supports cubic boxes only");
	return L.x;
}

// per-instance library state, keyed by object: the reference header fixes the class layout
struct State {
	oxgb_dna2 *h = nullptr;
	oxgb_dna2_settings s{};
	bool dna2 = false, ref_eps = false;
};
std::map<const CUDADNAInteraction *, State> g_state;

}  // namespace

CUDADNAInteraction::CUDADNAInteraction() {
	_use_debye_huckel = false;
	_use_oxDNA2_coaxial_stacking = false;
	_use_oxDNA2_FENE = false;
	_salt_concentration = 0.5f;
	_debye_huckel_half_charged_ends = true;
	_debye_huckel_prefactor = 0.0543f;
	_debye_huckel_lambdafactor = 0.3616455f;
	_debye_huckel_RC = _debye_huckel_RHIGH = _debye_huckel_B = _minus_kappa = 0.f;
	g_state[this] = State{};
}

CUDADNAInteraction::~CUDADNAInteraction() {
	auto it = g_state.find(this);
	if(it != g_state.end()) {
		if(it->second.h) oxgb_dna2_destroy(it->second.h);
		g_state.erase(it);
	}
}

void CUDADNAInteraction::get_settings(input_file &inp) {
	State &st = g_state[this];
	std::string inter_type;
	if(getInputString(&inp, "interaction_type", inter_type, 0) == KEY_FOUND && inter_type.compare("DNA2") == 0) {
		st.dna2 = true;
		_use_debye_huckel = true;
		_use_oxDNA2_coaxial_stacking = true;
		_use_oxDNA2_FENE = true;
		this->_grooving = true;
		float salt = 0.5f;
		getInputFloat(&inp, "salt_concentration", &salt, 1);
		_salt_concentration = salt;
		getInputBool(&inp, "dh_half_charged_ends", &_debye_huckel_half_charged_ends, 0);
		getInputFloat(&inp, "dh_lambda", &_debye_huckel_lambdafactor, 0);
		getInputFloat(&inp, "dh_strength", &_debye_huckel_prefactor, 0);
		getInputBool(&inp, "gb300_reference_cuda_eps", &st.ref_eps, 0);
	}
	DNAInteraction::get_settings(inp);
}

void CUDADNAInteraction::cuda_init(int N) {
	CUDABaseInteraction::cuda_init(N);
	DNAInteraction::init();
	State &st = g_state[this];
	if(!st.dna2) throw oxDNAException("the GB300 substitute implements interaction_type = DNA2");
	oxgb_dna2_default_settings(&st.s, _T, _salt_concentration);
	st.s.average = _average ? 1 : 0;
	st.s.hb_multiplier = _hb_multiplier;
	st.s.dh_half_charged_ends = _debye_huckel_half_charged_ends ? 1 : 0;
	st.s.dh_lambda = _debye_huckel_lambdafactor;
	st.s.dh_strength = _debye_huckel_prefactor;
	st.s.use_mbf = _use_mbf ? 1 : 0;
	st.s.mbf_fmax = _mbf_fmax;
	st.s.mbf_finf = _mbf_finf;
	st.s.reference_cuda_eps = st.ref_eps ? 1 : 0;
	if(!_average) throw oxDNAException("the GB300 substitute reads average-sequence parameters only (use the GB300DNA2 plugin)");
	oxgb_check(oxgb_dna2_create(&st.s, &st.h), "oxgb_dna2_create");
	double rc = 0.0;
	oxgb_check(oxgb_dna2_get_rcut(st.h, &rc), "oxgb_dna2_get_rcut");
	_rcut = rc;
	_sqr_rcut = rc * rc;
}

// CUDADNAInteraction::compute_forces (CUDADNAInteraction.cu:165-203): d_forces / d_torques arrive
// initialised (zeros or external forces) and are accumulated into.  The neighbour rows are read
// up to d_number_neighs, which the list keeps within its capacity (it refuses an overflow), so N
// bounds them.
void CUDADNAInteraction::compute_forces(CUDABaseList *lists, c_number4 *d_poss, GPU_quat *d_orientations, c_number4 *d_forces,
		c_number4 *d_torques, LR_bonds *d_bonds, CUDABox *d_box) {
	if(_use_edge) throw oxDNAException("the GB300 substitute does not implement use_edge");
	State &st = g_state[this];
	oxgb_check(oxgb_dna2_compute_forces(st.h, _N, cubic_side(), d_poss, d_orientations, d_forces, d_torques, d_bonds,
					   lists->d_matrix_neighs, lists->d_number_neighs, _N, 1, _N, nullptr),
			"oxgb_dna2_compute_forces");
}

void CUDADNAInteraction::_on_T_update() {
	DNAInteraction::_on_T_update();
	State &st = g_state[this];
	if(st.h) oxgb_check(oxgb_dna2_set_temperature(st.h, _T), "oxgb_dna2_set_temperature");
}

void CUDADNAInteraction::_init_strand_ends(LR_bonds *) {}

// the FFS backend's order parameters (CUDADNAInteraction.cu:205-218): the same kernels in liboxgb
// (the launch configuration is the library's own)
void CUDADNAInteraction::_hb_op_precalc(c_number4 *poss, GPU_quat *orientations, int *op_pairs1, int *op_pairs2, float *hb_energies,
		int n_threads, bool *, CUDA_kernel_cfg, CUDABox *) {
	oxgb_check(oxgb_dna2_hb_op_precalc(g_state[this].h, cubic_side(), poss, orientations, op_pairs1, op_pairs2, n_threads, hb_energies,
					   nullptr),
			"oxgb_dna2_hb_op_precalc");
}

void CUDADNAInteraction::_near_hb_op_precalc(c_number4 *poss, GPU_quat *orientations, int *op_pairs1, int *op_pairs2,
		bool *nearly_bonded_array, int n_threads, bool *, CUDA_kernel_cfg, CUDABox *) {
	oxgb_check(oxgb_dna2_near_hb_op_precalc(g_state[this].h, cubic_side(), poss, orientations, op_pairs1, op_pairs2, n_threads,
					   nearly_bonded_array, nullptr),
			"oxgb_dna2_near_hb_op_precalc");
}

void CUDADNAInteraction::_dist_op_precalc(c_number4 *poss, GPU_quat *orientations, int *op_pairs1, int *op_pairs2, c_number *op_dists,
		int n_threads, CUDA_kernel_cfg, CUDABox *) {
	static_assert(sizeof(c_number) == sizeof(float), "the order-parameter distances are FP32 (mixed or float backend)");
	oxgb_check(oxgb_dna2_dist_op_precalc(g_state[this].h, cubic_side(), poss, orientations, op_pairs1, op_pairs2, n_threads,
					   reinterpret_cast<float *>(op_dists), nullptr),
			"oxgb_dna2_dist_op_precalc");
}
