// Reference-side plugin over the oxgb C ABI: the reference's CUDA interaction and list
// interfaces implemented with liboxgb.so.
//
// CUDAGB300DNA2Interaction is a CUDABaseInteraction (src/CUDA/Interactions/CUDABaseInteraction.h:
// 20-64) and a DNA2Interaction (src/Interactions/DNA2Interaction.h), like the reference's
// CUDADNAInteraction (src/CUDA/Interactions/CUDADNAInteraction.h:18): the CPU class reads the
// input keys and initialises itself, then every force evaluation goes to
// oxgb_dna2_compute_forces on the reference's own device buffers.  GB300VerletList is a
// CUDABaseList (src/CUDA/Lists/CUDABaseList.h:25-62) over oxgb_verlet_*, publishing the
// column-major d_matrix_neighs / d_number_neighs the reference's kernels read.
//
// Built against the reference's headers and linked with -loxgb into CUDAGB300DNA2.so, it is
// loaded by PluginManager::get_interaction (src/PluginManagement/PluginManager.cpp:89-180) for
// interaction_type = GB300DNA2: CUDAInteractionFactory prefixes unknown names with CUDA and asks
// the plugin manager (src/CUDA/Interactions/CUDAInteractionFactory.cu:31-53).  Errors from the library become
// oxDNAException, as the reference reports its own.
//
//   nvcc -std=c++17 -shared -Xcompiler -fPIC -I<oxDNA>/src -I<oxDNA>/src/extern -DJSON_ENABLED \
//        -I<this repository>/include CUDAGB300DNA2Interaction.cu -L... -loxgb -o CUDAGB300DNA2.so

#include "CUDA/Interactions/CUDABaseInteraction.h"
#include "CUDA/Lists/CUDABaseList.h"
#include "Interactions/DNA2Interaction.h"
#include "Utilities/ConfigInfo.h"
#include "Utilities/oxDNAException.h"
#include "Utilities/parse_input/parse_input.h"

#include "oxgb.h"

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

namespace {

void oxgb_check(int rc, const char *what) {
	if(rc != OXGB_OK) throw oxDNAException("%s failed: %s", what, oxgb_last_error());
}

double cubic_side() {
	const LR_vector L = CONFIG_INFO->box->box_sides();
	if(L.x != L.y || L.x != L.z) throw oxDNAException("GB300DNA2 supports cubic boxes only");
	return L.x;
}

}  // namespace

// the Verlet list: CUDASimpleVerletList's keys, our build
class GB300VerletList: public CUDABaseList {
	oxgb_verlet *_h = nullptr;
	int _N = 0, _max_neigh = 0;
	c_number _skin = 0.05;
	bool _auto_opt = true;

public:
	void get_settings(input_file &inp) override {
		getInputNumber(&inp, "verlet_skin", &_skin, 1);
		getInputBool(&inp, "cells_auto_optimisation", &_auto_opt, 0);
	}

	void init(int N, c_number rcut, CUDABox *h_cuda_box, CUDABox *d_cuda_box) override {
		CUDABaseList::init(N, rcut, h_cuda_box, d_cuda_box);
		_N = N;
		oxgb_check(oxgb_verlet_create(N, cubic_side(), rcut, _skin, _auto_opt ? 1 : 0, 0, &_h), "oxgb_verlet_create");
		int n_side = 0;
		oxgb_check(oxgb_verlet_buffers(_h, &d_matrix_neighs, &d_number_neighs, &_max_neigh, &n_side), "oxgb_verlet_buffers");
	}

	void update(c_number4 *poss, c_number4 *list_poss, LR_bonds *bonds) override {
		oxgb_check(oxgb_verlet_update(_h, poss, list_poss, bonds, nullptr), "oxgb_verlet_update");
		// like the reference's overflow check, this synchronises
		oxgb_check(oxgb_verlet_status(_h), "Verlet list");
	}

	void clean() override {
		if(_h) oxgb_verlet_destroy(_h);
		_h = nullptr;
		d_matrix_neighs = d_number_neighs = nullptr;
	}

	int max_neigh() const { return _max_neigh; }

	~GB300VerletList() override { clean(); }
};

// the interaction: DNA2Interaction's keys and initialisation, our kernels
class CUDAGB300DNA2Interaction: public CUDABaseInteraction, public DNA2Interaction {
	oxgb_dna2 *_h = nullptr;
	oxgb_dna2_settings _s{};
	// gb300_dump_list: a file that receives the first neighbour list the backend hands over
	// (whatever CUDABaseList built it) with the positions it was built from, so that a test can
	// compare the reference's own list with the library's
	std::string _dump_list;
	bool _dumped = false;

	void _dump(CUDABaseList *lists, const c_number4 *d_poss) {
		if(cudaDeviceSynchronize() != cudaSuccess) throw oxDNAException("gb300_dump_list: CUDA error");
		const int N = _N;
		std::vector<int> cnt(N);
		cudaMemcpy(cnt.data(), lists->d_number_neighs, sizeof(int) * N, cudaMemcpyDeviceToHost);
		const int maxc = N > 0 ? *std::max_element(cnt.begin(), cnt.end()) : 0;
		std::vector<int> rows((size_t) maxc * N);  // column-major: entry k of i at [k N + i]
		if(maxc > 0) cudaMemcpy(rows.data(), lists->d_matrix_neighs, sizeof(int) * rows.size(), cudaMemcpyDeviceToHost);
		std::vector<float> pos((size_t) 4 * N);
		cudaMemcpy(pos.data(), d_poss, sizeof(float) * pos.size(), cudaMemcpyDeviceToHost);
		if(cudaGetLastError() != cudaSuccess) throw oxDNAException("gb300_dump_list: CUDA error");
		FILE *f = std::fopen(_dump_list.c_str(), "wb");
		if(!f) throw oxDNAException("gb300_dump_list: cannot open %s", _dump_list.c_str());
		const int head[2] = {N, maxc};
		std::fwrite(head, sizeof(int), 2, f);
		std::fwrite(cnt.data(), sizeof(int), cnt.size(), f);
		std::fwrite(rows.data(), sizeof(int), rows.size(), f);
		std::fwrite(pos.data(), sizeof(float), pos.size(), f);
		std::fclose(f);
	}

	// the oxgb settings from what the CPU class read and derived
	void _fill_settings() {
		oxgb_dna2_default_settings(&_s, _T, _salt_concentration);
		_s.average = _average ? 1 : 0;
		_s.hb_multiplier = _hb_multiplier;
		_s.dh_half_charged_ends = _debye_huckel_half_charged_ends ? 1 : 0;
		_s.dh_lambda = _debye_huckel_lambdafactor;
		_s.dh_strength = _debye_huckel_prefactor;
		_s.use_mbf = _use_mbf ? 1 : 0;
		_s.mbf_fmax = _mbf_fmax;
		_s.mbf_finf = _mbf_finf;
		if(!_average) {
			// the sequence-dependent file, read with the same keys as DNAInteraction::init
			input_file seq_file;
			seq_file.init_from_filename(_seq_filename.c_str());
			if(seq_file.state == ERROR) throw oxDNAException("cannot read sequence-dependence file '%s'", _seq_filename.c_str());
			float v;
			getInputFloat(&seq_file, "STCK_FACT_EPS", &v, 1);
			_s.seq_stck_fact_eps = v;
			const char bases[4] = {'A', 'G', 'C', 'T'};
			for(int i = 0; i < 4; i++)
				for(int j = 0; j < 4; j++) {
					const std::string key = std::string("STCK_") + bases[i] + "_" + bases[j];
					getInputFloat(&seq_file, key.c_str(), &v, 1);
					_s.seq_stck[i][j] = v;
				}
			if(getInputFloat(&seq_file, "HYDR_A_T", &v, 0) == KEY_NOT_FOUND) getInputFloat(&seq_file, "HYDR_T_A", &v, 1);
			_s.seq_hydr_at = v;
			if(getInputFloat(&seq_file, "HYDR_G_C", &v, 0) == KEY_NOT_FOUND) getInputFloat(&seq_file, "HYDR_C_G", &v, 1);
			_s.seq_hydr_gc = v;
		}
	}

public:
	void get_settings(input_file &inp) override {
		DNA2Interaction::get_settings(inp);
		getInputString(&inp, "gb300_dump_list", _dump_list, 0);
	}

	void cuda_init(int N) override {
		CUDABaseInteraction::cuda_init(N);
		DNA2Interaction::init();
		_fill_settings();
		oxgb_check(oxgb_dna2_create(&_s, &_h), "oxgb_dna2_create");
	}

	c_number get_cuda_rcut() override {
		double rc = 0.0;
		oxgb_check(oxgb_dna2_get_rcut(_h, &rc), "oxgb_dna2_get_rcut");
		return (c_number) rc;
	}

	// CUDADNAInteraction::compute_forces (CUDADNAInteraction.cu:165-203): d_forces / d_torques
	// arrive initialised (zeros or external forces) and are accumulated into
	void compute_forces(CUDABaseList *lists, c_number4 *d_poss, GPU_quat *d_orientations, c_number4 *d_forces, c_number4 *d_torques,
			LR_bonds *d_bonds, CUDABox *d_box) override {
		if(!_dump_list.empty() && !_dumped) {
			_dump(lists, d_poss);
			_dumped = true;
		}
		// the rows are read up to d_number_neighs, which the list keeps within its capacity
		oxgb_check(oxgb_dna2_compute_forces(_h, _N, cubic_side(), d_poss, d_orientations, d_forces, d_torques, d_bonds,
						   lists->d_matrix_neighs, lists->d_number_neighs, _N, 1, _N, nullptr),
				"oxgb_dna2_compute_forces");
	}

	// the FFS backend's order parameters (CUDABaseInteraction.h:61-63, CUDADNAInteraction.cu:205-218)
	void _hb_op_precalc(c_number4 *poss, GPU_quat *orientations, int *op_pairs1, int *op_pairs2, float *hb_energies, int n_threads,
			bool *, CUDA_kernel_cfg, CUDABox *) override {
		oxgb_check(oxgb_dna2_hb_op_precalc(_h, cubic_side(), poss, orientations, op_pairs1, op_pairs2, n_threads, hb_energies, nullptr),
				"oxgb_dna2_hb_op_precalc");
	}

	void _near_hb_op_precalc(c_number4 *poss, GPU_quat *orientations, int *op_pairs1, int *op_pairs2, bool *nearly_bonded_array,
			int n_threads, bool *, CUDA_kernel_cfg, CUDABox *) override {
		oxgb_check(oxgb_dna2_near_hb_op_precalc(_h, cubic_side(), poss, orientations, op_pairs1, op_pairs2, n_threads,
						   nearly_bonded_array, nullptr),
				"oxgb_dna2_near_hb_op_precalc");
	}

	void _dist_op_precalc(c_number4 *poss, GPU_quat *orientations, int *op_pairs1, int *op_pairs2, c_number *op_dists, int n_threads,
			CUDA_kernel_cfg, CUDABox *) override {
		static_assert(sizeof(c_number) == sizeof(float), "the order-parameter distances are FP32 (mixed or float backend)");
		oxgb_check(oxgb_dna2_dist_op_precalc(_h, cubic_side(), poss, orientations, op_pairs1, op_pairs2, n_threads,
						   reinterpret_cast<float *>(op_dists), nullptr),
				"oxgb_dna2_dist_op_precalc");
	}

	~CUDAGB300DNA2Interaction() override {
		if(_h) oxgb_dna2_destroy(_h);
	}

protected:
	void _on_T_update() override {
		DNA2Interaction::_on_T_update();
		if(_h) oxgb_check(oxgb_dna2_set_temperature(_h, _T), "oxgb_dna2_set_temperature");
	}
};

// PluginManager::_get_entry_point (PluginManager.cpp:123-137) looks up make_<name>: the CUDA
// backend asks for CUDAGB300DNA2 (this class), SimBackend's InteractionFactory for GB300DNA2 (the
// CPU-side interaction it keeps for output and analysis, the plain DNA2 class); the library is
// installed under both names.
extern "C" BaseInteraction *make_CUDAGB300DNA2() { return new CUDAGB300DNA2Interaction(); }
extern "C" BaseInteraction *make_GB300DNA2() { return new DNA2Interaction(); }

// CUDAListFactory (src/CUDA/Lists/CUDAListFactory.cu:15-30) has no plugin route; a one-line
// branch there (CUDA_list = gb300) calls this
extern "C" CUDABaseList *make_GB300VerletList() { return new GB300VerletList(); }
