// Link-time substitute for the reference's CUDASimpleVerletList (declared in
// src/CUDA/Lists/CUDASimpleVerletList.h, which this file includes unchanged): a reference program
// linked with this object instead of src/CUDA/Lists/CUDASimpleVerletList.cu builds its Verlet
// lists with liboxgb (oxgb_verlet_*: counting sort into cells, one warp per particle over the 27
// neighbouring cells), selected by the reference's own key CUDA_list = verlet through its
// unmodified CUDAListFactory (src/CUDA/Lists/CUDAListFactory.cu:15-30).  The published arrays
// are the reference's: d_matrix_neighs column-major (element k of particle i at [k N + i]) and
// d_number_neighs, with the same pairs (the reference's FP32 cell and minimum-image geometry).
//
// The constructor, the input keys and the release of a derived list's own buffers keep the
// reference's behaviour, so CUDABinVerletList (which derives from this class and allocates its
// cells itself) still works.  use_edge (the edge list of the pair-parallel kernels) is not
// provided.
//
// Built by oracle/ref/Makefile (target cuda-gb300) against the reference headers; not part of
// liboxgb itself.

#include "CUDA/Lists/CUDASimpleVerletList.h"
#include "Utilities/ConfigInfo.h"
#include "Utilities/oxDNAException.h"
#include "Boxes/BaseBox.h"

#include "oxgb.h"

#include <map>

namespace {

void oxgb_check(int rc, const char *what) {
	if(rc != OXGB_OK) throw oxDNAException("%s failed: %s", what, oxgb_last_error());
}

// the library handle of each list object (the reference header fixes the class layout)
std::map<const CUDASimpleVerletList *, oxgb_verlet *> g_handles;

}  // namespace

CUDASimpleVerletList::CUDASimpleVerletList() {
	_cells_kernel_cfg.threads_per_block = 0;
	_use_edge = false;
	_N_cells = _old_N_cells = N_edges = -1;
}

CUDASimpleVerletList::~CUDASimpleVerletList() {
	auto it = g_handles.find(this);
	if(it != g_handles.end()) {
		oxgb_verlet_destroy(it->second);
		g_handles.erase(it);
	}
}

void CUDASimpleVerletList::clean() {
	auto it = g_handles.find(this);
	if(it != g_handles.end()) {
		// the rows and counts belong to the library's handle
		oxgb_verlet_destroy(it->second);
		g_handles.erase(it);
		d_matrix_neighs = d_number_neighs = nullptr;
		return;
	}
	// a derived list (CUDABinVerletList) allocated these itself
	if(_d_cells != nullptr) {
		cudaFree(_d_cells);
		cudaFree(_d_counters_cells);
		cudaFree(d_matrix_neighs);
		cudaFree(d_number_neighs);
		cudaFreeHost(_d_cell_overflow);
		_d_cells = nullptr;
	}
}

void CUDASimpleVerletList::get_settings(input_file &inp) {
	getInputBool(&inp, "cells_auto_optimisation", &_auto_optimisation, 0);
	getInputBool(&inp, "print_problematic_ids", &_print_problematic_ids, 0);
	getInputNumber(&inp, "verlet_skin", &_verlet_skin, 1);
	getInputNumber(&inp, "max_density_multiplier", &_max_density_multiplier, 0);
	getInputBool(&inp, "use_edge", &_use_edge, 0);
	_sqr_verlet_skin = _verlet_skin * _verlet_skin;
}

void CUDASimpleVerletList::init(int N, c_number rcut, CUDABox *h_cuda_box, CUDABox *d_cuda_box) {
	CUDABaseList::init(N, rcut, h_cuda_box, d_cuda_box);
	if(_use_edge) throw oxDNAException("the GB300 Verlet list does not build the edge list (use_edge)");
	const LR_vector L = CONFIG_INFO->box->box_sides();
	if(L.x != L.y || L.x != L.z) throw oxDNAException("the GB300 Verlet list supports cubic boxes only");
	clean();
	oxgb_verlet *h = nullptr;
	oxgb_check(oxgb_verlet_create(N, L.x, rcut, _verlet_skin, _auto_optimisation ? 1 : 0, 0, &h), "oxgb_verlet_create");
	g_handles[this] = h;
	int n_side = 0;
	oxgb_check(oxgb_verlet_buffers(h, &d_matrix_neighs, &d_number_neighs, &_max_neigh, &n_side), "oxgb_verlet_buffers");
	_N_cells_side[0] = _N_cells_side[1] = _N_cells_side[2] = n_side;
	_N_cells = n_side * n_side * n_side;
	_sqr_rverlet = (rcut + 2 * _verlet_skin) * (rcut + 2 * _verlet_skin);
}

// CUDASimpleVerletList::update (src/CUDA/Lists/CUDASimpleVerletList.cu:231-289): like the
// reference's overflow check, this synchronises and throws on an overflowing row
void CUDASimpleVerletList::update(c_number4 *poss, c_number4 *list_poss, LR_bonds *bonds) {
	auto it = g_handles.find(this);
	if(it == g_handles.end()) throw oxDNAException("the GB300 Verlet list was not initialised");
	oxgb_check(oxgb_verlet_update(it->second, poss, list_poss, bonds, nullptr), "oxgb_verlet_update");
	oxgb_check(oxgb_verlet_status(it->second), "the GB300 Verlet list");
	// the rows' capacity may have grown
	int n_side = 0;
	oxgb_check(oxgb_verlet_buffers(it->second, &d_matrix_neighs, &d_number_neighs, &_max_neigh, &n_side), "oxgb_verlet_buffers");
}

// the reference's cell-sizing helpers: the library sizes its own cells
std::vector<int> CUDASimpleVerletList::is_large(c_number4 *) { return std::vector<int>(); }

void CUDASimpleVerletList::_compute_N_cells_side(int N_cells_side[3], number) {
	for(int k = 0; k < 3; k++) N_cells_side[k] = _N_cells_side[k];
}

int CUDASimpleVerletList::_largest_N_in_cells(c_number4 *, c_number) {
	throw oxDNAException("the GB300 Verlet list sizes its cells itself");
}

void CUDASimpleVerletList::_init_cells(c_number4 *) {}
