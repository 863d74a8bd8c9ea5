// Verlet-list build that allocates no device memory.
//
// oxgb_verlet_build_noalloc runs the same kernels as oxgb_verlet_update (lists.cu): counting
// sort into cells, then one warp per nucleotide over the 27 neighbouring cells.  Their scratch
// (cell of every nucleotide, the cell segments, the per-cell counts, starts and cursors, the
// scan tiles, the status word) lives in the file-scope device arrays below instead of buffers
// owned by an oxgb_verlet handle.  The caller owns every output buffer.
//
// Limits: N <= OXGB_NOALLOC_MAX_N nucleotides and at most OXGB_NOALLOC_MAX_CELLS cells (the
// cell grid follows the same sizing rule as the handle-based list); larger requests are
// rejected before anything is launched.  The scratch is ~1.2 MB of device memory per device,
// set aside when the module is loaded.
//
// The host finds the scratch with cudaGetSymbolAddress, once per device (with that device
// current), and checks on every call that the module was not reloaded since; the first call
// on a device may load the module, so it should come before any stream capture.  Calls on one device share the scratch: two calls
// that overlap in time (different streams or threads) race and must be serialised by the
// caller.  Each call clears what must start at zero (the status word; the cell counts are
// zeroed by the build itself), so consecutive calls never see each other's leftovers.
#include "kernels.h"
#include "params.h"

#include <mutex>
#include <string>

namespace oxgb {

int set_error(int code, const std::string &msg);
int list_status_code(int st);
std::string list_status_message(int st);

constexpr int NOALLOC_MAX_N = OXGB_NOALLOC_MAX_N;
constexpr int NOALLOC_MAX_CELLS = OXGB_NOALLOC_MAX_CELLS;
constexpr int NOALLOC_TILES = (NOALLOC_MAX_CELLS + 2047) / 2048 + 1;  // scan_tiles(max) + 1

static __device__ __align__(256) int g_cell_of[NOALLOC_MAX_N];
static __device__ __align__(256) int g_cell_tmp[NOALLOC_MAX_N];
static __device__ __align__(256) int g_cell_list[NOALLOC_MAX_N];
static __device__ __align__(256) int g_cell_count[NOALLOC_MAX_CELLS];
static __device__ __align__(256) int g_cell_start[NOALLOC_MAX_CELLS + 1];
static __device__ __align__(256) int g_cell_cursor[NOALLOC_MAX_CELLS];
static __device__ __align__(256) int g_scan_part[NOALLOC_TILES];
static __device__ __align__(256) int g_status[2];  // status word, rebuild flag

struct Scratch {
	int *cell_of, *cell_tmp, *cell_list, *cell_count, *cell_start, *cell_cursor, *scan_part, *status;
};

static std::mutex g_scratch_mutex;
static Scratch g_scratch[64];
static bool g_scratch_ok[64];

// device addresses of the scratch arrays on the current device: looked up together once per
// device; every later call looks up the status word's address alone (cheap once the module is
// loaded) and redoes the whole lookup if it moved, which happens when a device reset or a new
// primary context has loaded the module again
static cudaError_t scratch_of_current_device(Scratch &out) {
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if(e != cudaSuccess) return e;
	if(dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
	std::lock_guard<std::mutex> lock(g_scratch_mutex);
	if(g_scratch_ok[dev]) {
		void *p = nullptr;
		if((e = cudaGetSymbolAddress(&p, g_status)) != cudaSuccess) return e;
		if((int *) p != g_scratch[dev].status) g_scratch_ok[dev] = false;
	}
	if(!g_scratch_ok[dev]) {
		Scratch s{};
		void *p = nullptr;
		if((e = cudaGetSymbolAddress(&p, g_cell_of)) != cudaSuccess) return e;
		s.cell_of = (int *) p;
		if((e = cudaGetSymbolAddress(&p, g_cell_tmp)) != cudaSuccess) return e;
		s.cell_tmp = (int *) p;
		if((e = cudaGetSymbolAddress(&p, g_cell_list)) != cudaSuccess) return e;
		s.cell_list = (int *) p;
		if((e = cudaGetSymbolAddress(&p, g_cell_count)) != cudaSuccess) return e;
		s.cell_count = (int *) p;
		if((e = cudaGetSymbolAddress(&p, g_cell_start)) != cudaSuccess) return e;
		s.cell_start = (int *) p;
		if((e = cudaGetSymbolAddress(&p, g_cell_cursor)) != cudaSuccess) return e;
		s.cell_cursor = (int *) p;
		if((e = cudaGetSymbolAddress(&p, g_scan_part)) != cudaSuccess) return e;
		s.scan_part = (int *) p;
		if((e = cudaGetSymbolAddress(&p, g_status)) != cudaSuccess) return e;
		s.status = (int *) p;
		g_scratch[dev] = s;
		g_scratch_ok[dev] = true;
	}
	out = g_scratch[dev];
	return cudaSuccess;
}

}  // namespace oxgb

using namespace oxgb;

extern "C" int oxgb_verlet_build_noalloc(int N, double box, double rcut, double skin, int cells_auto_optimisation,
		const void *d_poss, void *d_list_poss, const void *d_bonds, int *d_matrix_neighs, int *d_number_neighs,
		int max_neigh, void *stream) {
	if(N <= 0 || !(box > 0) || !(rcut > 0) || skin < 0 || max_neigh <= 0)
		return set_error(OXGB_E_INVALID, "invalid argument");
	if(!d_poss || !d_list_poss || !d_bonds || !d_matrix_neighs || !d_number_neighs)
		return set_error(OXGB_E_INVALID, "null device buffer");
	if(N > NOALLOC_MAX_N)
		return set_error(OXGB_E_INVALID, "oxgb_verlet_build_noalloc: N = " + std::to_string(N) + " exceeds its limit of " +
				std::to_string(NOALLOC_MAX_N) + " nucleotides (use oxgb_verlet_create / oxgb_verlet_update)");
	const float rverlet = (float) rcut + 2.f * (float) skin;
	const int n_side = cells_per_side(N, (float) box, rverlet, cells_auto_optimisation != 0);
	const long long n_cells = (long long) n_side * n_side * n_side;
	if(n_cells > NOALLOC_MAX_CELLS)
		return set_error(OXGB_E_INVALID, "oxgb_verlet_build_noalloc: " + std::to_string(n_cells) + " cells exceed its limit of " +
				std::to_string(NOALLOC_MAX_CELLS) + " (use oxgb_verlet_create / oxgb_verlet_update)");
	Scratch sc;
	cudaError_t e = scratch_of_current_device(sc);
	if(e != cudaSuccess) return set_error(OXGB_E_CUDA, std::string("scratch lookup: ") + cudaGetErrorString(e));
	cudaStream_t s = (cudaStream_t) stream;
	// status word and rebuild flag start at zero on every call
	e = cudaMemsetAsync(sc.status, 0, 2 * sizeof(int), s);
	if(e != cudaSuccess) return set_error(OXGB_E_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
	ListArgs a{};
	a.N = N;
	a.pos = (const float4 *) d_poss;
	a.box = (float) box;
	a.rverlet2 = rverlet * rverlet;
	a.n_side = n_side;
	a.bonds = (const int2 *) d_bonds;
	a.cell_of = sc.cell_of;
	a.cell_count = sc.cell_count;
	a.cell_start = sc.cell_start;
	a.cell_cursor = sc.cell_cursor;
	a.cell_list = sc.cell_list;
	a.cell_tmp = sc.cell_tmp;
	a.scan_part = sc.scan_part;
	a.nb = d_matrix_neighs;
	a.nnb = d_number_neighs;
	a.max_nb = max_neigh;
	a.list_pos = (float4 *) d_list_poss;
	a.status = sc.status;
	a.flag = sc.status + 1;
	a.check_flag = 0;
	a.rebuilds = nullptr;
	a.col_major = 1;
	e = launch_list_build(a, s);
	if(e != cudaSuccess) return set_error(OXGB_E_CUDA, std::string("list build: ") + cudaGetErrorString(e));
	int st = 0;
	e = cudaMemcpyAsync(&st, sc.status, sizeof(int), cudaMemcpyDeviceToHost, s);
	if(e == cudaSuccess) e = cudaStreamSynchronize(s);
	if(e != cudaSuccess) return set_error(OXGB_E_CUDA, std::string("status read: ") + cudaGetErrorString(e));
	if(st) return set_error(list_status_code(st), list_status_message(st));
	return OXGB_OK;
}
