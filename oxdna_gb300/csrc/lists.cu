// Cell-binned Verlet list build.
//
// Replaces simple_fill_cells / simple_update_neigh_list (src/CUDA/Lists/CUDA_simple_verlet.cuh:
// 14-95) and the host control of CUDASimpleVerletList::update (src/CUDA/Lists/
// CUDASimpleVerletList.cu:231-289).  Cells are filled by a counting sort (count, scan,
// scatter, then each cell's short segment ordered by index), so there is no per-cell capacity
// to overflow and the neighbour order is deterministic run to run.  The geometry is the
// reference's fp32 geometry: cell coordinate ((x/L - floor(x/L)) * (1 - FLT_EPSILON)) * n and
// minimum-image squared distance against r_verlet^2, with IEEE division and the fused
// multiply-adds written out, so that oracle/dna2_oracle.c (oxo_verlet_f32) reproduces the
// pair set and the cell of every particle bit for bit.
#include "kernels.h"

#include <cfloat>

namespace oxgb {

__device__ __forceinline__ int cell_coord(float x, float L, int n) {
	const float s = __fdiv_rn(x, L);
	return (int) (((s - floorf(s)) * (1.f - FLT_EPSILON)) * (float) n);
}

__device__ __forceinline__ float sqr_min_image(float4 a, float4 b, float L) {
	float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
	dx = __fmaf_rn(-rintf(__fdiv_rn(dx, L)), L, dx);
	dy = __fmaf_rn(-rintf(__fdiv_rn(dy, L)), L, dy);
	dz = __fmaf_rn(-rintf(__fdiv_rn(dz, L)), L, dz);
	return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

#define SKIP_IF_FRESH(a) \
	if((a).check_flag && *(a).flag == 0) return

__global__ void k_zero_counts(ListArgs a, int n_cells) {
	SKIP_IF_FRESH(a);
	for(int c = blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += gridDim.x * blockDim.x) a.cell_count[c] = 0;
}

__global__ void k_cell_count(ListArgs a) {
	SKIP_IF_FRESH(a);
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= a.N) return;
	const float4 r = a.pos[i];
	if(!(fabsf(r.x) < 1e7f && fabsf(r.y) < 1e7f && fabsf(r.z) < 1e7f)) {
		atomicOr(a.status, OXGB_ERR_NONFINITE);
		a.cell_of[i] = 0;
		atomicAdd(a.cell_count, 1);
		return;
	}
	const int n = a.n_side;
	int cx = cell_coord(r.x, a.box, n), cy = cell_coord(r.y, a.box, n), cz = cell_coord(r.z, a.box, n);
	if(cx < 0 || cx >= n || cy < 0 || cy >= n || cz < 0 || cz >= n) {
		atomicOr(a.status, OXGB_ERR_CELL);
		cx = min(max(cx, 0), n - 1);
		cy = min(max(cy, 0), n - 1);
		cz = min(max(cz, 0), n - 1);
	}
	const int c = (cz * n + cy) * n + cx;
	a.cell_of[i] = c;
	atomicAdd(a.cell_count + c, 1);
}

// exclusive scan of the cell counts by one block; each thread owns a contiguous chunk
__global__ void __launch_bounds__(1024) k_cell_scan(ListArgs a, int n_cells) {
	SKIP_IF_FRESH(a);
	__shared__ int part[1024];
	const int t = threadIdx.x;
	const int chunk = (n_cells + blockDim.x - 1) / blockDim.x;
	const int lo = t * chunk, hi = min(lo + chunk, n_cells);
	int s = 0;
	for(int c = lo; c < hi; c++) s += a.cell_count[c];
	part[t] = s;
	__syncthreads();
	for(int off = 1; off < blockDim.x; off <<= 1) {
		const int v = (t >= off) ? part[t - off] : 0;
		__syncthreads();
		part[t] += v;
		__syncthreads();
	}
	int run = part[t] - s;
	for(int c = lo; c < hi; c++) {
		a.cell_start[c] = run;
		a.cell_cursor[c] = run;
		run += a.cell_count[c];
	}
	if(t == blockDim.x - 1) a.cell_start[n_cells] = part[t];
}

__global__ void k_cell_scatter(ListArgs a) {
	SKIP_IF_FRESH(a);
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= a.N) return;
	const int slot = atomicAdd(a.cell_cursor + a.cell_of[i], 1);
	a.cell_list[slot] = i;
}

// order each cell's segment by particle index (segments hold a handful of particles)
__global__ void k_cell_order(ListArgs a, int n_cells) {
	SKIP_IF_FRESH(a);
	const int c = blockIdx.x * blockDim.x + threadIdx.x;
	if(c >= n_cells) return;
	const int b = a.cell_start[c], e = a.cell_start[c + 1];
	for(int k = b + 1; k < e; k++) {
		const int v = a.cell_list[k];
		int m = k - 1;
		while(m >= b && a.cell_list[m] > v) {
			a.cell_list[m + 1] = a.cell_list[m];
			m--;
		}
		a.cell_list[m + 1] = v;
	}
}

// minimum-image separation vector (the reference's fp32 geometry, explicit fused multiply-adds)
__device__ __forceinline__ float3 min_image_vec(float4 a, float4 b, float L) {
	float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
	dx = __fmaf_rn(-rintf(__fdiv_rn(dx, L)), L, dx);
	dy = __fmaf_rn(-rintf(__fdiv_rn(dy, L)), L, dy);
	dz = __fmaf_rn(-rintf(__fdiv_rn(dz, L)), L, dz);
	return make_float3(dx, dy, dz);
}

__global__ void k_neighbours(ListArgs a) {
	SKIP_IF_FRESH(a);
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= a.N) return;
	const float4 r = a.pos[i];
	const int2 b = a.bonds[i];
	const int n = a.n_side;
	const int c = a.cell_of[i];
	const int cx = c % n, cy = (c / n) % n, cz = c / (n * n);
	const bool terms = a.ev_nb != nullptr;
	float4 a1i = make_float4(0.f, 0.f, 0.f, 0.f), bki = a1i;
	if(terms) {
		a1i = a.fa1[i];
		bki = a.fback[i];
	}
	const long long N = a.N;
	int cnt = 0, nev = 0, nbase = 0, nstk = 0;
	for(int dz = -1; dz <= 1; dz++) {
		const int z = (cz + dz + n) % n;
		for(int dy = -1; dy <= 1; dy++) {
			const int y = (cy + dy + n) % n;
			for(int dx = -1; dx <= 1; dx++) {
				const int x = (cx + dx + n) % n;
				const int cc = (z * n + y) * n + x;
				const int e = a.cell_start[cc + 1];
				for(int k = a.cell_start[cc]; k < e; k++) {
					const int j = a.cell_list[k];
					if(j == i || j == b.x || j == b.y) continue;
					const float4 rj = a.pos[j];
					const float d2 = sqr_min_image(r, rj, a.box);
					if(d2 < a.rverlet2) {
						if(cnt < a.max_nb) {
							if(a.col_major) a.nb[(long long) cnt * N + i] = j;
							else a.nb[(long long) i * a.max_nb + cnt] = j;
						}
						cnt++;
						if(terms && d2 < a.ev_r2) {
							if(nev < a.ev_cap) a.ev_nb[(long long) nev * N + i] = j;
							nev++;
							const float3 d = min_image_vec(r, rj, a.box);
							const float4 a1j = a.fa1[j];
							// base sites at 0.4 a1, stacking sites at 0.34 a1 from the centres
							const float bx = d.x + 0.4f * (a1j.x - a1i.x), by = d.y + 0.4f * (a1j.y - a1i.y),
									bz = d.z + 0.4f * (a1j.z - a1i.z);
							if(bx * bx + by * by + bz * bz < a.base_r2) {
								if(nbase < a.base_cap) a.base_nb[(long long) nbase * N + i] = j;
								nbase++;
							}
							const float sx = d.x + 0.34f * (a1j.x - a1i.x), sy = d.y + 0.34f * (a1j.y - a1i.y),
									sz = d.z + 0.34f * (a1j.z - a1i.z);
							if(sx * sx + sy * sy + sz * sz < a.stk_r2) {
								if(nstk < a.stk_cap) a.stk_nb[(long long) nstk * N + i] = j;
								nstk++;
							}
						}
					}
				}
			}
		}
	}
	if(cnt > a.max_nb) atomicOr(a.status, OXGB_ERR_NEIGH_OVERFLOW);
	a.nnb[i] = cnt;
	a.list_pos[i] = r;
	if(terms) {
		if(nev > a.ev_cap || nbase > a.base_cap || nstk > a.stk_cap) atomicOr(a.status, OXGB_ERR_NEIGH_OVERFLOW);
		a.ev_n[i] = nev;
		a.base_n[i] = nbase;
		a.stk_n[i] = nstk;
		a.list_a1[i] = a1i;
		a.list_back[i] = bki;
	}
}

// runs after every other list kernel: counts the build and clears the request
__global__ void k_list_done(ListArgs a) {
	if(threadIdx.x != 0 || blockIdx.x != 0) return;
	if(a.check_flag && *a.flag == 0) return;
	if(a.rebuilds) *a.rebuilds += 1;
	*a.flag = 0;
}

cudaError_t launch_list_build(const ListArgs &a, cudaStream_t s) {
	const int n_cells = a.n_side * a.n_side * a.n_side;
	const int tpb = 256;
	const int gp = (a.N + tpb - 1) / tpb;
	k_zero_counts<<<(n_cells + tpb - 1) / tpb, tpb, 0, s>>>(a, n_cells);
	k_cell_count<<<gp, tpb, 0, s>>>(a);
	k_cell_scan<<<1, 1024, 0, s>>>(a, n_cells);
	k_cell_scatter<<<gp, tpb, 0, s>>>(a);
	k_cell_order<<<(n_cells + tpb - 1) / tpb, tpb, 0, s>>>(a, n_cells);
	k_neighbours<<<gp, tpb, 0, s>>>(a);
	k_list_done<<<1, 32, 0, s>>>(a);
	return cudaGetLastError();
}

}  // namespace oxgb
