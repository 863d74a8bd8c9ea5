// Cell-binned Verlet list build.
//
// Replaces simple_fill_cells / simple_update_neigh_list (src/CUDA/Lists/CUDA_simple_verlet.cuh:
// 14-95) and the host control of CUDASimpleVerletList::update (src/CUDA/Lists/
// CUDASimpleVerletList.cu:231-289).  Cells are filled by a counting sort (count, scan,
// scatter, then each particle placed by the rank of its caller's index within its cell), so there is no
// per-cell capacity to overflow and the neighbour order is deterministic run to run.  The geometry is the
// reference's fp32 geometry: cell coordinate ((x/L - floor(x/L)) * (1 - FLT_EPSILON)) * n and
// minimum-image squared distance against r_verlet^2, with IEEE division and the fused
// multiply-adds written out, so that oracle/dna2_oracle.c (oxo_verlet_f32) reproduces the
// pair set and the cell of every particle bit for bit.
#include "kernels.h"

#include <cfloat>
#include <climits>

namespace oxgb {

__device__ __forceinline__ int cell_coord(float x, float L, int n) {
	const float s = __fdiv_rn(x, L);
	return (int) (((s - floorf(s)) * (1.f - FLT_EPSILON)) * (float) n);
}

// Squared minimum-image separation in the reference's FP32 geometry (CUDABox.h:42-60: d - rint(d /
// L) L per axis, then the sum of squares as fused multiply-adds), with the image picked by a
// product with 1 / L rounded by the 1.5 * 2^23 addition instead of the IEEE quotient: the two
// images differ only where d / L sits within an ulp of a half-integer, i.e. |d| ~ L / 2, where both
// images leave a separation of ~L / 2 > the Verlet radius (L > 2 r_verlet).  So every pair that is
// listed, and its d^2, are exactly those of the quotient form (listed pairs have |d| < r_verlet,
// image 0 either way).
__device__ __forceinline__ float sqr_min_image_inv(float4 a, float4 b, float L, float inv) {
	float d[3] = {b.x - a.x, b.y - a.y, b.z - a.z};
#pragma unroll
	for(int k = 0; k < 3; k++) d[k] = __fmaf_rn(-__fsub_rn(__fmaf_rn(d[k], inv, 12582912.f), 12582912.f), L, d[k]);
	return __fmaf_rn(d[2], d[2], __fmaf_rn(d[1], d[1], __fmul_rn(d[0], d[0])));
}

#define SKIP_IF_FRESH(a) \
	if((a).check_flag && *(a).flag == 0) return

// the scan kernels' copy for the Hilbert order runs only in the builds that sort
#define SKIP_IF_NO_SORT(a) \
	if((a).hilbert_pass && !((a).sort_every > 0 && (a).id && ((a).rebuilds ? *(a).rebuilds : 0ull) % (unsigned long long) (a).sort_every == 0ull)) \
		return

// geometry of system s: box side, r_verlet^2, cells per side, first cell, bound of the
// Debye-Hueckel rows (squared, on backbone sites)
struct CellGeo {
	float box, rv2;
	int n, cell0;
	float dh2;
};

__device__ __forceinline__ int sys_of(const ListArgs &a, int i) { return a.sys ? a.sys[i] : 0; }

__device__ __forceinline__ CellGeo cell_geo(const ListArgs &a, int s) {
	if(!a.sys) return CellGeo{a.box, a.rverlet2, a.n_side, 0, a.dh_r2};
	return CellGeo{a.sys_box[s], a.sys_rv2[s], a.sys_nside[s], a.sys_cell0[s], a.sys_dh2 ? a.sys_dh2[s] : a.dh_r2};
}

// system s is rebuilt in this pass (always, unless per-system requests are given)
__device__ __forceinline__ bool rebuilt(const ListArgs &a, int s) { return !a.sys_stale || a.sys_stale[s] != 0; }

__global__ void k_zero_counts(ListArgs a, int n_cells) {
	SKIP_IF_FRESH(a);
	for(int c = blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += gridDim.x * blockDim.x)
		if(!a.cell_sys || rebuilt(a, a.cell_sys[c])) a.cell_count[c] = 0;
}

__global__ void k_cell_count(ListArgs a) {
	SKIP_IF_FRESH(a);
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= a.N) return;
	const int s = sys_of(a, i);
	if(!rebuilt(a, s)) return;
	const CellGeo g = cell_geo(a, s);
	const float4 r = a.pos[i];
	if(!(fabsf(r.x) < 1e7f && fabsf(r.y) < 1e7f && fabsf(r.z) < 1e7f)) {
		atomicOr(a.status, OXGB_ERR_NONFINITE);
		a.cell_of[i] = g.cell0;
		atomicAdd(a.cell_count + g.cell0, 1);
		return;
	}
	const int n = g.n;
	int cx = cell_coord(r.x, g.box, n), cy = cell_coord(r.y, g.box, n), cz = cell_coord(r.z, g.box, n);
	if(cx < 0 || cx >= n || cy < 0 || cy >= n || cz < 0 || cz >= n) {
		atomicOr(a.status, OXGB_ERR_CELL);
		cx = min(max(cx, 0), n - 1);
		cy = min(max(cy, 0), n - 1);
		cz = min(max(cz, 0), n - 1);
	}
	const int c = g.cell0 + (cz * n + cy) * n + cx;
	a.cell_of[i] = c;
	atomicAdd(a.cell_count + c, 1);
}

// Exclusive scan of the cell counts in three passes: block sums, a scan of the block sums by
// one block, then each block's own scan plus its offset.  SCAN_TILE cells per block.
#define SCAN_TPB 512
#define SCAN_TILE (SCAN_TPB * 4)

__device__ __forceinline__ int block_incl_scan(int v, int *warp_tot) {
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
	for(int off = 1; off < 32; off <<= 1) {
		const int u = __shfl_up_sync(0xffffffffu, v, off);
		if(lane >= off) v += u;
	}
	if(lane == 31) warp_tot[w] = v;
	__syncthreads();
	if(w == 0) {
		int t = lane < (int) (blockDim.x >> 5) ? warp_tot[lane] : 0;
#pragma unroll
		for(int off = 1; off < 32; off <<= 1) {
			const int u = __shfl_up_sync(0xffffffffu, t, off);
			if(lane >= off) t += u;
		}
		warp_tot[lane] = t;  // inclusive over warps
	}
	__syncthreads();
	return v + (w > 0 ? warp_tot[w - 1] : 0);
}

__global__ void __launch_bounds__(SCAN_TPB) k_scan_tiles(ListArgs a, int n_cells) {
	SKIP_IF_FRESH(a);
	SKIP_IF_NO_SORT(a);
	__shared__ int wt[32];
	const int base = blockIdx.x * SCAN_TILE + threadIdx.x * 4;
	int v = 0;
#pragma unroll
	for(int k = 0; k < 4; k++)
		if(base + k < n_cells) v += a.cell_count[base + k];
	const int incl = block_incl_scan(v, wt);
	if(threadIdx.x == blockDim.x - 1) a.scan_part[blockIdx.x] = incl;
}

// exclusive scan of the tile sums in place (one block, any number of tiles)
__global__ void __launch_bounds__(SCAN_TPB) k_scan_top(ListArgs a, int n_tiles) {
	SKIP_IF_FRESH(a);
	SKIP_IF_NO_SORT(a);
	__shared__ int wt[32];
	__shared__ int carry;
	if(threadIdx.x == 0) carry = 0;
	__syncthreads();
	for(int b = 0; b < n_tiles; b += blockDim.x) {
		const int t = b + threadIdx.x;
		const int v = t < n_tiles ? a.scan_part[t] : 0;
		const int incl = block_incl_scan(v, wt);
		const int c0 = carry;
		if(t < n_tiles) a.scan_part[t] = c0 + incl - v;
		__syncthreads();
		if(threadIdx.x == blockDim.x - 1) carry = c0 + incl;
		__syncthreads();
	}
	if(threadIdx.x == 0) a.scan_part[n_tiles] = carry;
}

__global__ void __launch_bounds__(SCAN_TPB) k_scan_apply(ListArgs a, int n_cells, int n_tiles) {
	SKIP_IF_FRESH(a);
	SKIP_IF_NO_SORT(a);
	__shared__ int wt[32];
	const int base = blockIdx.x * SCAN_TILE + threadIdx.x * 4;
	int c[4], v = 0;
#pragma unroll
	for(int k = 0; k < 4; k++) {
		c[k] = base + k < n_cells ? a.cell_count[base + k] : 0;
		v += c[k];
	}
	int run = block_incl_scan(v, wt) - v + a.scan_part[blockIdx.x];
#pragma unroll
	for(int k = 0; k < 4; k++) {
		if(base + k < n_cells) {
			a.cell_start[base + k] = run;
			a.cell_cursor[base + k] = run;
		}
		run += c[k];
	}
	if(blockIdx.x == 0 && threadIdx.x == 0) a.cell_start[n_cells] = a.scan_part[n_tiles];
}

// particles into their cells' segments, in arbitrary order (cell_tmp)
__global__ void k_cell_scatter(ListArgs a) {
	SKIP_IF_FRESH(a);
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= a.N || !rebuilt(a, sys_of(a, i))) return;
	const int slot = atomicAdd(a.cell_cursor + a.cell_of[i], 1);
	a.cell_tmp[slot] = i;
}

// the caller's index of slot i (slot i itself while the engine was never sorted)
__device__ __forceinline__ int id_of(const ListArgs &a, int i) { return a.id ? a.id[i] : i; }

// each particle's rank by caller's index within its cell gives the deterministic order (cell_list)
__global__ void k_cell_rank(ListArgs a) {
	SKIP_IF_FRESH(a);
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= a.N || !rebuilt(a, sys_of(a, i))) return;
	const int c = a.cell_of[i];
	const int b = a.cell_start[c], e = a.cell_start[c + 1];
	const int key = id_of(a, i);
	int rank = 0;
	for(int k = b; k < e; k++) rank += id_of(a, a.cell_tmp[k]) < key;
	a.cell_list[b + rank] = i;
}

// ---------------------------------------------------------------- cell-order storage
// (CUDABaseBackend::_sort_particles, CUDABaseBackend.cu:263-281, with the cell order of this
// build in place of a Hilbert key: the order is the one the counting sort just produced)

// this build moves nucleotides: sorting on, and the build count a multiple of sort_every
__device__ __forceinline__ bool sort_now(const ListArgs &a) {
	return a.sort_every > 0 && a.id && (a.rebuilds ? *a.rebuilds : 0ull) % (unsigned long long) a.sort_every == 0ull;
}

// new slot k takes old slot perm[k] = cell_list[k] (rebuilt systems; the others stay)
__global__ void k_sort_perm(ListArgs a) {
	SKIP_IF_FRESH(a);
	if(!sort_now(a)) return;
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= a.N) return;
	const int from = rebuilt(a, sys_of(a, k)) ? a.cell_list[k] : k;
	a.perm[k] = from;
	a.inv[from] = k;
}

// Hilbert order: every cell's count at its Hilbert position (counts of systems not rebuilt are
// those of their last build, so every system's cells still hold exactly its nucleotides)
__global__ void k_sort_hcount(ListArgs a, int n_cells) {
	SKIP_IF_FRESH(a);
	if(!sort_now(a)) return;
	const int c = blockIdx.x * blockDim.x + threadIdx.x;
	if(c < n_cells) a.hcount[a.cell_hil[c]] = a.cell_count[c];
}

// Hilbert order: the nucleotide at position p of the cell-ordered list moves to the position of
// its cell along the curve plus its rank within the cell (rebuilt systems; the others stay)
__global__ void k_sort_perm_hilbert(ListArgs a) {
	SKIP_IF_FRESH(a);
	if(!sort_now(a)) return;
	const int p = blockIdx.x * blockDim.x + threadIdx.x;
	if(p >= a.N) return;
	if(!rebuilt(a, sys_of(a, p))) {
		a.perm[p] = p;
		a.inv[p] = p;
		return;
	}
	const int i = a.cell_list[p];
	const int c = a.cell_of[i];
	const int q = a.hstart[a.cell_hil[c]] + (p - a.cell_start[c]);
	a.perm[q] = i;
	a.inv[i] = q;
}

// everything of old slot perm[k] into the staging buffer at k; bonds renumbered
__global__ void k_sort_gather(ListArgs a) {
	SKIP_IF_FRESH(a);
	if(!sort_now(a)) return;
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= a.N) return;
	const long long N = a.N;
	const int from = a.perm[k];
	double4_32a *sd = reinterpret_cast<double4_32a *>(a.scratch);
	float4 *sf = reinterpret_cast<float4 *>(a.scratch + 4 * 32 * N);
	int2 *sb = reinterpret_cast<int2 *>(a.scratch + (4 * 32 + SORT_MIRRORS * 16) * N);
	int *si = reinterpret_cast<int *>(a.scratch + (4 * 32 + SORT_MIRRORS * 16 + 8) * N);
#pragma unroll
	for(int t = 0; t < 4; t++) sd[t * N + k] = a.st[t][from];
#pragma unroll
	for(int t = 0; t < SORT_MIRRORS; t++)
		if(a.mir[t]) sf[t * N + k] = a.mir[t][from];
	const int2 b = a.bonds_rw[from];
	sb[k] = make_int2(b.x >= 0 ? a.inv[b.x] : -1, b.y >= 0 ? a.inv[b.y] : -1);
	si[k] = a.id[from];
	si[N + k] = a.cell_of[from];
	// segment entries name slots: renamed in place (each k touches its own entry)
	a.cell_list[k] = a.inv[a.cell_list[k]];
}

// the staging buffer back into the arrays, and the inverse map
__global__ void k_sort_scatter(ListArgs a) {
	SKIP_IF_FRESH(a);
	if(!sort_now(a)) return;
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= a.N) return;
	const long long N = a.N;
	const double4_32a *sd = reinterpret_cast<const double4_32a *>(a.scratch);
	const float4 *sf = reinterpret_cast<const float4 *>(a.scratch + 4 * 32 * N);
	const int2 *sb = reinterpret_cast<const int2 *>(a.scratch + (4 * 32 + SORT_MIRRORS * 16) * N);
	const int *si = reinterpret_cast<const int *>(a.scratch + (4 * 32 + SORT_MIRRORS * 16 + 8) * N);
#pragma unroll
	for(int t = 0; t < 4; t++) a.st[t][k] = sd[t * N + k];
#pragma unroll
	for(int t = 0; t < SORT_MIRRORS; t++)
		if(a.mir[t]) a.mir[t][k] = sf[t * N + k];
	a.bonds_rw[k] = sb[k];
	const int id = si[k];
	a.id[k] = id;
	a.slot[id] = k;
	a.cell_of[k] = si[N + k];
}

// the minimum-image separation vector of a listed pair (the reference's FP32 geometry, explicit
// fused multiply-adds), the image picked as in sqr_min_image_inv: the same integer as the IEEE
// quotient's rint for any pair closer than the Verlet radius, so the same vector
__device__ __forceinline__ float3 min_image_vec_inv(float4 a, float4 b, float L, float inv) {
	float d[3] = {b.x - a.x, b.y - a.y, b.z - a.z};
#pragma unroll
	for(int k = 0; k < 3; k++) d[k] = __fmaf_rn(-__fsub_rn(__fmaf_rn(d[k], inv, 12582912.f), 12582912.f), L, d[k]);
	return make_float3(d[0], d[1], d[2]);
}

// squared distance of the backbone sites of a listed pair (d: the centres' separation, bk: the
// backbone offsets)
__device__ __forceinline__ float back_sq(float3 d, float4 bki, float4 bkj) {
	const float x = d.x + bkj.x - bki.x, y = d.y + bkj.y - bki.y, z = d.z + bkj.z - bki.z;
	return x * x + y * y + z * z;
}

// A pair's excluded volume can act before the next rebuild only if one of its four site pairs
// (backbone-backbone, base-base, backbone-base both ways) is within that pair's cutoff plus twice
// the skin: the staleness test rebuilds before any site moves farther than the skin.  d is the
// centres' separation, a1 and bk the axes and backbone offsets (base site at 0.4 a1).
__device__ __forceinline__ bool ev_sites_near(const ListArgs &a, float3 d, float4 a1i, float4 bki, float4 a1j, float4 bkj) {
	const float ix = 0.4f * a1i.x, iy = 0.4f * a1i.y, iz = 0.4f * a1i.z;
	const float jx = 0.4f * a1j.x, jy = 0.4f * a1j.y, jz = 0.4f * a1j.z;
	auto sq = [](float x, float y, float z) { return x * x + y * y + z * z; };
	return sq(d.x + bkj.x - bki.x, d.y + bkj.y - bki.y, d.z + bkj.z - bki.z) < a.evs_r2[0] ||
			sq(d.x + jx - ix, d.y + jy - iy, d.z + jz - iz) < a.evs_r2[1] ||
			sq(d.x + jx - bki.x, d.y + jy - bki.y, d.z + jz - bki.z) < a.evs_r2[2] ||
			sq(d.x + bkj.x - ix, d.y + bkj.y - iy, d.z + bkj.z - iz) < a.evs_r2[2];
}

__device__ __forceinline__ void put(int *rows, bool col_major, long long N, int stride, int i, int k, int j) {
	if(col_major) rows[(long long) k * N + i] = j;
	else rows[(long long) i * stride + k] = j;
}

// One warp per nucleotide.  The candidates of the 27 cells, in the serial scan order (dz, dy, dx
// from -1 to 1, each cell's segment by index), are numbered 0..C-1; lane l takes candidates
// l, l + 32, ... and the hits of every round are compacted in order with a ballot, so each row
// comes out exactly as a serial scan would write it.
__global__ void __launch_bounds__(256) k_neighbours(ListArgs a) {
	SKIP_IF_FRESH(a);
	const int lane = threadIdx.x & 31;
	const int i = (int) (((long long) blockIdx.x * blockDim.x + threadIdx.x) >> 5);
	if(i >= a.N) return;  // warp-uniform
	const int sy = sys_of(a, i);
	if(!rebuilt(a, sy)) return;  // warp-uniform
	const CellGeo g = cell_geo(a, sy);
	const float4 r = a.pos[i];
	const int2 b = a.bonds[i];
	const int n = g.n;
	const int c = a.cell_of[i] - g.cell0;
	const int cx = c % n, cy = (c / n) % n, cz = c / (n * n);
	const bool terms = a.ev_nb != nullptr;
	const long long N = a.N;
	const float inv_box = __frcp_rn(g.box);
	// lane l < 27 owns the l-th cell of the scan
	int cs = 0, cn = 0;
	if(lane < 27) {
		// wrapped with compares (an integer modulo by the grid size costs a division)
		int z = cz + lane / 9 - 1, y = cy + (lane / 3) % 3 - 1, x = cx + lane % 3 - 1;
		z += z < 0 ? n : (z >= n ? -n : 0);
		y += y < 0 ? n : (y >= n ? -n : 0);
		x += x < 0 ? n : (x >= n ? -n : 0);
		const int cc = g.cell0 + (z * n + y) * n + x;
		cs = a.cell_start[cc];
		cn = a.cell_start[cc + 1] - cs;
	}
	int incl = cn;
#pragma unroll
	for(int off = 1; off < 32; off <<= 1) {
		const int u = __shfl_up_sync(0xffffffffu, incl, off);
		if(lane >= off) incl += u;
	}
	const int total = __shfl_sync(0xffffffffu, incl, 31);
	const int excl = incl - cn;
	const bool dhl = a.dh_nb != nullptr;
	float4 a1i = make_float4(0.f, 0.f, 0.f, 0.f), bki = a1i;
	if(terms || dhl) {
		a1i = a.fa1[i];
		bki = a.fback[i];
	}
	const unsigned below = (1u << lane) - 1u;
	int cnt = 0, nev = 0, nbase = 0, nstk = 0, ndh = 0;
	for(int t0 = 0; t0 < total; t0 += 32) {
		const int t = t0 + lane;
		// the cell holding candidate t: the first lane whose inclusive count exceeds t
		int l = 0;
#pragma unroll
		for(int step = 16; step > 0; step >>= 1) {
			const int v = __shfl_sync(0xffffffffu, incl, l + step - 1);
			if(v <= t) l += step;
		}
		const int cs_l = __shfl_sync(0xffffffffu, cs, l & 31), ex_l = __shfl_sync(0xffffffffu, excl, l & 31);
		bool hit = false, hev = false, hbase = false, hstk = false, hdh = false;
		int j = -1;
		if(t < total) {
			j = a.cell_list[cs_l + (t - ex_l)];
			if(j != i && j != b.x && j != b.y) {
				const float4 rj = a.pos[j];
				const float d2 = sqr_min_image_inv(r, rj, g.box, inv_box);
				hit = d2 < g.rv2;
				if(hit && (terms || dhl)) {
					const float3 d = min_image_vec_inv(r, rj, g.box, inv_box);
					const float4 bkj = a.fback[j];
					hdh = dhl && back_sq(d, bki, bkj) < g.dh2;
					if(terms && d2 < a.ev_r2) {
						const float4 a1j = a.fa1[j];
						hev = ev_sites_near(a, d, a1i, bki, a1j, bkj);
						// base sites at 0.4 a1, stacking sites at 0.34 a1 from the centres
						const float bx = d.x + 0.4f * (a1j.x - a1i.x), by = d.y + 0.4f * (a1j.y - a1i.y),
								bz = d.z + 0.4f * (a1j.z - a1i.z);
						hbase = bx * bx + by * by + bz * bz < a.base_r2;
						const float sx = d.x + 0.34f * (a1j.x - a1i.x), sy = d.y + 0.34f * (a1j.y - a1i.y),
								sz = d.z + 0.34f * (a1j.z - a1i.z);
						hstk = sx * sx + sy * sy + sz * sz < a.stk_r2;
					}
				}
			}
		}
		const unsigned m = __ballot_sync(0xffffffffu, hit);
		if(hit) {
			const int k = cnt + __popc(m & below);
			if(k < a.max_nb) put(a.nb, a.col_major != 0, N, a.max_nb, i, k, j);
		}
		cnt += __popc(m);
		if(dhl) {
			const unsigned md = __ballot_sync(0xffffffffu, hdh);
			if(hdh) {
				const int k = ndh + __popc(md & below);
				if(k < a.max_nb) a.dh_nb[(long long) k * N + i] = j;
			}
			ndh += __popc(md);
		}
		if(terms) {
			const unsigned me = __ballot_sync(0xffffffffu, hev), mb = __ballot_sync(0xffffffffu, hbase),
					ms = __ballot_sync(0xffffffffu, hstk);
			if(hev) {
				const int k = nev + __popc(me & below);
				if(k < a.ev_cap) a.ev_nb[(long long) k * N + i] = j;
			}
			if(hbase) {
				const int k = nbase + __popc(mb & below);
				if(k < a.base_cap) a.base_nb[(long long) k * N + i] = j;
			}
			if(hstk) {
				const int k = nstk + __popc(ms & below);
				if(k < a.stk_cap) a.stk_nb[(long long) k * N + i] = j;
			}
			nev += __popc(me);
			nbase += __popc(mb);
			nstk += __popc(ms);
		}
	}
	if(lane != 0) return;
	if(cnt > a.max_nb) atomicOr(a.status, OXGB_ERR_NEIGH_OVERFLOW);
	if(a.term_max && cnt > a.term_max[3]) atomicMax(a.term_max + 3, cnt);
	a.nnb[i] = cnt;
	if(dhl) a.dh_n[i] = ndh;
	a.list_pos[i] = r;
	if(terms) {
		if(nev > a.ev_cap || nbase > a.base_cap || nstk > a.stk_cap) atomicOr(a.status, OXGB_ERR_NEIGH_OVERFLOW);
		if(a.term_max) {  // read first: the maxima rarely grow, so few atomics reach them
			if(nev > a.term_max[0]) atomicMax(a.term_max, nev);
			if(nbase > a.term_max[1]) atomicMax(a.term_max + 1, nbase);
			if(nstk > a.term_max[2]) atomicMax(a.term_max + 2, nstk);
		}
		a.ev_n[i] = nev;
		a.base_n[i] = nbase;
		a.stk_n[i] = nstk;
		a.list_a1[i] = a1i;
		a.list_back[i] = bki;
	}
}

// One thread per nucleotide, the 27 cells in the same serial order (dz, dy, dx from -1 to 1, each
// cell's segment by index) and the same FP32 tests, so the rows are those of k_neighbours entry for
// entry.  Consecutive threads are consecutive nucleotides, so the stores of entry k into the
// column-major rows ([k N + i]) of a warp fall into one or two sectors, where k_neighbours' lanes
// store the entries of one row N apart.  Fewer instructions and coalesced stores win where a
// nucleotide's 27 cells hold few candidates (measured: the 250,000-nucleotide melt, 0.8 per cell);
// the warp kernel wins where they hold many (clustered duplexes): the engine's autotuner times both.
__global__ void __launch_bounds__(128) k_neighbours_thread(ListArgs a) {
	SKIP_IF_FRESH(a);
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= a.N) return;
	const int sy = sys_of(a, i);
	if(!rebuilt(a, sy)) return;
	const CellGeo g = cell_geo(a, sy);
	const float4 r = a.pos[i];
	const int2 b = a.bonds[i];
	const int n = g.n;
	const int c = a.cell_of[i] - g.cell0;
	const int cx = c % n, cy = (c / n) % n, cz = c / (n * n);
	const bool terms = a.ev_nb != nullptr;
	const long long N = a.N;
	const bool dhl = a.dh_nb != nullptr;
	float4 a1i = make_float4(0.f, 0.f, 0.f, 0.f), bki = a1i;
	if(terms || dhl) {
		a1i = a.fa1[i];
		bki = a.fback[i];
	}
	int cnt = 0, nev = 0, nbase = 0, nstk = 0, ndh = 0;
	const float inv_box = __frcp_rn(g.box);
	// the 27 cells in the serial order (dz, dy, dx from -1 to 1), wrapped without integer division.
	// The cells x = cx - 1, cx, cx + 1 of a (z, y) row are consecutive cells, so their segments
	// are one run of cell_list: cells [x0, e0) of the row, and where the row wraps at the box face
	// a second run [x1, e1) -- nine rows of at most two runs instead of 27 cells
	int x0, e0, x1 = 0, e1 = 0;
	if(cx > 0 && cx < n - 1) x0 = cx - 1, e0 = cx + 2;
	else if(cx == 0) x0 = n - 1, e0 = n, e1 = 2;  // cells n - 1 | 0, 1
	else x0 = n - 2, e0 = n, e1 = 1;              // cells n - 2, n - 1 | 0
	for(int zy = 0; zy < 9; zy++)
	for(int run = 0; run < 2; run++) {
		const int xa = run ? x1 : x0, xb = run ? e1 : e0;
		if(xa >= xb) continue;
		int z = cz + zy / 3 - 1, y = cy + zy % 3 - 1;
		z += z < 0 ? n : (z >= n ? -n : 0);
		y += y < 0 ? n : (y >= n ? -n : 0);
		const int row = g.cell0 + (z * n + y) * n;
		const int s1 = a.cell_start[row + xb];
		for(int u = a.cell_start[row + xa]; u < s1; u++) {
			const int j = a.cell_list[u];
			if(j == i || j == b.x || j == b.y) continue;
			const float4 rj = a.pos[j];
			const float d2 = sqr_min_image_inv(r, rj, g.box, inv_box);
			if(!(d2 < g.rv2)) continue;
			if(cnt < a.max_nb) put(a.nb, a.col_major != 0, N, a.max_nb, i, cnt, j);
			cnt++;
			if(!(terms || dhl)) continue;
			const float3 d = min_image_vec_inv(r, rj, g.box, inv_box);
			const float4 bkj = a.fback[j];
			if(dhl && back_sq(d, bki, bkj) < g.dh2) {
				if(ndh < a.max_nb) a.dh_nb[(long long) ndh * N + i] = j;
				ndh++;
			}
			if(terms && d2 < a.ev_r2) {
				const float4 a1j = a.fa1[j];
				if(ev_sites_near(a, d, a1i, bki, a1j, bkj)) {
					if(nev < a.ev_cap) a.ev_nb[(long long) nev * N + i] = j;
					nev++;
				}
				// base sites at 0.4 a1, stacking sites at 0.34 a1 from the centres
				const float bx = d.x + 0.4f * (a1j.x - a1i.x), by = d.y + 0.4f * (a1j.y - a1i.y),
						bz = d.z + 0.4f * (a1j.z - a1i.z);
				if(bx * bx + by * by + bz * bz < a.base_r2) {
					if(nbase < a.base_cap) a.base_nb[(long long) nbase * N + i] = j;
					nbase++;
				}
				const float sx = d.x + 0.34f * (a1j.x - a1i.x), sy2 = d.y + 0.34f * (a1j.y - a1i.y),
						sz = d.z + 0.34f * (a1j.z - a1i.z);
				if(sx * sx + sy2 * sy2 + sz * sz < a.stk_r2) {
					if(nstk < a.stk_cap) a.stk_nb[(long long) nstk * N + i] = j;
					nstk++;
				}
			}
		}
	}
	if(cnt > a.max_nb) atomicOr(a.status, OXGB_ERR_NEIGH_OVERFLOW);
	if(a.term_max && cnt > a.term_max[3]) atomicMax(a.term_max + 3, cnt);
	a.nnb[i] = cnt;
	if(dhl) a.dh_n[i] = ndh;
	a.list_pos[i] = r;
	if(terms) {
		if(nev > a.ev_cap || nbase > a.base_cap || nstk > a.stk_cap) atomicOr(a.status, OXGB_ERR_NEIGH_OVERFLOW);
		if(a.term_max) {
			if(nev > a.term_max[0]) atomicMax(a.term_max, nev);
			if(nbase > a.term_max[1]) atomicMax(a.term_max + 1, nbase);
			if(nstk > a.term_max[2]) atomicMax(a.term_max + 2, nstk);
		}
		a.ev_n[i] = nev;
		a.base_n[i] = nbase;
		a.stk_n[i] = nstk;
		a.list_a1[i] = a1i;
		a.list_back[i] = bki;
	}
}

// K lanes per nucleotide (K = 4, 8 or 16; 128 / K nucleotides per block): the rows of
// k_neighbours, entry for entry, with shorter serial chains than the thread kernel and fewer idle
// lanes than the warp kernel where a nucleotide has a few dozen candidates.  Lane s of a group
// owns the C = ceil(27 / K) consecutive cells s C .. s C + C - 1 of the serial scan order and
// counts them; a group scan gives every cell's first candidate number, kept with its segment
// start in shared memory; then the group takes candidates t0 + s, t0 + K + s, ..., each lane
// finding its candidate's cell by a binary search of those numbers, and the hits of every round
// are compacted in order with a ballot over the group's lanes.  All lanes of a group see the same
// candidate count, so a group never diverges; the groups of a warp may.
template <int K>
__global__ void __launch_bounds__(128) k_neighbours_group(ListArgs a) {
	constexpr int C = (27 + K - 1) / K;
	constexpr int G = 128 / K;
	__shared__ int s_first[G][32], s_start[G][32];  // per group: cell l's first candidate, its segment start
	SKIP_IF_FRESH(a);
	const int lane = threadIdx.x & 31, sub = lane % K, grp = (int) threadIdx.x / K;
	const unsigned gmask = (K == 32 ? 0xffffffffu : ((1u << K) - 1u)) << (lane - sub);
	const int i = (int) (((long long) blockIdx.x * blockDim.x + threadIdx.x) / K);
	if(i >= a.N) return;  // group-uniform
	const int sy = sys_of(a, i);
	if(!rebuilt(a, sy)) return;  // group-uniform
	const CellGeo g = cell_geo(a, sy);
	const float4 r = a.pos[i];
	const int2 b = a.bonds[i];
	const int n = g.n;
	const int c = a.cell_of[i] - g.cell0;
	const int cx = c % n, cy = (c / n) % n, cz = c / (n * n);
	const bool terms = a.ev_nb != nullptr;
	const long long N = a.N;
	const float inv_box = __frcp_rn(g.box);
	// this lane's cells: segment starts and counts, and their running total
	int st[C], ct[C], run = 0;
#pragma unroll
	for(int q = 0; q < C; q++) {
		const int l = sub * C + q;
		st[q] = 0;
		ct[q] = 0;
		if(l < 27) {
			int z = cz + l / 9 - 1, y = cy + (l / 3) % 3 - 1, x = cx + l % 3 - 1;
			z += z < 0 ? n : (z >= n ? -n : 0);
			y += y < 0 ? n : (y >= n ? -n : 0);
			x += x < 0 ? n : (x >= n ? -n : 0);
			const int cc = g.cell0 + (z * n + y) * n + x;
			st[q] = a.cell_start[cc];
			ct[q] = a.cell_start[cc + 1] - st[q];
		}
		run += ct[q];
	}
	// exclusive scan of the lanes' totals over the group
	int incl = run;
#pragma unroll
	for(int off = 1; off < K; off <<= 1) {
		const int u = __shfl_up_sync(gmask, incl, off, K);
		if(sub >= off) incl += u;
	}
	const int total = __shfl_sync(gmask, incl, K - 1, K);
	int first = incl - run;
#pragma unroll
	for(int q = 0; q < C; q++) {
		const int l = sub * C + q;
		if(l < 32) {
			s_first[grp][l] = l < 27 ? first : INT_MAX;
			s_start[grp][l] = st[q];
		}
		first += ct[q];
	}
	// the padding entries 27..31 (cells of no lane when K C < 32)
	for(int l = K * C + sub; l < 32; l += K) s_first[grp][l] = INT_MAX;
	__syncwarp(gmask);
	const bool dhl = a.dh_nb != nullptr;
	float4 a1i = make_float4(0.f, 0.f, 0.f, 0.f), bki = a1i;
	if(terms || dhl) {
		a1i = a.fa1[i];
		bki = a.fback[i];
	}
	const unsigned below = ((1u << lane) - 1u) & gmask;
	int cnt = 0, nev = 0, nbase = 0, nstk = 0, ndh = 0;
	for(int t0 = 0; t0 < total; t0 += K) {
		const int t = t0 + sub;
		bool hit = false, hev = false, hbase = false, hstk = false, hdh = false;
		int j = -1;
		if(t < total) {
			// the cell holding candidate t: the last one whose first candidate is at most t
			int l = 0;
#pragma unroll
			for(int step = 16; step > 0; step >>= 1)
				if(s_first[grp][l + step] <= t) l += step;
			j = a.cell_list[s_start[grp][l] + (t - s_first[grp][l])];
			if(j != i && j != b.x && j != b.y) {
				const float4 rj = a.pos[j];
				const float d2 = sqr_min_image_inv(r, rj, g.box, inv_box);
				hit = d2 < g.rv2;
				if(hit && (terms || dhl)) {
					const float3 d = min_image_vec_inv(r, rj, g.box, inv_box);
					const float4 bkj = a.fback[j];
					hdh = dhl && back_sq(d, bki, bkj) < g.dh2;
					if(terms && d2 < a.ev_r2) {
						const float4 a1j = a.fa1[j];
						hev = ev_sites_near(a, d, a1i, bki, a1j, bkj);
						// base sites at 0.4 a1, stacking sites at 0.34 a1 from the centres
						const float bx = d.x + 0.4f * (a1j.x - a1i.x), by = d.y + 0.4f * (a1j.y - a1i.y),
								bz = d.z + 0.4f * (a1j.z - a1i.z);
						hbase = bx * bx + by * by + bz * bz < a.base_r2;
						const float sx = d.x + 0.34f * (a1j.x - a1i.x), sy2 = d.y + 0.34f * (a1j.y - a1i.y),
								sz = d.z + 0.34f * (a1j.z - a1i.z);
						hstk = sx * sx + sy2 * sy2 + sz * sz < a.stk_r2;
					}
				}
			}
		}
		const unsigned m = __ballot_sync(gmask, hit) & gmask;
		if(hit) {
			const int k = cnt + __popc(m & below);
			if(k < a.max_nb) put(a.nb, a.col_major != 0, N, a.max_nb, i, k, j);
		}
		cnt += __popc(m);
		if(dhl) {
			const unsigned md = __ballot_sync(gmask, hdh) & gmask;
			if(hdh) {
				const int k = ndh + __popc(md & below);
				if(k < a.max_nb) a.dh_nb[(long long) k * N + i] = j;
			}
			ndh += __popc(md);
		}
		if(terms) {
			const unsigned me = __ballot_sync(gmask, hev) & gmask, mb = __ballot_sync(gmask, hbase) & gmask,
					ms = __ballot_sync(gmask, hstk) & gmask;
			if(hev) {
				const int k = nev + __popc(me & below);
				if(k < a.ev_cap) a.ev_nb[(long long) k * N + i] = j;
			}
			if(hbase) {
				const int k = nbase + __popc(mb & below);
				if(k < a.base_cap) a.base_nb[(long long) k * N + i] = j;
			}
			if(hstk) {
				const int k = nstk + __popc(ms & below);
				if(k < a.stk_cap) a.stk_nb[(long long) k * N + i] = j;
			}
			nev += __popc(me);
			nbase += __popc(mb);
			nstk += __popc(ms);
		}
	}
	if(sub != 0) return;
	if(cnt > a.max_nb) atomicOr(a.status, OXGB_ERR_NEIGH_OVERFLOW);
	if(a.term_max && cnt > a.term_max[3]) atomicMax(a.term_max + 3, cnt);
	a.nnb[i] = cnt;
	if(dhl) a.dh_n[i] = ndh;
	a.list_pos[i] = r;
	if(terms) {
		if(nev > a.ev_cap || nbase > a.base_cap || nstk > a.stk_cap) atomicOr(a.status, OXGB_ERR_NEIGH_OVERFLOW);
		if(a.term_max) {
			if(nev > a.term_max[0]) atomicMax(a.term_max, nev);
			if(nbase > a.term_max[1]) atomicMax(a.term_max + 1, nbase);
			if(nstk > a.term_max[2]) atomicMax(a.term_max + 2, nstk);
		}
		a.ev_n[i] = nev;
		a.base_n[i] = nbase;
		a.stk_n[i] = nstk;
		a.list_a1[i] = a1i;
		a.list_back[i] = bki;
	}
}

// For every base / stack list entry (k, i) with partner j above i by caller's index (i owns the
// pair, as in an unsorted run): where i sits in
// j's list (the lists are symmetric: the pair criteria are exactly symmetric in FP32).  One
// thread per nucleotide and term (blocks 0 .. base_blocks - 1: base lists).
__global__ void k_term_pos(ListArgs a, int base_blocks) {
	SKIP_IF_FRESH(a);
	const bool is_base = (int) blockIdx.x < base_blocks;
	const int i = (is_base ? blockIdx.x : blockIdx.x - base_blocks) * blockDim.x + threadIdx.x;
	if(i >= a.N || !rebuilt(a, sys_of(a, i))) return;
	const long long N = a.N;
	const int cap = is_base ? a.base_cap : a.stk_cap;
	const int *nb = is_base ? a.base_nb : a.stk_nb;
	int *pos = is_base ? a.base_pos : a.stk_pos;
	const int n = min(is_base ? a.base_n[i] : a.stk_n[i], cap);
	for(int k = 0; k < n; k++) {
		const int j = nb[(long long) k * N + i];
		int r = -1;
		if(id_of(a, j) > id_of(a, i)) {
			const int nj = min(is_base ? a.base_n[j] : a.stk_n[j], cap);
			for(int m = 0; m < nj; m++)
				if(nb[(long long) m * N + j] == i) {
					r = m;
					break;
				}
			if(r < 0) atomicOr(a.status, OXGB_ERR_NEIGH_OVERFLOW);  // an asymmetric (overflowed) list
		}
		pos[(long long) k * N + i] = r;
	}
}

// runs after every other list kernel: counts the build and clears the requests
__global__ void k_list_done(ListArgs a) {
	if(blockIdx.x != 0) return;
	if(a.check_flag && *a.flag == 0) return;
	if(a.sys_stale)
		for(int s = threadIdx.x; s < a.n_systems; s += blockDim.x) a.sys_stale[s] = 0;
	if(threadIdx.x != 0) return;
	if(a.rebuilds) *a.rebuilds += 1;
	*a.flag = 0;
}

int scan_tiles(int n_cells) { return (n_cells + SCAN_TILE - 1) / SCAN_TILE; }

cudaError_t launch_list_build(const ListArgs &a, cudaStream_t s) {
	const int n_cells = a.n_cells_total > 0 ? a.n_cells_total : a.n_side * a.n_side * a.n_side;
	const int tpb = 256;
	const int gp = (a.N + tpb - 1) / tpb;
	const int tiles = scan_tiles(n_cells);
	k_zero_counts<<<(n_cells + tpb - 1) / tpb, tpb, 0, s>>>(a, n_cells);
	k_cell_count<<<gp, tpb, 0, s>>>(a);
	k_scan_tiles<<<tiles, SCAN_TPB, 0, s>>>(a, n_cells);
	k_scan_top<<<1, SCAN_TPB, 0, s>>>(a, tiles);
	k_scan_apply<<<tiles, SCAN_TPB, 0, s>>>(a, n_cells, tiles);
	k_cell_scatter<<<gp, tpb, 0, s>>>(a);
	k_cell_rank<<<gp, tpb, 0, s>>>(a);
	if(a.sort_every > 0 && a.id && a.cell_hil) {
		// the counts in Hilbert order, scanned by the same three kernels on a copy of the
		// arguments, then the permutation
		k_sort_hcount<<<(n_cells + tpb - 1) / tpb, tpb, 0, s>>>(a, n_cells);
		ListArgs h = a;
		h.cell_count = a.hcount;
		h.cell_start = a.hstart;
		h.cell_cursor = a.hcursor;
		h.hilbert_pass = 1;
		k_scan_tiles<<<tiles, SCAN_TPB, 0, s>>>(h, n_cells);
		k_scan_top<<<1, SCAN_TPB, 0, s>>>(h, tiles);
		k_scan_apply<<<tiles, SCAN_TPB, 0, s>>>(h, n_cells, tiles);
		k_sort_perm_hilbert<<<gp, tpb, 0, s>>>(a);
		k_sort_gather<<<gp, tpb, 0, s>>>(a);
		k_sort_scatter<<<gp, tpb, 0, s>>>(a);
	}
	else if(a.sort_every > 0 && a.id) {
		k_sort_perm<<<gp, tpb, 0, s>>>(a);
		k_sort_gather<<<gp, tpb, 0, s>>>(a);
		k_sort_scatter<<<gp, tpb, 0, s>>>(a);
	}
	switch(a.list_kind) {
	case OXGB_LIST_THREAD: k_neighbours_thread<<<(a.N + 127) / 128, 128, 0, s>>>(a); break;
	case OXGB_LIST_GROUP4: k_neighbours_group<4><<<(int) (((long long) a.N * 4 + 127) / 128), 128, 0, s>>>(a); break;
	case OXGB_LIST_GROUP8: k_neighbours_group<8><<<(int) (((long long) a.N * 8 + 127) / 128), 128, 0, s>>>(a); break;
	case OXGB_LIST_GROUP16: k_neighbours_group<16><<<(int) (((long long) a.N * 16 + 127) / 128), 128, 0, s>>>(a); break;
	default: {
		const long long warps = (long long) a.N * 32;
		k_neighbours<<<(int) ((warps + tpb - 1) / tpb), tpb, 0, s>>>(a);
	}
	}
	if(a.base_pos && a.stk_pos) k_term_pos<<<2 * gp, tpb, 0, s>>>(a, gp);
	k_list_done<<<1, 256, 0, s>>>(a);
	return cudaGetLastError();
}

}  // namespace oxgb
