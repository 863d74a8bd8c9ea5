// oxDNA2 force and torque kernel: one warp per nucleotide.
//
// Lanes stride over the nucleotide's neighbour row (full list: every pair is seen from both
// ends, so no atomics and a fixed summation order); lanes 0 and 1 also take the 3' and 5'
// bonded pairs.  Each lane accumulates its pair forces, lab-frame torques and energies with
// compensated (Kahan) sums, the warp combines them with an error-free TwoSum butterfly, and
// lane 0 rotates the torque into the body frame and writes the result.  Replaces the
// reference's thread-per-nucleotide dna_forces (src/CUDA/Interactions/CUDA_DNA.cuh:832-904).
//
// Three instantiations:
//  * FP32 "mixed" path: positions as a hi/lo float pair so that pair separations keep ~1e-7
//    absolute accuracy in boxes of side 200+, quaternions in FP32, FP32 pair math;
//  * FP64 path: the same physics in double, for parity against the FP64 oracle;
//  * reference layout: float4 positions with btype/index packed in w, float4 quaternions,
//    int2 bonds and a neighbour matrix of any stride, accumulating into forces and torques
//    initialised by the caller, exactly the contract of CUDABaseInteraction::compute_forces.
#include "kernels.h"
#include "split.cuh"

#include <cuda_runtime.h>

namespace oxgb {

template <typename R>
struct KahanV {
	v3<R> s, c;
	OXGB_HD void add(v3<R> x) {
		kadd(s.x, c.x, x.x);
		kadd(s.y, c.y, x.y);
		kadd(s.z, c.z, x.z);
	}
	static OXGB_HD void kadd(R &sum, R &comp, R x) {
		const R y = x - comp;
		const R t = sum + y;
		comp = (t - sum) - y;
		sum = t;
	}
};

// sum over the warp of (s - c) pairs with TwoSum at every butterfly level; all lanes get it
template <typename R>
__device__ __forceinline__ R warp_sum_comp(R s, R c) {
	R err = -c;
#pragma unroll
	for(int off = 16; off > 0; off >>= 1) {
		const R so = __shfl_xor_sync(0xffffffffu, s, off);
		const R eo = __shfl_xor_sync(0xffffffffu, err, off);
		const R t = s + so;
		const R bp = t - s;
		const R e2 = (s - (t - bp)) + (so - bp);
		s = t;
		err += eo + e2;
	}
	return s + err;
}

__device__ __forceinline__ int ref_type_of_btype(int bt) {
	return (bt > 0) ? (bt & 3) : 3 - ((3 - bt) & 3);
}

template <typename R>
__device__ __forceinline__ void load_table(const DNA2Table<R> *g, DNA2Table<R> *s) {
	const int n = sizeof(DNA2Table<R>) / sizeof(int);
	const int *src = reinterpret_cast<const int *>(g);
	int *dst = reinterpret_cast<int *>(s);
	for(int k = threadIdx.x; k < n; k += blockDim.x) dst[k] = src[k];
	__syncthreads();
}

// The tables of the systems the nucleotides first .. last of this block belong to, copied into
// dynamic shared memory (a plain run has one system); returns the first of those systems.
// The host sizes the shared memory for the largest span of any block (ForceArgs::tab_span).
template <typename R>
__device__ __forceinline__ int load_table_span(const ForceArgs &a, int first, int last, DNA2Table<R> *s) {
	const int s0 = a.sys ? a.sys[first] : 0;
	const int s1 = a.sys ? a.sys[last] : 0;
	const int n = (s1 - s0 + 1) * (int) (sizeof(DNA2Table<R>) / sizeof(int));
	const int *src = reinterpret_cast<const int *>(reinterpret_cast<const DNA2Table<R> *>(a.table) + s0);
	int *dst = reinterpret_cast<int *>(s);
	for(int k = threadIdx.x; k < n; k += blockDim.x) dst[k] = src[k];
	__syncthreads();
	return s0;
}

extern __shared__ __align__(16) unsigned char g_tables_smem[];

// ---------------------------------------------------------------- particle loaders

struct LoadMixed {
	const float4 *pos_hi, *pos_lo, *fa1, *fa3;
	__device__ __forceinline__ void load(int i, const DNA2Table<float> &P, const int2 b, Nuc<float> &n, float4 &hi,
			float4 &lo) const {
		hi = __ldg(pos_hi + i);
		lo = __ldg(pos_lo + i);
		const float4 x1 = __ldg(fa1 + i), x3 = __ldg(fa3 + i);
		n.a1 = v3<float>{x1.x, x1.y, x1.z};
		n.a3 = v3<float>{x3.x, x3.y, x3.z};
		n.a2 = cross(n.a3, n.a1);
		make_sites(P, n);
		n.btype = __float_as_int(hi.w) >> 22;
		n.type = __float_as_int(lo.w) & 7;
		n.is_end = (b.x < 0 || b.y < 0);
	}
	// minimum image of q - p as hi + lo.  The image m = round(d / box) of a listed pair
	// (|q - p| < r_verlet, far below box / 2) has d / box at least 0.4 from a half-integer, so
	// the product with an approximate inverse rounds to the same integer as the quotient;
	// rounding by the 1.5 * 2^23 addition (|d / box| < 2^22) keeps it on the FMA pipe.
	// The FP32 difference of the hi parts is exact only for coordinates of one sign within a
	// factor of two of each other.  Otherwise -- coordinates on both sides of zero (a few per
	// cent of the nucleotides of a large box, in each dimension), or unwrapped coordinates a box
	// side or more apart -- it rounds at half an ulp of the result (2e-8 for a bonded
	// separation of 0.66, 3.8e-6 across the images of a box of 158), which the stiff excluded
	// volume (force slope up to 1.6e4) turns into force errors of 1e-4 and more.  The exact
	// remainder of the hi difference (two_sum) therefore always joins the low part.  The shift
	// by m box sides is then exact (the result is a small multiple of the ulp of d and of
	// box_hi); the box remainder goes to lo.  sep_soft leaves the remainder out, for
	// Debye-Hueckel and for screening: Debye-Hueckel's force slope is below 0.1, so the 3.8e-6
	// moves its force by less than 1e-6.
	template <bool EXACT = true>
	__device__ __forceinline__ Sep<float> sep(const float4 &ph, const float4 &pl, const float4 &qh, const float4 &ql,
			const DNA2Table<float> &P) const {
		const float qv[3] = {qh.x, qh.y, qh.z}, pv[3] = {ph.x, ph.y, ph.z};
		float d[3], l[3] = {ql.x - pl.x, ql.y - pl.y, ql.z - pl.z};
#pragma unroll
		for(int k = 0; k < 3; k++) {
			if(EXACT) {
				const F2 t = two_sum(qv[k], -pv[k]);
				d[k] = t.s;
				l[k] = __fadd_rn(l[k], t.e);
			}
			else {
				d[k] = qv[k] - pv[k];
			}
		}
#pragma unroll
		for(int k = 0; k < 3; k++) {
			const float m = __fsub_rn(__fmaf_rn(d[k], P.inv_box, 12582912.f), 12582912.f);
			d[k] = fmaf(-m, P.box_hi, d[k]);
			l[k] = fmaf(-m, P.box_lo, l[k]);
		}
		return Sep<float>{v3<float>{d[0], d[1], d[2]}, v3<float>{l[0], l[1], l[2]}};
	}
	__device__ __forceinline__ Sep<float> sep_soft(const float4 &ph, const float4 &pl, const float4 &qh, const float4 &ql,
			const DNA2Table<float> &P) const {
		return sep<false>(ph, pl, qh, ql, P);
	}
	// bonded neighbours: no periodic image; the hi difference's remainder as in sep
	__device__ __forceinline__ Sep<float> diff(const float4 &ph, const float4 &pl, const float4 &qh, const float4 &ql) const {
		const F2 x = two_sum(qh.x, -ph.x), y = two_sum(qh.y, -ph.y), z = two_sum(qh.z, -ph.z);
		return Sep<float>{v3<float>{x.s, y.s, z.s}, v3<float>{__fadd_rn(ql.x - pl.x, x.e), __fadd_rn(ql.y - pl.y, y.e),
				__fadd_rn(ql.z - pl.z, z.e)}};
	}
};

struct LoadDouble {
	const double4_32a *pos, *quat;
	const float4 *meta;  // pos_hi of the mixed layout: w carries btype; lo.w carries the type
	const float4 *meta_lo;
	__device__ __forceinline__ void load(int i, const DNA2Table<double> &P, const int2 b, Nuc<double> &n, double4_32a &ps,
			double4_32a &unused) const {
		ps = pos[i];
		const double4_32a q = quat[i];
		quat_frame(q.x, q.y, q.z, q.w, n.a1, n.a2, n.a3);
		make_sites(P, n);
		n.btype = __float_as_int(meta[i].w) >> 22;
		n.type = __float_as_int(meta_lo[i].w) & 7;
		n.is_end = (b.x < 0 || b.y < 0);
	}
	__device__ __forceinline__ Sep<double> sep(const double4_32a &p, const double4_32a &, const double4_32a &q, const double4_32a &,
			const DNA2Table<double> &P) const {
		double d[3] = {q.x - p.x, q.y - p.y, q.z - p.z};
		const double L = P.box_hi + P.box_lo;
#pragma unroll
		for(int k = 0; k < 3; k++) d[k] = d[k] - rint(d[k] / L) * L;
		return Sep<double>{v3<double>{d[0], d[1], d[2]}, v3<double>{0., 0., 0.}};
	}
	__device__ __forceinline__ Sep<double> diff(const double4_32a &p, const double4_32a &, const double4_32a &q, const double4_32a &) const {
		return Sep<double>{v3<double>{q.x - p.x, q.y - p.y, q.z - p.z}, v3<double>{0., 0., 0.}};
	}
};

struct LoadRef {
	const float4 *pos, *quat;
	__device__ __forceinline__ void load(int i, const DNA2Table<float> &P, const int2 b, Nuc<float> &n, float4 &hi,
			float4 &lo) const {
		hi = pos[i];
		lo = make_float4(0.f, 0.f, 0.f, 0.f);
		const float4 q = quat[i];
		quat_frame(q.x, q.y, q.z, q.w, n.a1, n.a2, n.a3);
		make_sites(P, n);
		n.btype = __float_as_int(hi.w) >> 22;
		n.type = ref_type_of_btype(n.btype);
		n.is_end = (b.x < 0 || b.y < 0);
	}
	__device__ __forceinline__ Sep<float> sep(const float4 &ph, const float4 &, const float4 &qh, const float4 &,
			const DNA2Table<float> &P) const {
		float d[3] = {qh.x - ph.x, qh.y - ph.y, qh.z - ph.z};
#pragma unroll
		for(int k = 0; k < 3; k++) d[k] = fmaf(-rintf(d[k] / P.box_hi), P.box_hi, d[k]);
		return Sep<float>{v3<float>{d[0], d[1], d[2]}, v3<float>{0.f, 0.f, 0.f}};
	}
	__device__ __forceinline__ Sep<float> diff(const float4 &ph, const float4 &, const float4 &qh, const float4 &) const {
		return Sep<float>{v3<float>{qh.x - ph.x, qh.y - ph.y, qh.z - ph.z}, v3<float>{0.f, 0.f, 0.f}};
	}
};

template <typename R>
struct Vec4Of;
template <>
struct Vec4Of<float> {
	using T = float4;
};
template <>
struct Vec4Of<double> {
	using T = double4_32a;
};

// ---------------------------------------------------------------- the kernel

template <typename R, class Loader, bool SPLIT, bool ACCUMULATE>
__global__ void __launch_bounds__(128) k_forces(ForceArgs a, Loader ld) {
	using V4 = typename Vec4Of<R>::T;
	__shared__ DNA2Table<R> P;
	load_table(reinterpret_cast<const DNA2Table<R> *>(a.table), &P);

	const int lane = threadIdx.x & 31;
	const int warps_per_block = blockDim.x >> 5;
	const int gw = blockIdx.x * warps_per_block + (threadIdx.x >> 5);
	const int nw = gridDim.x * warps_per_block;
	V4 *F4 = reinterpret_cast<V4 *>(a.forces);
	V4 *T4 = reinterpret_cast<V4 *>(a.torques);

	for(int i = gw; i < a.N; i += nw) {
		const int2 bi = a.bonds[i];
		Nuc<R> p;
		V4 ph, pl;
		ld.load(i, P, bi, p, ph, pl);

		KahanV<R> F{}, T{};
		R E = R(0), Ec = R(0), Eh = R(0), Ehc = R(0);
		R split[N_TERMS];
		if(SPLIT) {
#pragma unroll
			for(int k = 0; k < N_TERMS; k++) split[k] = R(0);
		}

		// bonded pairs: lane 0 the 3' neighbour (p = i), lane 1 the 5' neighbour (q = i)
		if(lane < 2) {
			const int j = (lane == 0) ? bi.x : bi.y;
			if(j >= 0) {
				const int2 bj = a.bonds[j];
				Nuc<R> q;
				V4 qh, ql;
				ld.load(j, P, bj, q, qh, ql);
				PairOut<R> o{};
				bool ok;
				if(lane == 0) ok = bonded<R, SPLIT, false>(P, p, q, ld.diff(ph, pl, qh, ql), o);
				else ok = bonded<R, SPLIT, true>(P, q, p, ld.diff(qh, ql, ph, pl), o);
				if(!ok) atomicOr(a.status, OXGB_ERR_FENE);
				F.add(o.F);
				T.add(o.T);
				KahanV<R>::kadd(E, Ec, o.E);
				if(SPLIT) {
#pragma unroll
					for(int k = 0; k < N_TERMS; k++) split[k] += o.split[k];
				}
			}
		}

		const int nn = a.nnb[i];
		if(nn > a.max_nb) atomicOr(a.status, OXGB_ERR_NEIGH_OVERFLOW);
		const int nlim = nn < a.max_nb ? nn : a.max_nb;
		const long long row = (long long) i * a.nb_stride_i;
		for(int k = lane; k < nlim; k += 32) {
			const int j = a.nb[row + (long long) k * a.nb_stride_k];
			if(j == i || j == bi.x || j == bi.y) continue;
			const int2 bj = a.bonds[j];
			Nuc<R> q;
			V4 qh, ql;
			ld.load(j, P, bj, q, qh, ql);
			PairOut<R> o{};
			nonbonded_p<R, SPLIT>(P, p, q, ld.sep(ph, pl, qh, ql, P), o);
			F.add(o.F);
			T.add(o.T);
			KahanV<R>::kadd(E, Ec, o.E);
			KahanV<R>::kadd(Eh, Ehc, o.Ehb);
			if(SPLIT) {
#pragma unroll
				for(int k2 = 0; k2 < N_TERMS; k2++) split[k2] += o.split[k2];
			}
		}

		const R fx = warp_sum_comp(F.s.x, F.c.x), fy = warp_sum_comp(F.s.y, F.c.y), fz = warp_sum_comp(F.s.z, F.c.z);
		const R tx = warp_sum_comp(T.s.x, T.c.x), ty = warp_sum_comp(T.s.y, T.c.y), tz = warp_sum_comp(T.s.z, T.c.z);
		const R e = warp_sum_comp(E, Ec), eh = warp_sum_comp(Eh, Ehc);
		if(SPLIT) {
#pragma unroll
			for(int k = 0; k < N_TERMS; k++) split[k] = warp_sum_comp(split[k], R(0));
		}
		if(lane == 0) {
			const v3<R> tl{tx, ty, tz};
			// body frame: components along a1, a2, a3
			const R bx = dot(p.a1, tl), by = dot(p.a2, tl), bz = dot(p.a3, tl);
			V4 fo, to;
			if(ACCUMULATE) {
				fo = F4[i];
				to = T4[i];
				fo.x += fx;
				fo.y += fy;
				fo.z += fz;
				fo.w += e;
				to.x += bx;
				to.y += by;
				to.z += bz;
				to.w = eh;
			}
			else {
				fo.x = fx;
				fo.y = fy;
				fo.z = fz;
				fo.w = e;
				to.x = bx;
				to.y = by;
				to.z = bz;
				to.w = eh;
			}
			F4[i] = fo;
			T4[i] = to;
			if(SPLIT) {
#pragma unroll
				for(int k = 0; k < N_TERMS; k++) atomicAdd(a.esplit + k, 0.5 * (double) split[k]);
			}
		}
	}
}

// ---------------------------------------------------------------- host launchers

static int grid_for(int N, int warps_per_block) {
	const int blocks = (N + warps_per_block - 1) / warps_per_block;
	return blocks > 0 ? blocks : 1;
}

cudaError_t launch_forces_reference_layout(const ForceArgs &a, cudaStream_t s) {
	LoadRef ld{a.pos_hi, a.quat};
	k_forces<float, LoadRef, false, true><<<grid_for(a.N, 4), 128, 0, s>>>(a, ld);
	return cudaGetLastError();
}

// FFS order parameters on the reference layout (hb_op_precalc, near_hb_op_precalc and
// dist_op_precalc, src/CUDA/Interactions/CUDA_DNA.cuh:910-1067): one thread per listed pair
// (op1[k], op2[k]), centre separation at its FP32 minimum image, base sites at POS_BASE a1.
//   MODE 0: the pair's hydrogen-bonding energy f1 f4(t1) f4(t2) f4(t3) f4(t4) f4(t7) f4(t8)
//           (no hb_multiplier, as the reference's kernel), 0 unless the bases are complementary
//           and their distance is inside the hydrogen-bonding window;
//   MODE 1: "nearly bonded": at least six of those seven factors on (f1 < 0, each f4 > 0);
//   MODE 2: the base-base distance.
template <int MODE>
__global__ void k_order_params(const float4 *poss, const float4 *quat, const int *op1, const int *op2, int n,
		const DNA2Table<float> *table, float *val, bool *flag) {
	__shared__ DNA2Table<float> P;
	load_table(table, &P);
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= n) return;
	const LoadRef ld{poss, quat};
	Nuc<float> p, q;
	float4 ph, pl, qh, ql;
	ld.load(op1[k], P, make_int2(0, 0), p, ph, pl);
	ld.load(op2[k], P, make_int2(0, 0), q, qh, ql);
	const v3<float> rb = site_vec(ld.sep(ph, pl, qh, ql, P), q.base, p.base);
	const float r2 = dot(rb, rb);
	if(MODE == 2) {
		val[k] = m_sqrt(r2);
		return;
	}
	float e = 0.f;
	bool near = false;
	if(p.btype + q.btype == 3 && float(OXM_HYDR_RCLOW) * float(OXM_HYDR_RCLOW) < r2 &&
			r2 < float(OXM_HYDR_RCHIGH) * float(OXM_HYDR_RCHIGH)) {
		const float rmod = m_sqrt(r2);
		const v3<float> rd = rb * (1.f / rmod);
		float f1, f1d, g[6], gd;
		f1_both(P, rmod, OXM_F1_HB, p.type, q.type, f1, f1d);
		f4_both(P, -dot(p.a1, q.a1), sin_between(p.a1, q.a1), OXM_F4_HB_T1, g[0], gd);
		f4_both(P, -dot(q.a1, rd), sin_between(q.a1, rd), OXM_F4_HB_T2, g[1], gd);
		f4_both(P, dot(p.a1, rd), sin_between(p.a1, rd), OXM_F4_HB_T2, g[2], gd);
		f4_both(P, dot(p.a3, q.a3), sin_between(p.a3, q.a3), OXM_F4_HB_T4, g[3], gd);
		f4_both(P, -dot(rd, q.a3), sin_between(q.a3, rd), OXM_F4_HB_T7, g[4], gd);
		f4_both(P, dot(rd, p.a3), sin_between(p.a3, rd), OXM_F4_HB_T7, g[5], gd);
		e = f1;
		int on = f1 < 0.f;
#pragma unroll
		for(int m = 0; m < 6; m++) {
			e *= g[m];
			on += g[m] > 0.f;
		}
		near = on >= 6;
	}
	if(MODE == 0) val[k] = e;
	else flag[k] = near;
}

cudaError_t launch_order_params(int mode, const float4 *poss, const float4 *quat, const int *op1, const int *op2, int n,
		const void *table, float *val, bool *flag, cudaStream_t s) {
	const int blocks = (n + 127) / 128;
	const DNA2Table<float> *t = reinterpret_cast<const DNA2Table<float> *>(table);
	if(mode == 0) k_order_params<0><<<blocks, 128, 0, s>>>(poss, quat, op1, op2, n, t, val, flag);
	else if(mode == 1) k_order_params<1><<<blocks, 128, 0, s>>>(poss, quat, op1, op2, n, t, val, flag);
	else k_order_params<2><<<blocks, 128, 0, s>>>(poss, quat, op1, op2, n, t, val, flag);
	return cudaGetLastError();
}

}  // namespace oxgb

// ====================================================================== split path
//
// The warp-per-nucleotide kernel above leaves most lanes idle: a nucleotide has ~20-30
// neighbours, only a few of them close enough for hydrogen bonding, cross or coaxial
// stacking, and the two bonded pairs ran on two lanes.  The split path instead
//  * evaluates every bonded pair once, one thread per bond, for both nucleotides;
//  * runs the non-bonded terms one thread per nucleotide, one loop per term over the term
//    lists of the Verlet build (full rows for Debye-Hueckel, centre-close pairs for the
//    excluded volume, base-close pairs for hydrogen bonding + cross stacking, stack-close
//    pairs for coaxial stacking), so all lanes of a warp run the same term code;
//  * gathers the bonded results in the non-bonded kernel's epilogue (fixed order, no atomics).

namespace oxgb {

// the remainders of nucleotide k's a1 and backbone offset (written with the mirrors)
__device__ __forceinline__ SiteLo site_lo(const float4 *a1lo, const float4 *backlo, int k) {
	const float4 u = __ldg(a1lo + k), v = __ldg(backlo + k);
	return SiteLo{v3<float>{u.x, u.y, u.z}, v3<float>{v.x, v.y, v.z}};
}

// the refined excluded volume of a stiff bonded contact (rare): out of line, so that the kernel's
// register allocation stays that of its common path
template <int K>
__device__ __noinline__ float ev_refined_call(const float4 *a1lo, const float4 *backlo, int i, int j, Sep<float> sep,
		v3<float> ps, v3<float> pa1, int pbase, v3<float> qs, v3<float> qa1, int qbase, v3<float> *f) {
	v3<float> fo;
	const float e = ev_refined<K>(sep, ps, pa1, site_lo(a1lo, backlo, i), pbase, qs, qa1, site_lo(a1lo, backlo, j), qbase, fo);
	*f = fo;
	return e;
}

// a non-bonded pair with a site pair inside its excluded-volume cutoff, refined: force and torque
// on nucleotide i (of p) and the energy (rare; out of line, so that the non-bonded kernel's loops
// keep their register allocation)
__device__ __noinline__ float4 ev_pair_refined_call(const float4 *a1lo, const float4 *backlo, int i, int j, float4 sh,
		float4 sl, float4 pb, float4 pk, float4 pa, float4 qb, float4 qk, float4 qa, float3 *T) {
	Nuc<float> p, q;
	p.back = v3<float>{pb.x, pb.y, pb.z}, p.base = v3<float>{pk.x, pk.y, pk.z}, p.a1 = v3<float>{pa.x, pa.y, pa.z};
	q.back = v3<float>{qb.x, qb.y, qb.z}, q.base = v3<float>{qk.x, qk.y, qk.z}, q.a1 = v3<float>{qa.x, qa.y, qa.z};
	const Sep<float> sep{v3<float>{sh.x, sh.y, sh.z}, v3<float>{sl.x, sl.y, sl.z}};
	v3<float> F{0.f, 0.f, 0.f}, t{0.f, 0.f, 0.f};
	const float e = pair_ev_refined(sep, p, site_lo(a1lo, backlo, i), q, site_lo(a1lo, backlo, j), F, t);
	*T = make_float3(t.x, t.y, t.z);
	return make_float4(F.x, F.y, F.z, e);
}

// refines the FP32 engine path for pair (i, j): the site offsets' remainders for the stiff
// radial factors, and the stiff excluded-volume contacts
struct StoredLo {
	static constexpr bool on = true;
	const float4 *a1lo, *backlo;
	int i, j;
	__device__ __forceinline__ SiteLo lo(int which) const { return site_lo(a1lo, backlo, which ? j : i); }
	template <int K>
	__device__ __forceinline__ float ev(const Sep<float> &sep, v3<float> ps, v3<float> pa1, int pbase, v3<float> qs,
			v3<float> qa1, int qbase, v3<float> &f) const {
		return ev_refined_call<K>(a1lo, backlo, i, j, sep, ps, pa1, pbase, qs, qa1, qbase, &f);
	}
};

struct SplitMixed {
	const float4 *hi, *lo, *fa1, *fa3, *fback;
	const float4 *a1lo, *backlo;  // remainders of fa1 / fback (StoredLo)
	__device__ __forceinline__ StoredLo refine(int i, int j) const { return StoredLo{a1lo, backlo, i, j}; }
	__device__ __forceinline__ void full(int j, Nuc<float> &n, float4 &h, float4 &l) const {
		h = __ldg(hi + j);
		l = __ldg(lo + j);
		const float4 x1 = __ldg(fa1 + j), x3 = __ldg(fa3 + j), bk = __ldg(fback + j);
		n.a1 = v3<float>{x1.x, x1.y, x1.z};
		n.a3 = v3<float>{x3.x, x3.y, x3.z};
		n.a2 = cross(n.a3, n.a1);
		n.back = v3<float>{bk.x, bk.y, bk.z};
		n.stack = n.a1 * float(OXM_POS_STACK);
		n.base = n.a1 * float(OXM_POS_BASE);
		n.btype = __float_as_int(h.w) >> 22;
		n.type = __float_as_int(l.w) & 7;
		n.is_end = bk.w != 0.f;
	}
	__device__ __forceinline__ void dh(int j, Nuc<float> &n, float4 &h, float4 &l) const {
		h = __ldg(hi + j);
		l = __ldg(lo + j);
		const float4 bk = __ldg(fback + j);
		n.back = v3<float>{bk.x, bk.y, bk.z};
		n.is_end = bk.w != 0.f;
	}
	__device__ __forceinline__ Sep<float> sep(const float4 &ph, const float4 &pl, const float4 &qh, const float4 &ql,
			const DNA2Table<float> &P) const {
		return LoadMixed{}.sep(ph, pl, qh, ql, P);
	}
	__device__ __forceinline__ Sep<float> sep_soft(const float4 &ph, const float4 &pl, const float4 &qh, const float4 &ql,
			const DNA2Table<float> &P) const {
		return LoadMixed{}.sep_soft(ph, pl, qh, ql, P);
	}
	__device__ __forceinline__ Sep<float> diff(const float4 &ph, const float4 &pl, const float4 &qh, const float4 &ql) const {
		return LoadMixed{}.diff(ph, pl, qh, ql);
	}
};

struct SplitDouble {
	const double4_32a *pos, *quat;
	const float4 *meta, *meta_lo;
	const int2 *bonds;
	__device__ __forceinline__ NoRefine refine(int, int) const { return NoRefine{}; }
	__device__ __forceinline__ Sep<double> sep(const double4_32a &p, const double4_32a &, const double4_32a &q,
			const double4_32a &, const DNA2Table<double> &P) const {
		return LoadDouble{}.sep(p, p, q, q, P);
	}
	__device__ __forceinline__ Sep<double> sep_soft(const double4_32a &p, const double4_32a &, const double4_32a &q,
			const double4_32a &, const DNA2Table<double> &P) const {
		return LoadDouble{}.sep(p, p, q, q, P);
	}
	__device__ __forceinline__ Sep<double> diff(const double4_32a &p, const double4_32a &, const double4_32a &q,
			const double4_32a &) const {
		return LoadDouble{}.diff(p, p, q, q);
	}
};

// FP64 loads need the table (for the base-site ratio), so the double loader takes it explicitly
template <class Loader, typename R>
__device__ __forceinline__ void load_full(const Loader &ld, int j, const DNA2Table<R> &P, Nuc<R> &n,
		typename Vec4Of<R>::T &h, typename Vec4Of<R>::T &l);
template <>
__device__ __forceinline__ void load_full<SplitMixed, float>(const SplitMixed &ld, int j, const DNA2Table<float> &, Nuc<float> &n,
		float4 &h, float4 &l) {
	ld.full(j, n, h, l);
}
template <>
__device__ __forceinline__ void load_full<SplitDouble, double>(const SplitDouble &ld, int j, const DNA2Table<double> &P,
		Nuc<double> &n, double4_32a &h, double4_32a &l) {
	LoadDouble{ld.pos, ld.quat, ld.meta, ld.meta_lo}.load(j, P, ld.bonds[j], n, h, l);
}
template <class Loader, typename R>
__device__ __forceinline__ void load_dh(const Loader &ld, int j, const DNA2Table<R> &P, Nuc<R> &n, typename Vec4Of<R>::T &h,
		typename Vec4Of<R>::T &l) {
	load_full<Loader, R>(ld, j, P, n, h, l);
}
template <>
__device__ __forceinline__ void load_dh<SplitMixed, float>(const SplitMixed &ld, int j, const DNA2Table<float> &, Nuc<float> &n,
		float4 &h, float4 &l) {
	ld.dh(j, n, h, l);
}

// bonded block b: one bond (owner p, partner q = n3[p]) per thread; the bonded blocks cover
// every nucleotide
template <typename R, class Loader, bool SPLIT, bool ENERGY>
__device__ __forceinline__ void bonded_block(const ForceArgs &a, const Loader &ld, int b) {
	using V4 = typename Vec4Of<R>::T;
	const int first = b * blockDim.x;
	DNA2Table<R> *Ps = reinterpret_cast<DNA2Table<R> *>(g_tables_smem);
	const int s0 = load_table_span<R>(a, first, min(first + (int) blockDim.x, a.N) - 1, Ps);
	// an MD step: from here on its second half kick is pending (the first step has read the mark)
	if(a.th.open_step && b == 0 && threadIdx.x == 0) *a.th.open_step = *a.th.step_base + a.th.step_offset;
	const int p = first + threadIdx.x;
	if(p < a.N) {
		const int q = a.bonds[p].x;
		if(q < 0) return;
		const int sy = a.sys ? a.sys[p] : 0;
		const DNA2Table<R> &P = Ps[sy - s0];
		Nuc<R> np, nq;
		V4 ph, pl, qh, ql;
		load_full<Loader, R>(ld, p, P, np, ph, pl);
		load_full<Loader, R>(ld, q, P, nq, qh, ql);
		BondOut<R> b;
		if(!bonded_both(P, np, nq, ld.diff(ph, pl, qh, ql), b, ld.refine(p, q))) atomicOr(a.status, OXGB_ERR_FENE);
		V4 f, tp, tq;
		f.x = b.f.x, f.y = b.f.y, f.z = b.f.z, f.w = ENERGY ? b.E : R(0);
		tp.x = b.tp.x, tp.y = b.tp.y, tp.z = b.tp.z, tp.w = R(0);
		tq.x = b.tq.x, tq.y = b.tq.y, tq.z = b.tq.z, tq.w = R(0);
		reinterpret_cast<V4 *>(a.bond_f)[p] = f;
		reinterpret_cast<V4 *>(a.bond_tp)[p] = tp;
		reinterpret_cast<V4 *>(a.bond_tq)[p] = tq;
		if(SPLIT) {
			atomicAdd(a.esplit + 8 * sy + T_FENE, (double) b.split[0]);
			atomicAdd(a.esplit + 8 * sy + T_BEXC, (double) b.split[1]);
			atomicAdd(a.esplit + 8 * sy + T_STCK, (double) b.split[2]);
		}
	}
}

// per-lane compensated sums of a nucleotide's pair terms; ENERGY = false leaves the energies out
// (an MD step needs only forces and torques: the energy arithmetic of the pair functions is then
// dead code)
// Terms of bounded size (Debye-Hueckel, excluded volume) go to a plain per-lane sum when
// OXGB_NB_PLAIN_SHORT is set: a lane adds only a few of them, whose rounding is far below the
// compensated sums of the large bonded and pair terms; they join the compensated sum before the
// group reduction.
#ifndef OXGB_NB_PLAIN_SHORT
#define OXGB_NB_PLAIN_SHORT 0
#endif

template <typename R, bool SPLIT, bool ENERGY = true>
struct SplitAcc {
	KahanV<R> F, T;
	v3<R> Fp, Tp;
	R E, Ec, Eh, Ehc;
	R split[N_TERMS];
	__device__ __forceinline__ void add_short(const PairOut<R> &o) {
		if(!OXGB_NB_PLAIN_SHORT) {
			add(o);
			return;
		}
		Fp = Fp + o.F;
		Tp = Tp + o.T;
		if(ENERGY) {
			KahanV<R>::kadd(E, Ec, o.E);
			KahanV<R>::kadd(Eh, Ehc, o.Ehb);
		}
		if(SPLIT) {
#pragma unroll
			for(int k = 0; k < N_TERMS; k++) split[k] += o.split[k];
		}
	}
	__device__ __forceinline__ void fold_short() {
		if(OXGB_NB_PLAIN_SHORT) {
			F.add(Fp);
			T.add(Tp);
		}
	}
	__device__ __forceinline__ void add(const PairOut<R> &o) {
		F.add(o.F);
		T.add(o.T);
		if(ENERGY) {
			KahanV<R>::kadd(E, Ec, o.E);
			KahanV<R>::kadd(Eh, Ehc, o.Ehb);
		}
		if(SPLIT) {
#pragma unroll
			for(int k = 0; k < N_TERMS; k++) split[k] += o.split[k];
		}
	}
	// entry k of nucleotide i's list: its result, written by the pair blocks of k_bonded_pairs
	template <typename V4>
	__device__ __forceinline__ void add_slot(const V4 *res, long long N, int i, int k) {
		const long long s = (long long) k * N + i;
		const V4 f = res[2 * s], t = res[2 * s + 1];
		F.add(v3<R>{f.x, f.y, f.z});
		T.add(v3<R>{t.x, t.y, t.z});
		if(ENERGY) {
			KahanV<R>::kadd(E, Ec, f.w);
			KahanV<R>::kadd(Eh, Ehc, t.w);
		}
	}
};

// Base-base pairs (hydrogen bonding + cross stacking; blocks 0 .. base_blocks - 1) and
// stack-stack pairs (coaxial stacking; the other blocks), each evaluated once, by its lower
// nucleotide i (partner j above i by caller's index, at position k of i's list and m of j's): slot k of i gets
// (force on i, E), (torque on i, E_hb) and slot m of j gets (-force, E), (torque on j, E_hb), at
// [2 (k N + i) + 0..1] of base_res / stk_res.  Every slot of every list is written by its pair
// alone.  These are the costliest terms and their lists are short, so the owned slots of a
// warp's nucleotides are queued (a warp prefix sum over the per-lane counts) and dealt 32 at a
// time: every lane works on a pair in every round but the last.
// nucleotides per warp in a pair block: a full warp (32) fills each queue round with the most
// pairs; measured against 16 it is faster by 1.0 us per force launch at 40k and 12.5 us on
// the 250k melt (8 is slower still)
#ifndef OXGB_PAIR_NPW
#define OXGB_PAIR_NPW 32
#endif

__device__ __forceinline__ void atomic_add_v4(float4 *p, const float4 &v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_v4(double4_32a *p, const double4_32a &v) {
	atomicAdd(&p->x, v.x);
	atomicAdd(&p->y, v.y);
	atomicAdd(&p->z, v.z);
	atomicAdd(&p->w, v.w);
}

// one term (0 hydrogen bonding, 1 cross stacking, 2 coaxial stacking; warp-uniform) of the
// queued pairs t[0 .. n - 1], lane l taking t[l]: the pair's result is added to its two slots
// (zeroed when the pair was screened).  A slot receives at most two terms (hydrogen bonding and
// cross stacking of one pair), whose sum does not depend on their order.  Not inlined: it is
// called from several places, and one compiled copy gives a pair the same rounding wherever
// its batch is evaluated (inlined copies may contract products into FMAs differently); the term
// is evaluated only if this copy's own screening admits it.
template <typename R, class Loader, bool SPLIT, bool ENERGY>
__device__ __noinline__ void eval_terms(const ForceArgs &a, const Loader &ld, const DNA2Table<R> *Ps, int s0,
		const int4 *t, int n, int term) {
	using V4 = typename Vec4Of<R>::T;
	const int lane = threadIdx.x & 31;
	if(lane >= n) return;
	const int4 it = t[lane];
	const int i = it.x, j = it.y, k = it.z, m = it.w;
	const long long N = a.N;
	const int sy = a.sys ? a.sys[i] : 0;
	const DNA2Table<R> &P = Ps[sy - s0];
	Nuc<R> p, qn;
	V4 ph, pl, qh, ql;
	load_full<Loader, R>(ld, i, P, p, ph, pl);
	load_full<Loader, R>(ld, j, P, qn, qh, ql);
	const Sep<R> d = ld.sep(ph, pl, qh, ql, P);
	PairOut<R> o{};
	// FP32 engine path: the remainder of the site distance (the stiff radial factors, see rdiff)
	const auto x = ld.refine(i, j);
	if(term == 2) {
		const StackGeo<R> g = stack_geo(P, p, qn, d);
		R rl = R(0);
		if constexpr(decltype(x)::on) {
			if(g.cxst) rl = site_dist_remainder(d, p, x.lo(0), qn, x.lo(1), true, g.rmod);
		}
		if(g.cxst) cxst_term<R, SPLIT>(P, p, qn, g, o, rl);
	}
	else {
		const BaseGeo<R> g = base_geo(P, p, qn, d);
		R rl = R(0);
		if constexpr(decltype(x)::on) {
			if((term == 0 && g.hb) || (term == 1 && g.crst)) rl = site_dist_remainder(d, p, x.lo(0), qn, x.lo(1), false, g.rmod);
		}
		if(term == 0 && g.hb) hb_term<R, SPLIT>(P, p, qn, g, o, rl);
		if(term == 1 && g.crst) crst_term<R, SPLIT>(P, p, qn, g, o, rl);
	}
	// the potential is invariant under rigid rotations, so the torques balance:
	// T_j = -T_i + (r_j - r_i) x F_i, the cross product with error-free products
	const v3<R> c = cross_accurate(d, o.F);
	V4 fi, ti, fj, tj;
	fi.x = o.F.x, fi.y = o.F.y, fi.z = o.F.z, fi.w = ENERGY ? o.E : R(0);
	ti.x = o.T.x, ti.y = o.T.y, ti.z = o.T.z, ti.w = ENERGY ? o.Ehb : R(0);
	fj.x = -o.F.x, fj.y = -o.F.y, fj.z = -o.F.z, fj.w = fi.w;
	tj.x = c.x - o.T.x, tj.y = c.y - o.T.y, tj.z = c.z - o.T.z, tj.w = ti.w;
	V4 *res = reinterpret_cast<V4 *>(term == 2 ? a.stk_res : a.base_res);
	atomic_add_v4(res + 2 * ((long long) k * N + i), fi);
	atomic_add_v4(res + 2 * ((long long) k * N + i) + 1, ti);
	if(m >= 0) {  // (a missing position is flagged by the list build)
		atomic_add_v4(res + 2 * ((long long) m * N + j), fj);
		atomic_add_v4(res + 2 * ((long long) m * N + j) + 1, tj);
	}
	if(SPLIT) {
#pragma unroll
		for(int u = 0; u < N_TERMS; u++)
			if(o.split[u] != R(0)) atomicAdd(a.esplit + 8 * sy + u, (double) o.split[u]);
	}
}

// Pair block b: base-base pairs (hydrogen bonding + cross stacking; blocks 0 .. base_blocks -
// 1) or stack-stack pairs (coaxial stacking; the other blocks).  Each warp deals the owned pairs
// of its nucleotides 32 at a time (as above) and screens them (base_geo / stack_geo: distance
// windows and angular supports); only about a third of the pairs has a non-zero term, so the
// live terms go to per-warp queues in shared memory and are evaluated 32 at a time, every lane
// on the same term, instead of on the few lanes of each round whose pair happens to be live.
template <typename R, class Loader, bool SPLIT, bool ENERGY, int NPW>
__device__ __forceinline__ void pair_block(const ForceArgs &a, const Loader &ld, int b, int base_blocks) {
	using V4 = typename Vec4Of<R>::T;
	__shared__ int4 tq[4][2][64];  // per warp: live hydrogen-bonding (or coaxial) and cross-stacking terms
	const bool is_base = b < base_blocks;
	const int per_block = (blockDim.x / 32) * NPW;
	const int first = (is_base ? b : b - base_blocks) * per_block;
	DNA2Table<R> *Ps = reinterpret_cast<DNA2Table<R> *>(g_tables_smem);
	const int s0 = load_table_span<R>(a, first, min(first + per_block, a.N) - 1, Ps);
	const long long N = a.N;
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	const int wbase = first + w * NPW;
	if(wbase >= a.N) return;  // warp-uniform
	const int cap = is_base ? a.base_cap : a.stk_cap;
	const int *nb = is_base ? a.base_nb : a.stk_nb;
	V4 *res = reinterpret_cast<V4 *>(is_base ? a.base_res : a.stk_res);
	// this lane's nucleotide (lanes below NPW): which of its entries it owns (partner above
	// it by caller's index), as a bit mask
	const int il = wbase + lane;
	unsigned lo = 0u, hi = 0u;
	if(lane < NPW && il < a.N) {
		const int n = min(min(is_base ? a.base_n[il] : a.stk_n[il], cap), 64);
		const int key = a.id ? a.id[il] : il;
		for(int k = 0; k < n; k++) {
			const int j = nb[(long long) k * N + il];
			if((a.id ? a.id[j] : j) > key) {
				if(k < 32) lo |= 1u << k;
				else hi |= 1u << (k - 32);
			}
		}
	}
	const int own = __popc(lo) + __popc(hi);
	int incl = own;
#pragma unroll
	for(int off = 1; off < 32; off <<= 1) {
		const int u = __shfl_up_sync(0xffffffffu, incl, off);
		if(lane >= off) incl += u;
	}
	const int total = __shfl_sync(0xffffffffu, incl, 31);
	const int excl = incl - own;
	const unsigned below = (1u << lane) - 1u;
	int n0 = 0, n1 = 0;  // queued terms (warp-uniform)
	const int term0 = is_base ? 0 : 2;
	for(int q0 = 0; q0 < total; q0 += 32) {
		const int q = q0 + lane;
		// the lane that owns queue entry q: the first whose inclusive count exceeds q
		int l = 0;
#pragma unroll
		for(int step = 16; step > 0; step >>= 1) {
			const int v = __shfl_sync(0xffffffffu, incl, l + step - 1);
			if(v <= q) l += step;
		}
		const int ex_l = __shfl_sync(0xffffffffu, excl, l & 31);
		const unsigned lo_l = __shfl_sync(0xffffffffu, lo, l & 31), hi_l = __shfl_sync(0xffffffffu, hi, l & 31);
		bool live0 = false, live1 = false;
		int4 item = make_int4(0, 0, 0, -1);
		if(q < total) {
			// the r-th owned entry of nucleotide i
			const int r = q - ex_l, nlo = __popc(lo_l);
			const int k = r < nlo ? (int) __fns(lo_l, 0u, r + 1) : 32 + (int) __fns(hi_l, 0u, r - nlo + 1);
			const int i = wbase + l;
			const int j = nb[(long long) k * N + i];
			const int m = (is_base ? a.base_pos : a.stk_pos)[(long long) k * N + i];
			const int sy = a.sys ? a.sys[i] : 0;
			const DNA2Table<R> &P = Ps[sy - s0];
			Nuc<R> p, qn;
			V4 ph, pl, qh, ql;
			load_full<Loader, R>(ld, i, P, p, ph, pl);
			load_full<Loader, R>(ld, j, P, qn, qh, ql);
			const Sep<R> d = ld.sep(ph, pl, qh, ql, P);
			if(is_base) {
				const BaseGeo<R> g = base_geo(P, p, qn, d);
				live0 = g.hb;
				live1 = g.crst;
			}
			else {
				live0 = stack_geo(P, p, qn, d).cxst;
			}
			// both slots start from zero; the live terms add into them
			V4 z;
			z.x = z.y = z.z = z.w = R(0);
			res[2 * ((long long) k * N + i)] = z;
			res[2 * ((long long) k * N + i) + 1] = z;
			if(m >= 0) {
				res[2 * ((long long) m * N + j)] = z;
				res[2 * ((long long) m * N + j) + 1] = z;
			}
			item = make_int4(i, j, k, m);
		}
		const unsigned b0 = __ballot_sync(0xffffffffu, live0), b1 = __ballot_sync(0xffffffffu, live1);
		if(live0) tq[w][0][n0 + __popc(b0 & below)] = item;
		if(live1) tq[w][1][n1 + __popc(b1 & below)] = item;
		n0 += __popc(b0);
		n1 += __popc(b1);
		__syncwarp();  // the queued items and the zeroed slots are visible to the whole warp
		if(n0 >= 32) {
			n0 -= 32;
			eval_terms<R, Loader, SPLIT, ENERGY>(a, ld, Ps, s0, tq[w][0] + n0, 32, term0);
			__syncwarp();
		}
		if(n1 >= 32) {
			n1 -= 32;
			eval_terms<R, Loader, SPLIT, ENERGY>(a, ld, Ps, s0, tq[w][1] + n1, 32, 1);
			__syncwarp();
		}
	}
	if(n0 > 0) eval_terms<R, Loader, SPLIT, ENERGY>(a, ld, Ps, s0, tq[w][0], n0, term0);
	if(n1 > 0) eval_terms<R, Loader, SPLIT, ENERGY>(a, ld, Ps, s0, tq[w][1], n1, 1);
}

// minimum resident blocks per SM asked of the register allocator for the bonded/pair kernel
#ifndef OXGB_PAIR_MINB
#define OXGB_PAIR_MINB 5
#endif


// compensated sum over the K lanes of a group (TwoSum at every level); every lane of the group
// receives it
template <typename R, int K>
__device__ __forceinline__ R group_sum_comp(R s, R c) {
	R err = -c;
#pragma unroll
	for(int off = K / 2; off > 0; off >>= 1) {
		const R so = __shfl_xor_sync(0xffffffffu, s, off, K);
		const R eo = __shfl_xor_sync(0xffffffffu, err, off, K);
		const R t = s + so;
		const R bp = t - s;
		const R e2 = (s - (t - bp)) + (so - bp);
		s = t;
		err += eo + e2;
	}
	return s + err;
}

// Edge block b (use_edge): K lanes per nucleotide i take the entries of its full row and of its
// excluded-volume list whose partner j lies above i (by slot), so every unordered pair is
// evaluated once -- the pair-parallel scheme of the reference's use_edge kernels
// (CUDA_DNA.cuh:727-775), with a nucleotide's pairs kept on one lane group.  The partner's
// share goes to edge_acc[j] by atomic vector adds (force with energy, lab torque), the
// nucleotide's own share to edge_acc[i] after a compensated group sum; the non-bonded kernel
// gathers edge_acc.  The partner's Debye-Hueckel torque is its backbone offset times its force;
// the excluded volume's follows from the rigid-rotation balance T_j = -T_i + d x F_i (error-free
// products).  Atomic adds make the summation order, and so the last bits, vary from run to run.
template <typename R, class Loader, bool SPLIT, bool ENERGY, int K>
__device__ __forceinline__ void edge_block(const ForceArgs &a, const Loader &ld, int b) {
	using V4 = typename Vec4Of<R>::T;
	const long long N = a.N;
	const int sub = threadIdx.x % K;
	const int per_block = blockDim.x / K;
	const int first = b * per_block;
	DNA2Table<R> *Ps = reinterpret_cast<DNA2Table<R> *>(g_tables_smem);
	const int s0 = load_table_span<R>(a, first, min(first + per_block, a.N) - 1, Ps);
	const int i_raw = first + (int) threadIdx.x / K;
	const bool live = i_raw < a.N;
	const int i = live ? i_raw : a.N - 1;
	const int sy = a.sys ? a.sys[i] : 0;
	const DNA2Table<R> &P = Ps[sy - s0];
	Nuc<R> p;
	V4 ph, pl;
	load_full<Loader, R>(ld, i, P, p, ph, pl);
	SplitAcc<R, SPLIT, ENERGY> acc{};
	V4 *out = reinterpret_cast<V4 *>(a.edge_acc);
	auto partner = [&](int j, const v3<R> &fj, const v3<R> &tj, R e) {
		V4 f, t;
		f.x = fj.x, f.y = fj.y, f.z = fj.z, f.w = ENERGY ? e : R(0);
		t.x = tj.x, t.y = tj.y, t.z = tj.z, t.w = R(0);
		atomic_add_v4(out + 2 * (long long) j, f);
		atomic_add_v4(out + 2 * (long long) j + 1, t);
	};
	// Debye-Hueckel over the owned entries of the full row
	const int ndh = live ? min(a.nnb[i], a.max_nb) : 0;
	for(int k = sub; k < ndh; k += K) {
		const int j = a.nb[(long long) k * N + i];
		if(j < i) continue;
		Nuc<R> q;
		V4 qh, ql;
		load_dh<Loader, R>(ld, j, P, q, qh, ql);
		PairOut<R> o{};
		pair_dh<R, SPLIT>(P, p, q, ld.sep_soft(ph, pl, qh, ql, P).plain(), o);
		acc.add(o);
		if(o.F.x != R(0) || o.F.y != R(0) || o.F.z != R(0)) partner(j, -o.F, cross(q.back, -o.F), o.E);
	}
	// excluded volume over the owned centre-close pairs
	const int nev = live ? min(a.ev_n[i], a.ev_cap) : 0;
	for(int k = sub; k < nev; k += K) {
		const int j = a.ev_nb[(long long) k * N + i];
		if(j < i) continue;
		Nuc<R> q;
		V4 qh, ql;
		load_full<Loader, R>(ld, j, P, q, qh, ql);
		PairOut<R> o{};
		const Sep<R> sp = ld.sep(ph, pl, qh, ql, P);
		if constexpr(decltype(ld.refine(0, 0))::on) {
			if(!ev_contact(p, q, sp.plain())) continue;
			float3 t;
			const float4 fe = ev_pair_refined_call(ld.a1lo, ld.backlo, i, j, make_float4(sp.hi.x, sp.hi.y, sp.hi.z, 0.f),
					make_float4(sp.lo.x, sp.lo.y, sp.lo.z, 0.f), make_float4(p.back.x, p.back.y, p.back.z, 0.f),
					make_float4(p.base.x, p.base.y, p.base.z, 0.f), make_float4(p.a1.x, p.a1.y, p.a1.z, 0.f),
					make_float4(q.back.x, q.back.y, q.back.z, 0.f), make_float4(q.base.x, q.base.y, q.base.z, 0.f),
					make_float4(q.a1.x, q.a1.y, q.a1.z, 0.f), &t);
			o.F = v3<R>{fe.x, fe.y, fe.z};
			o.T = v3<R>{t.x, t.y, t.z};
			add_e<R, SPLIT>(o, T_NEXC, fe.w);
		}
		else {
			pair_ev<R, SPLIT>(p, q, sp, o);
		}
		if(o.F.x == R(0) && o.F.y == R(0) && o.F.z == R(0) && o.E == R(0)) continue;
		acc.add(o);
		partner(j, -o.F, cross_accurate(sp, o.F) - o.T, o.E);
	}
	if(SPLIT && live) {
#pragma unroll
		for(int k = 0; k < N_TERMS; k++)
			if(acc.split[k] != R(0)) atomicAdd(a.esplit + 8 * sy + k, (double) acc.split[k]);
	}
	const R fx = group_sum_comp<R, K>(acc.F.s.x, acc.F.c.x), fy = group_sum_comp<R, K>(acc.F.s.y, acc.F.c.y),
			fz = group_sum_comp<R, K>(acc.F.s.z, acc.F.c.z);
	const R tx = group_sum_comp<R, K>(acc.T.s.x, acc.T.c.x), ty = group_sum_comp<R, K>(acc.T.s.y, acc.T.c.y),
			tz = group_sum_comp<R, K>(acc.T.s.z, acc.T.c.z);
	const R e = ENERGY ? group_sum_comp<R, K>(acc.E, acc.Ec) : R(0);
	if(sub == 0 && live) partner(i, v3<R>{fx, fy, fz}, v3<R>{tx, ty, tz}, e);
}

// The bonded and the base/stack pair work are independent (both read the mirrors, each writes
// its own result buffers), so they share one launch: blocks 0 .. 2 pair_blocks - 1 are pair
// blocks (the costliest, dispatched first), then the bonded blocks, which fill the tail, and
// with use_edge the edge blocks.
template <typename R, class Loader, bool SPLIT, bool ENERGY, int NPW = OXGB_PAIR_NPW, bool EDGE = false, int K = 4>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? OXGB_PAIR_MINB : 1) k_bonded_pairs(ForceArgs a, Loader ld, int pair_blocks) {
	pdl_trigger();  // the non-bonded kernel may start (it waits before reading these results)
	const int b = blockIdx.x;
	const int bonded_blocks = (a.N + (int) blockDim.x - 1) / (int) blockDim.x;
	if(b < 2 * pair_blocks) pair_block<R, Loader, SPLIT, ENERGY, NPW>(a, ld, b, pair_blocks);
	else if(!EDGE || b < 2 * pair_blocks + bonded_blocks) bonded_block<R, Loader, SPLIT, ENERGY>(a, ld, b - 2 * pair_blocks);
	else if constexpr(EDGE) edge_block<R, Loader, SPLIT, ENERGY, K>(a, ld, b - 2 * pair_blocks - bonded_blocks);
}

// K lanes per nucleotide: lane l of a group takes entries l, l + K, ... of every term list, so a
// warp holds 32 / K nucleotides and all its lanes run the same term loop
// minimum resident blocks per SM asked of the register allocator for the non-bonded kernel
#ifndef OXGB_NB_MINB
#define OXGB_NB_MINB 8
#endif

template <typename R, class Loader, bool SPLIT, bool ENERGY, int K, int MINB = OXGB_NB_MINB, bool EDGE = false>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? MINB : 1) k_nonbonded_split(ForceArgs a, Loader ld) {
	using V4 = typename Vec4Of<R>::T;
	const long long N = a.N;
	const int sub = threadIdx.x % K;
	// one nucleotide per group of K lanes: the grid covers every nucleotide (nonbonded_blocks);
	// the lanes of a group past the last nucleotide still take part in the shuffles
	const int i_raw = (blockIdx.x * blockDim.x + threadIdx.x) / K;
	const int first = blockIdx.x * (blockDim.x / K);
	DNA2Table<R> *Ps = reinterpret_cast<DNA2Table<R> *>(g_tables_smem);
	const int s0 = load_table_span<R>(a, first, min(first + (int) (blockDim.x / K), a.N) - 1, Ps);
	{
		const bool live = i_raw < a.N;
		const int i = live ? i_raw : a.N - 1;
		const int sy = a.sys ? a.sys[i] : 0;
		const DNA2Table<R> &P = Ps[sy - s0];
		Nuc<R> p;
		V4 ph, pl;
		load_full<Loader, R>(ld, i, P, p, ph, pl);
		SplitAcc<R, SPLIT, ENERGY> acc{};

		// Debye-Hueckel over the full Verlet row (use_edge: the edge blocks did it).  The lever
		// arm of every pair's torque on i is i's backbone offset, so the forces are summed
		// (compensated) and the torque is taken once from the sum.
		// (the engine's Debye-Hueckel rows where built: the full rows' entries whose backbone sites
		// are within the cutoff plus twice the skin)
		const int *dhr = a.dh_nb ? a.dh_nb : a.nb;
		const int ndh = (live && !EDGE) ? min(a.dh_nb ? a.dh_n[i] : a.nnb[i], a.max_nb) : 0;
		{
			KahanV<R> fdh{};
			// the next partner's data is loaded before this partner's arithmetic, and the index
			// after it one iteration earlier still: two gathers in flight per lane (measured with
			// the torque taken from the sum: -3.6 % per MD step at 40k, -4.7 % at 250k)
			Nuc<R> qn;
			V4 qhn, qln;
			int k = sub;
			if(k < ndh) load_dh<Loader, R>(ld, dhr[(long long) k * N + i], P, qn, qhn, qln);
			int jnn = (k + K < ndh) ? dhr[(long long) (k + K) * N + i] : 0;
			for(; k < ndh; k += K) {
				const v3<R> qback = qn.back;
				const bool qend = qn.is_end;
				const V4 qh = qhn, ql = qln;
				if(k + K < ndh) load_dh<Loader, R>(ld, jnn, P, qn, qhn, qln);
				if(k + 2 * K < ndh) jnn = dhr[(long long) (k + 2 * K) * N + i];
				v3<R> f;
				R e;
				if(dh_sites(P, ld.sep_soft(ph, pl, qh, ql, P).plain() + qback - p.back, p.is_end, qend, f, e)) {
					fdh.add(f);
					if(ENERGY) KahanV<R>::kadd(acc.E, acc.Ec, e);
					if(SPLIT) acc.split[T_DH] += e;
				}
			}
			const v3<R> fs{fdh.s.x - fdh.c.x, fdh.s.y - fdh.c.y, fdh.s.z - fdh.c.z};
			acc.F.add(fs);
			acc.T.add(cross(p.back, fs));
		}
		// excluded volume over centre-close pairs (use_edge: the edge blocks did it)
		const int nev = (live && !EDGE) ? min(a.ev_n[i], a.ev_cap) : 0;
		if constexpr(decltype(ld.refine(0, 0))::on) {
			// FP32: each window of 64 of the lane's entries is screened (a site pair inside its
			// cutoff: a few in a thousand entries); the pairs found are evaluated refined after the
			// window, outside the screening loop, and the others contribute nothing
			for(int w0 = 0; w0 < nev; w0 += 64 * K) {
				const int wend = min(nev, w0 + 64 * K);
				unsigned long long stiff = 0ull;
				int m = 0;
				for(int k = w0 + sub; k < wend; k += K, m++) {
					const int j = a.ev_nb[(long long) k * N + i];
					Nuc<R> q;
					V4 qh, ql;
					load_full<Loader, R>(ld, j, P, q, qh, ql);
					if(ev_contact(p, q, ld.sep_soft(ph, pl, qh, ql, P).plain())) stiff |= 1ull << m;
				}
				while(stiff) {
					const int mm = __ffsll((long long) stiff) - 1;
					stiff &= stiff - 1ull;
					const int j = a.ev_nb[(long long) (w0 + sub + mm * K) * N + i];
					Nuc<R> q;
					V4 qh, ql;
					load_full<Loader, R>(ld, j, P, q, qh, ql);
					PairOut<R> o{};
					const Sep<R> sp = ld.sep(ph, pl, qh, ql, P);
					float3 t;
					const float4 fe = ev_pair_refined_call(
							ld.a1lo, ld.backlo, i, j, make_float4(sp.hi.x, sp.hi.y, sp.hi.z, 0.f), make_float4(sp.lo.x, sp.lo.y, sp.lo.z, 0.f),
							make_float4(p.back.x, p.back.y, p.back.z, 0.f), make_float4(p.base.x, p.base.y, p.base.z, 0.f),
							make_float4(p.a1.x, p.a1.y, p.a1.z, 0.f), make_float4(q.back.x, q.back.y, q.back.z, 0.f),
							make_float4(q.base.x, q.base.y, q.base.z, 0.f), make_float4(q.a1.x, q.a1.y, q.a1.z, 0.f), &t);
					o.F = v3<R>{fe.x, fe.y, fe.z};
					o.T = v3<R>{t.x, t.y, t.z};
					add_e<R, SPLIT>(o, T_NEXC, fe.w);
					acc.add_short(o);
				}
			}
		}
		else {
			for(int k = sub; k < nev; k += K) {
				const int j = a.ev_nb[(long long) k * N + i];
				Nuc<R> q;
				V4 qh, ql;
				load_full<Loader, R>(ld, j, P, q, qh, ql);
				PairOut<R> o{};
				pair_ev<R, SPLIT>(p, q, ld.sep(ph, pl, qh, ql, P), o);
				acc.add_short(o);
			}
		}
		// hydrogen bonding + cross stacking and coaxial stacking: evaluated per list slot by
		// the pair blocks of k_bonded_pairs, gathered here (the terms above read only the
		// mirrors and lists, complete before k_bonded_pairs started)
		pdl_wait();
		pdl_trigger();
		// the base slots then the stack slots as one sequence, the next slot loaded before the
		// current one is added
		const int nb_ = live ? min(a.base_n[i], a.base_cap) : 0;
		const int ns = live ? min(a.stk_n[i], a.stk_cap) : 0;
		{
			const int nt = nb_ + ns;
			const V4 *rb = reinterpret_cast<const V4 *>(a.base_res), *rs = reinterpret_cast<const V4 *>(a.stk_res);
			auto slot = [&](int k) { return k < nb_ ? rb + 2 * ((long long) k * N + i) : rs + 2 * ((long long) (k - nb_) * N + i); };
			V4 f, t;
			int k = sub;
			if(k < nt) {
				const V4 *q = slot(k);
				f = q[0];
				t = q[1];
			}
			for(; k < nt; k += K) {
				const V4 cf = f, ct = t;
				if(k + K < nt) {
					const V4 *q = slot(k + K);
					f = q[0];
					t = q[1];
				}
				acc.F.add(v3<R>{cf.x, cf.y, cf.z});
				acc.T.add(v3<R>{ct.x, ct.y, ct.z});
				if(ENERGY) {
					KahanV<R>::kadd(acc.E, acc.Ec, cf.w);
					KahanV<R>::kadd(acc.Eh, acc.Ehc, ct.w);
				}
			}
		}
		if(SPLIT && live) {
#pragma unroll
			for(int k = 0; k < N_TERMS; k++)
				if(acc.split[k] != R(0)) atomicAdd(a.esplit + 8 * sy + k, 0.5 * (double) acc.split[k]);
		}

		// bonded pairs of this nucleotide, evaluated by the bonded blocks of k_bonded_pairs (first
		// lane of the group); with use_edge also its Debye-Hueckel and excluded-volume sums, which
		// are cleared for the next evaluation
		if(sub == 0 && live) {
			if constexpr(EDGE) {
				V4 *ea = reinterpret_cast<V4 *>(a.edge_acc) + 2 * (long long) i;
				const V4 f = ea[0], t = ea[1];
				acc.F.add(v3<R>{f.x, f.y, f.z});
				acc.T.add(v3<R>{t.x, t.y, t.z});
				if(ENERGY) KahanV<R>::kadd(acc.E, acc.Ec, f.w);
				V4 z;
				z.x = z.y = z.z = z.w = R(0);
				ea[0] = z;
				ea[1] = z;
			}
			const int2 bi = a.bonds[i];
			const V4 *bf = reinterpret_cast<const V4 *>(a.bond_f);
			if(bi.x >= 0) {
				const V4 f = bf[i], t = reinterpret_cast<const V4 *>(a.bond_tp)[i];
				acc.F.add(v3<R>{-f.x, -f.y, -f.z});
				acc.T.add(v3<R>{t.x, t.y, t.z});
				if(ENERGY) KahanV<R>::kadd(acc.E, acc.Ec, f.w);
			}
			if(bi.y >= 0) {
				const V4 f = bf[bi.y], t = reinterpret_cast<const V4 *>(a.bond_tq)[bi.y];
				acc.F.add(v3<R>{f.x, f.y, f.z});
				acc.T.add(v3<R>{t.x, t.y, t.z});
				if(ENERGY) KahanV<R>::kadd(acc.E, acc.Ec, f.w);
			}
		}

		acc.fold_short();
		const R fx = group_sum_comp<R, K>(acc.F.s.x, acc.F.c.x), fy = group_sum_comp<R, K>(acc.F.s.y, acc.F.c.y),
				fz = group_sum_comp<R, K>(acc.F.s.z, acc.F.c.z);
		const v3<R> tl{group_sum_comp<R, K>(acc.T.s.x, acc.T.c.x), group_sum_comp<R, K>(acc.T.s.y, acc.T.c.y),
				group_sum_comp<R, K>(acc.T.s.z, acc.T.c.z)};
		const R e = ENERGY ? group_sum_comp<R, K>(acc.E, acc.Ec) : R(0);
		const R eh = ENERGY ? group_sum_comp<R, K>(acc.Eh, acc.Ehc) : R(0);
		if(sub == 0 && live) {
			V4 fo, to;
			fo.x = fx;
			fo.y = fy;
			fo.z = fz;
			fo.w = e;
			to.x = dot(p.a1, tl);
			to.y = dot(p.a2, tl);
			to.z = dot(p.a3, tl);
			to.w = eh;
			reinterpret_cast<V4 *>(a.forces)[i] = fo;
			reinterpret_cast<V4 *>(a.torques)[i] = to;
		}
	}
}

// lanes per nucleotide in the non-bonded kernel
#ifndef OXGB_NB_LANES
#define OXGB_NB_LANES 4
#endif

int nonbonded_blocks(int N, int lanes) {
	const long long threads = (long long) (N > 0 ? N : 1) * lanes;
	return (int) ((threads + 127) / 128);
}

// The shapes of the MD step's force kernels (engine, mixed and float precision) the autotuner
// chooses among: nucleotides per pair-block warp queue, lanes per nucleotide in the non-bonded
// kernel and the resident blocks per SM its register cap asks for.  Shape 0 is the default, the
// best of hand sweeps on the 40k and 250k workloads.
struct ForceShapeDef {
	int npw, lanes, minb;
};
constexpr ForceShapeDef FORCE_SHAPES[] = {{32, 4, 8}, {16, 4, 8}, {32, 8, 6}, {16, 8, 6}, {32, 2, 8}, {16, 2, 8}};
constexpr int N_FORCE_SHAPES = sizeof(FORCE_SHAPES) / sizeof(FORCE_SHAPES[0]);

int force_shape_count() { return N_FORCE_SHAPES; }

void force_shape_of(int k, int *npw, int *lanes, int *minb) {
	const ForceShapeDef &d = FORCE_SHAPES[k >= 0 && k < N_FORCE_SHAPES ? k : 0];
	if(npw) *npw = d.npw;
	if(lanes) *lanes = d.lanes;
	if(minb) *minb = d.minb;
}

// External forces (CUDA_MD.cuh:97-555): one thread per nucleotide that has some, its records
// in order (deterministic), added to the force the pair kernels left; FP64 positions.
template <typename V4>
__global__ void k_external(ForceArgs a) {
	pdl_wait();
	pdl_trigger();
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= a.ext_n) return;
	// records name caller's indices
	const int i = a.slot ? a.slot[a.ext_nuc[k]] : a.ext_nuc[k];
	const long long step = a.th.step_base ? *a.th.step_base + a.th.step_offset : 0;
	const double st = (double) step;
	const oxgb_ext_force *rec = reinterpret_cast<const oxgb_ext_force *>(a.ext_rec);
	const double4_32a r = a.posd[i];
	double fx = 0, fy = 0, fz = 0;
	for(int m = a.ext_off[k]; m < a.ext_off[k + 1]; m++) {
		const oxgb_ext_force &e = rec[m];
		switch(e.type) {
		case OXGB_FORCE_CONSTANT: {
			const double in = e.F0 + st * e.rate;
			double dx = e.dir[0], dy = e.dir[1], dz = e.dir[2];
			if(e.flags & 1) {
				dx -= r.x, dy -= r.y, dz -= r.z;
				const double n = sqrt(dx * dx + dy * dy + dz * dz);
				dx /= n, dy /= n, dz /= n;
			}
			fx += dx * in, fy += dy * in, fz += dz * in;
			break;
		}
		case OXGB_FORCE_MUTUAL_TRAP: {
			const double4_32a q = a.posd[a.slot ? a.slot[e.ref_particle] : e.ref_particle];
			double dx = q.x - r.x, dy = q.y - r.y, dz = q.z - r.z;
			if(e.flags & 1) {
				const double L = a.sys_box ? (double) a.sys_box[a.sys ? a.sys[i] : 0] : (double) a.box;
				dx -= rint(dx / L) * L, dy -= rint(dy / L) * L, dz -= rint(dz / L) * L;
			}
			const double d = sqrt(dx * dx + dy * dy + dz * dz);
			const double c = (d - (e.r0 + e.rate * st)) * (e.stiff + st * e.stiff_rate) / d;
			fx += dx * c, fy += dy * c, fz += dz * c;
			break;
		}
		case OXGB_FORCE_MOVING_TRAP:
		case OXGB_FORCE_LOWDIM_TRAP: {
			const double tx = e.pos0[0] + e.rate * st * e.dir[0], ty = e.pos0[1] + e.rate * st * e.dir[1],
						 tz = e.pos0[2] + e.rate * st * e.dir[2];
			const bool all = e.type == OXGB_FORCE_MOVING_TRAP;
			if(all || (e.flags & 2)) fx += -e.stiff * (r.x - tx);
			if(all || (e.flags & 4)) fy += -e.stiff * (r.y - ty);
			if(all || (e.flags & 8)) fz += -e.stiff * (r.z - tz);
			break;
		}
		case OXGB_FORCE_REPULSION_PLANE: {
			double p = e.position + e.rate * st;
			if(e.r0 > e.position && p > e.r0) p = e.r0;
			if(e.r0 < e.position && p < e.r0) p = e.r0;
			const double d = e.dir[0] * r.x + e.dir[1] * r.y + e.dir[2] * r.z + p;
			if(d < 0.0) fx += -d * e.stiff * e.dir[0], fy += -d * e.stiff * e.dir[1], fz += -d * e.stiff * e.dir[2];
			break;
		}
		case OXGB_FORCE_ATTRACTION_PLANE: {
			const double d = e.dir[0] * r.x + e.dir[1] * r.y + e.dir[2] * r.z + e.position;
			if(d < 0.0) fx += -d * e.stiff * e.dir[0], fy += -d * e.stiff * e.dir[1], fz += -d * e.stiff * e.dir[2];
			else fx += -e.stiff * e.dir[0], fy += -e.stiff * e.dir[1], fz += -e.stiff * e.dir[2];
			break;
		}
		case OXGB_FORCE_SPHERE:
		case OXGB_FORCE_SPHERE_SMOOTH: {
			// RepulsiveSphere / RepulsiveSphereSmooth::force (src/Forces/RepulsiveSphere*.cpp):
			// minimum image of r - centre
			const double L = a.sys_box ? (double) a.sys_box[a.sys ? a.sys[i] : 0] : (double) a.box;
			double dx = r.x - e.pos0[0], dy = r.y - e.pos0[1], dz = r.z - e.pos0[2];
			dx -= rint(dx / L) * L, dy -= rint(dy / L) * L, dz -= rint(dz / L) * L;
			const double m = sqrt(dx * dx + dy * dy + dz * dz);
			double c = 0.0;
			if(e.type == OXGB_FORCE_SPHERE) {
				const double R = e.r0 + e.rate * st;
				if(m > R && m < e.cutoff) c = -e.stiff * (1.0 - R / m);
			}
			else if(!(m < e.r0 || m > e.cutoff)) {
				if(m >= e.p1) c = -(e.stiff * 0.5 * exp((m - e.p1) / e.sigma)) / m;
				else c = -(e.stiff * m - e.stiff * 0.5 * exp(-(m - e.p1) / e.sigma)) / m;
			}
			fx += dx * c, fy += dy * c, fz += dz * c;
			break;
		}
		case OXGB_FORCE_LJ_WALL: {
			// LJWall::force (src/Forces/LJWall.cpp)
			const double x = e.dir[0] * r.x + e.dir[1] * r.y + e.dir[2] * r.z + e.position;
			const double y = x / e.sigma;
			if(y <= e.cutoff) {
				const double lj = pow(y, (double) -e.n);
				const double c = 4.0 * e.n * e.stiff * (2.0 * lj * lj - lj) / x;
				fx += e.dir[0] * c, fy += e.dir[1] * c, fz += e.dir[2] * c;
			}
			break;
		}
		case OXGB_FORCE_CENTRAL: {
			// GenericCentralForce::force, force_type = gravity (src/Forces/GenericCentralForce.cpp)
			const double dx = e.pos0[0] - r.x, dy = e.pos0[1] - r.y, dz = e.pos0[2] - r.z;
			const double d2 = dx * dx + dy * dy + dz * dz;
			if(!(d2 < e.p1 * e.p1) && !(e.p2 > 0.0 && d2 > e.p2 * e.p2)) {
				const double c = e.F0 / sqrt(d2);
				fx += dx * c, fy += dy * c, fz += dz * c;
			}
			break;
		}
		case OXGB_FORCE_REPULSION_PLANE_MOVING: {
			// RepulsionPlaneMoving::force (src/Forces/RepulsionPlaneMoving.cpp), one reference particle
			const double4_32a q = a.posd[a.slot ? a.slot[e.ref_particle] : e.ref_particle];
			const double x = (r.x - q.x) * e.dir[0] + (r.y - q.y) * e.dir[1] + (r.z - q.z) * e.dir[2];
			const double c = -e.stiff * fmin(x, 0.0);
			fx += e.dir[0] * c, fy += e.dir[1] * c, fz += e.dir[2] * c;
			break;
		}
		case OXGB_FORCE_LJ_CONE: {
			// LJCone::force (src/Forces/LJCone.cpp): apex pos0, axis dir, half-angle p1
			const double vx = r.x - e.pos0[0], vy = r.y - e.pos0[1], vz = r.z - e.pos0[2];
			const double along = vx * e.dir[0] + vy * e.dir[1] + vz * e.dir[2];
			const double wx = e.dir[0] * along - vx, wy = e.dir[1] * along - vy, wz = e.dir[2] * along - vz;
			const double from_axis = sqrt(wx * wx + wy * wy + wz * wz);
			const double x = along * sin(e.p1) - from_axis * cos(e.p1);
			const double y = x / e.sigma;
			if(y <= e.cutoff) {
				const double C = from_axis * tan(e.p1);
				double nx = (along + C) * e.dir[0] - vx, ny = (along + C) * e.dir[1] - vy, nz = (along + C) * e.dir[2] - vz;
				const double nn = sqrt(nx * nx + ny * ny + nz * nz);
				nx /= nn, ny /= nn, nz /= nn;
				const double lj = pow(y, (double) -e.n);
				const double c = 4.0 * e.n * e.stiff * (2.0 * lj * lj - lj) / x;
				fx += nx * c, fy += ny * c, fz += nz * c;
			}
			break;
		}
		case OXGB_FORCE_TWIST: {
			// ConstantRateTorque::force (src/Forces/ConstantRateTorque.cpp): the trap pos0 rotated
			// about the axis dir through the centre v1 by F0 + rate step radians (Rodrigues'
			// matrix), the pull masked component-wise by v2
			const double t = e.F0 + e.rate * st;
			const double sn = sin(t), cs = cos(t), oc = 1.0 - cs;
			const double ax = e.dir[0], ay = e.dir[1], az = e.dir[2];
			const double ux = e.pos0[0] - e.v1[0], uy = e.pos0[1] - e.v1[1], uz = e.pos0[2] - e.v1[2];
			const double tx = (ax * ax * oc + cs) * ux + (ax * ay * oc - az * sn) * uy + (ax * az * oc + ay * sn) * uz + e.v1[0];
			const double ty = (ax * ay * oc + az * sn) * ux + (ay * ay * oc + cs) * uy + (ay * az * oc - ax * sn) * uz + e.v1[1];
			const double tz = (ax * az * oc - ay * sn) * ux + (ay * az * oc + ax * sn) * uy + (az * az * oc + cs) * uz + e.v1[2];
			fx += -e.stiff * (r.x - tx) * e.v2[0];
			fy += -e.stiff * (r.y - ty) * e.v2[1];
			fz += -e.stiff * (r.z - tz) * e.v2[2];
			break;
		}
		case OXGB_FORCE_ELLIPSOID: {
			// RepulsiveEllipsoid::force (src/Forces/RepulsiveEllipsoid.cpp): pushed towards the
			// centre unless inside r_2 and outside r_1
			const double L = a.sys_box ? (double) a.sys_box[a.sys ? a.sys[i] : 0] : (double) a.box;
			double dx = r.x - e.pos0[0], dy = r.y - e.pos0[1], dz = r.z - e.pos0[2];
			dx -= rint(dx / L) * L, dy -= rint(dy / L) * L, dz -= rint(dz / L) * L;
			const double in = dx * dx / (e.v2[0] * e.v2[0]) + dy * dy / (e.v2[1] * e.v2[1]) + dz * dz / (e.v2[2] * e.v2[2]);
			const double out = dx * dx / (e.v1[0] * e.v1[0]) + dy * dy / (e.v1[1] * e.v1[1]) + dz * dz / (e.v1[2] * e.v1[2]);
			if(!(in < 1.0 && out > 1.0)) {
				const double m = sqrt(dx * dx + dy * dy + dz * dz);
				fx += -e.stiff * dx / m, fy += -e.stiff * dy / m, fz += -e.stiff * dz / m;
			}
			break;
		}
		case OXGB_FORCE_COM: {
			// COMForce::force (src/Forces/COMForce.cpp): centres of mass of group n (com_list) and
			// of group ref_particle (ref_list) from the unwrapped FP64 positions
			double c[2][3] = {{0, 0, 0}, {0, 0, 0}};
			int cnt[2];
			const int gs[2] = {e.n, e.ref_particle};
			for(int w = 0; w < 2; w++) {
				const int g0 = a.grp_off[gs[w]], g1 = a.grp_off[gs[w] + 1];
				cnt[w] = g1 - g0;
				for(int u = g0; u < g1; u++) {
					const double4_32a q = a.posd[a.slot ? a.slot[a.grp_mem[u]] : a.grp_mem[u]];
					c[w][0] += q.x, c[w][1] += q.y, c[w][2] += q.z;
				}
				for(int d = 0; d < 3; d++) c[w][d] /= (double) cnt[w];
			}
			const double dx = c[1][0] - c[0][0], dy = c[1][1] - c[0][1], dz = c[1][2] - c[0][2];
			const double m = sqrt(dx * dx + dy * dy + dz * dz);
			const double f = (m - (e.r0 + e.rate * st)) * e.stiff / (double) cnt[0] / m;
			fx += dx * f, fy += dy * f, fz += dz * f;
			break;
		}
		case OXGB_FORCE_YUKAWA_SPHERE: {
			// YukawaSphere::force (src/Forces/YukawaSphere.cpp): screened repulsion from the inside
			// of a sphere of radius r0, with a WCA core near its surface
			const double L = a.sys_box ? (double) a.sys_box[a.sys ? a.sys[i] : 0] : (double) a.box;
			double dx = r.x - e.pos0[0], dy = r.y - e.pos0[1], dz = r.z - e.pos0[2];
			dx -= rint(dx / L) * L, dy -= rint(dy / L) * L, dz -= rint(dz / L) * L;
			const double m = sqrt(dx * dx + dy * dy + dz * dz);
			const double sd = e.r0 - m;
			if(sd < e.cutoff) {
				double c = e.F0 * exp(-sd / e.p2) * (1.0 / (sd * e.p2) + 1.0 / (sd * sd));
				if(sd < e.p1) {
					const double w = pow(e.sigma / sd, 6.0);
					c += 4.0 * e.stiff * e.n * (2.0 * w * w - w) / sd;
				}
				fx += -dx / m * c, fy += -dy / m * c, fz += -dz / m * c;
			}
			break;
		}
		case OXGB_FORCE_SPHERE_MOVING: {
			// RepulsiveSphereMoving::force (src/Forces/RepulsiveSphereMoving.cpp): WCA (the
			// 2x-x form with x = 2, sigma = 1, eps = stiff) of the gap to a growing sphere whose
			// centre moves from v1 to v2 over p1 steps
			double t = 0.0;
			if(e.p1 > 0.0) t = fmin(fmax(st / floor(e.p1), 0.0), 1.0);
			const double cx = e.v1[0] + (e.v2[0] - e.v1[0]) * t, cy = e.v1[1] + (e.v2[1] - e.v1[1]) * t,
						 cz = e.v1[2] + (e.v2[2] - e.v1[2]) * t;
			const double L = a.sys_box ? (double) a.sys_box[a.sys ? a.sys[i] : 0] : (double) a.box;
			double dx = r.x - cx, dy = r.y - cy, dz = r.z - cz;
			dx -= rint(dx / L) * L, dy -= rint(dy / L) * L, dz -= rint(dz / L) * L;
			const double m = sqrt(dx * dx + dy * dy + dz * dz);
			const double g = m - (e.r0 + e.rate * st);
			if(!(g >= e.cutoff) && m > 0.0 && g < 1.4142135623730951) {
				const double gs = g > 1e-9 ? g : 1e-9;
				const double A = 1.0 / (gs * gs);
				const double c = 8.0 * e.stiff * (2.0 * A - 1.0) * A / gs / m;
				fx += dx * c, fy += dy * c, fz += dz * c;
			}
			break;
		}
		default:
			break;
		}
	}
	V4 *F = reinterpret_cast<V4 *>(a.forces);
	V4 f = F[i];
	f.x += fx;
	f.y += fy;
	f.z += fz;
	F[i] = f;
}

template <typename R, class Loader, bool SPLIT, bool ENERGY, int NPW = OXGB_PAIR_NPW, int K = OXGB_NB_LANES,
		int NBMINB = OXGB_NB_MINB, bool EDGE = false>
static void launch_split_t(const ForceArgs &a, Loader ld, cudaStream_t s, cudaEvent_t wait) {
	const int tpb = 128;
	const int blocks = a.N > 0 ? (a.N + tpb - 1) / tpb : 1;
	const size_t smem = sizeof(DNA2Table<R>) * (size_t) (a.tab_span > 0 ? a.tab_span : 1);
	// pair blocks of 4 warps x NPW nucleotides per term, then one bonded block per 128
	// nucleotides, then (use_edge) one edge block per 128 / K nucleotides
	const int pair_blocks = (a.N + 4 * NPW - 1) / (4 * NPW);
	const int edge_blocks = EDGE ? nonbonded_blocks(a.N, K) : 0;
	k_bonded_pairs<R, Loader, SPLIT, ENERGY, NPW, EDGE, K><<<2 * pair_blocks + blocks + edge_blocks, tpb, smem, s>>>(a, ld, pair_blocks);
	// the non-bonded kernel starts its Debye-Hueckel and excluded-volume work while the tail of
	// the bonded and pair blocks runs; the external forces follow it the same way
	if(wait) cudaStreamWaitEvent(s, wait, 0);
	if(wait) k_nonbonded_split<R, Loader, SPLIT, ENERGY, K, NBMINB, EDGE><<<nonbonded_blocks(a.N, K), tpb, smem, s>>>(a, ld);
	else launch_after(k_nonbonded_split<R, Loader, SPLIT, ENERGY, K, NBMINB, EDGE>, dim3(nonbonded_blocks(a.N, K)), dim3(tpb), smem,
			s, a, ld);
	if(a.ext_n > 0) launch_after(k_external<typename Vec4Of<R>::T>, dim3((a.ext_n + tpb - 1) / tpb), dim3(tpb), 0, s, a);
}

template <typename R, class Loader, bool SPLIT, bool ENERGY, int NPW = OXGB_PAIR_NPW, int K = OXGB_NB_LANES,
		int NBMINB = OXGB_NB_MINB, bool EDGE = false>
static cudaError_t allow_smem_t(int bytes) {
	cudaError_t e = cudaFuncSetAttribute(k_bonded_pairs<R, Loader, SPLIT, ENERGY, NPW, EDGE, K>,
			cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
	if(e == cudaSuccess)
		e = cudaFuncSetAttribute(k_nonbonded_split<R, Loader, SPLIT, ENERGY, K, NBMINB, EDGE>,
				cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
	return e;
}

// the MD step's kernels (mixed / float engine) in shape k of FORCE_SHAPES
template <int k>
static void launch_md_shape(const ForceArgs &a, const SplitMixed &ld, cudaStream_t s, cudaEvent_t wait) {
	constexpr ForceShapeDef d = FORCE_SHAPES[k];
	launch_split_t<float, SplitMixed, false, false, d.npw, d.lanes, d.minb>(a, ld, s, wait);
}

template <int k>
static cudaError_t allow_smem_shape(int bytes) {
	constexpr ForceShapeDef d = FORCE_SHAPES[k];
	return allow_smem_t<float, SplitMixed, false, false, d.npw, d.lanes, d.minb>(bytes);
}

template <typename R, class Loader>
static cudaError_t allow_smem(int bytes) {
	cudaError_t e = allow_smem_t<R, Loader, true, true>(bytes);
	if(e == cudaSuccess) e = allow_smem_t<R, Loader, false, true>(bytes);
	if(e == cudaSuccess) e = allow_smem_t<R, Loader, false, false>(bytes);
	if(e == cudaSuccess) e = allow_smem_t<R, Loader, true, true, OXGB_PAIR_NPW, OXGB_NB_LANES, OXGB_NB_MINB, true>(bytes);
	if(e == cudaSuccess) e = allow_smem_t<R, Loader, false, true, OXGB_PAIR_NPW, OXGB_NB_LANES, OXGB_NB_MINB, true>(bytes);
	if(e == cudaSuccess) e = allow_smem_t<R, Loader, false, false, OXGB_PAIR_NPW, OXGB_NB_LANES, OXGB_NB_MINB, true>(bytes);
	if constexpr(sizeof(R) == 4) {
		if(e == cudaSuccess) e = allow_smem_shape<1>(bytes);
		if(e == cudaSuccess) e = allow_smem_shape<2>(bytes);
		if(e == cudaSuccess) e = allow_smem_shape<3>(bytes);
		if(e == cudaSuccess) e = allow_smem_shape<4>(bytes);
		if(e == cudaSuccess) e = allow_smem_shape<5>(bytes);
	}
	return e;
}

int set_forces_smem(bool dbl, size_t bytes) {
	if(bytes <= 48 * 1024) return 0;
	if(bytes > 160 * 1024) return 1;
	return (dbl ? allow_smem<double, SplitDouble>((int) bytes) : allow_smem<float, SplitMixed>((int) bytes)) != cudaSuccess;
}

// use_edge: the default shape with the edge blocks
template <typename R, class Loader>
static void launch_edge(const ForceArgs &a, Loader ld, bool split, bool energy, cudaStream_t s, cudaEvent_t wait) {
	constexpr int NPW = OXGB_PAIR_NPW, K = OXGB_NB_LANES, MB = OXGB_NB_MINB;
	if(split) launch_split_t<R, Loader, true, true, NPW, K, MB, true>(a, ld, s, wait);
	else if(energy) launch_split_t<R, Loader, false, true, NPW, K, MB, true>(a, ld, s, wait);
	else launch_split_t<R, Loader, false, false, NPW, K, MB, true>(a, ld, s, wait);
}

cudaError_t launch_forces_split(const ForceArgs &a, bool dbl, bool split, bool energy, cudaStream_t s, cudaEvent_t wait) {
	if(a.edge) {
		if(dbl) launch_edge<double, SplitDouble>(a, SplitDouble{a.posd, a.quatd, a.pos_hi, a.pos_lo, a.bonds}, split, energy, s, wait);
		else launch_edge<float, SplitMixed>(a, SplitMixed{a.pos_hi, a.pos_lo, a.fa1, a.fa3, a.fback, a.fa1lo, a.fbacklo}, split, energy,
				s, wait);
		return cudaGetLastError();
	}
	if(dbl) {
		SplitDouble ld{a.posd, a.quatd, a.pos_hi, a.pos_lo, a.bonds};
		if(split) launch_split_t<double, SplitDouble, true, true>(a, ld, s, wait);
		else if(energy) launch_split_t<double, SplitDouble, false, true>(a, ld, s, wait);
		else launch_split_t<double, SplitDouble, false, false>(a, ld, s, wait);
	}
	else {
		SplitMixed ld{a.pos_hi, a.pos_lo, a.fa1, a.fa3, a.fback, a.fa1lo, a.fbacklo};
		if(split) launch_split_t<float, SplitMixed, true, true>(a, ld, s, wait);
		else if(energy) launch_split_t<float, SplitMixed, false, true>(a, ld, s, wait);
		else {
			static_assert(N_FORCE_SHAPES == 6, "one case per shape");
			switch(a.shape) {
			case 1: launch_md_shape<1>(a, ld, s, wait); break;
			case 2: launch_md_shape<2>(a, ld, s, wait); break;
			case 3: launch_md_shape<3>(a, ld, s, wait); break;
			case 4: launch_md_shape<4>(a, ld, s, wait); break;
			case 5: launch_md_shape<5>(a, ld, s, wait); break;
			default: launch_md_shape<0>(a, ld, s, wait); break;
			}
		}
	}
	return cudaGetLastError();
}

}  // namespace oxgb
