// Velocity-Verlet integration in FP64 and the Brownian ("john") and Bussi thermostats.
//
// Replaces first_step_mixed / second_step_mixed (src/CUDA/Backends/CUDA_mixed.cuh:8-93) and the
// CUDA thermostats (src/CUDA/Thermostats/CUDABrownianThermostat.cu:15-51,
// CUDABussiThermostat.cu:55-122 with the host kinetic-energy update of
// src/Backends/Thermostats/BussiThermostat.cpp:44-160).  Differences by design: positions,
// velocities, angular momenta and quaternions stay FP64 throughout (the half kicks convert the
// FP32 forces to double before multiplying by dt), the quaternion is renormalised every step,
// random numbers come from a counter-based Philox-4x32-10 stream keyed by (seed, step,
// particle) so that runs are reproducible and graph-replayable, and the Bussi kinetic-energy
// update runs on the device (its gamma deviate uses the same algorithm as the reference).
// The second half kick of a step and its thermostat are deferred to the next first step (or
// to the flush at the end of a run), where they run one thread per nucleotide next to the
// first half kick; the Bussi sums run beside (k_bussi_prep) and after (k_bussi_sums, with the update) the forces, and its
// draws on a parallel branch of the step graph (k_bussi_noise).  No FP64 work is left in the force
// kernels, whose lanes are mostly idle at the epilogue.
#include "split.cuh"
#include "thermo.cuh"

namespace oxgb {

// ---------------------------------------------------------------- FP32 mirrors

// The FP32 mirrors of nucleotide i from its FP64 state: the position as hi + lo, the body
// axes a1, a3 and the grooved backbone offset (src/Particles/DNANucleotide.cpp:79), each
// rounded once (to within an ulp) from exact values; conversions and products on the FP32 and
// integer pipes (split.cuh).  Each part returns what the staleness test needs.
__device__ __forceinline__ float3 mirror_position(const StepArgs &a, int i, const double4_32a &r) {
	float4 hi = a.pos_hi[i], lo = a.pos_lo[i];
	split_rn(r.x, hi.x, lo.x);
	split_rn(r.y, hi.y, lo.y);
	split_rn(r.z, hi.z, lo.z);
	a.pos_hi[i] = hi;
	a.pos_lo[i] = lo;
	return make_float3(hi.x, hi.y, hi.z);
}

// returns a1 and the backbone offset; with a.fa1lo also the remainders of a1 and the backbone
// offset (exact value = mirror + remainder to ~2^-46), which the force kernels use for the stiff
// radial factors and excluded-volume contacts
__device__ __forceinline__ void mirror_frame(const StepArgs &a, int i, const double4_32a &q, float3 &a1o, float3 &backo) {
	float qh[4], ql[4], a1[3], a3[3], bk[3], a1l[3], bkl[3];
	split_rn(q.x, qh[0], ql[0]);
	split_rn(q.y, qh[1], ql[1]);
	split_rn(q.z, qh[2], ql[2]);
	split_rn(q.w, qh[3], ql[3]);
	if(a.fa1lo) {
		frame_mirror_rem(qh, ql, OXM_POS_MM_BACK1, OXM_POS_MM_BACK2, a1, a3, bk, a1l, bkl);
		a.fa1lo[i] = make_float4(a1l[0], a1l[1], a1l[2], 0.f);
		a.fbacklo[i] = make_float4(bkl[0], bkl[1], bkl[2], 0.f);
	}
	else frame_mirror(qh, ql, OXM_POS_MM_BACK1, OXM_POS_MM_BACK2, a1, a3, bk);
	a.fa1[i] = make_float4(a1[0], a1[1], a1[2], 0.f);
	a.fa3[i] = make_float4(a3[0], a3[1], a3[2], 0.f);
	// the strand-end flag rides in w
	if(a.fback) {
		const int2 bd = a.bonds[i];
		a.fback[i] = make_float4(bk[0], bk[1], bk[2], (bd.x < 0 || bd.y < 0) ? 1.f : 0.f);
	}
	a1o = make_float3(a1[0], a1[1], a1[2]);
	backo = make_float3(bk[0], bk[1], bk[2]);
}

// true if the centre or any interaction site moved more than the skin since the last list build
// (lp, la1, lbk: centre, a1 and backbone offset at the last build; r: the new centre in FP32,
// a1 and back: the new axis and backbone offset)
__device__ __forceinline__ bool list_stale(const StepArgs &a, const float4 &lp, const float4 &la1, const float4 &lbk, float3 r,
		float3 a1, float3 bk) {
	const float dx = r.x - lp.x, dy = r.y - lp.y, dz = r.z - lp.z;
	if(dx * dx + dy * dy + dz * dz > a.skin2) return true;
	if(!a.list_a1) return false;
	const float ex = a1.x - la1.x, ey = a1.y - la1.y, ez = a1.z - la1.z;
	float sx = dx + 0.4f * ex, sy = dy + 0.4f * ey, sz = dz + 0.4f * ez;  // base site
	if(sx * sx + sy * sy + sz * sz > a.skin2) return true;
	sx = dx + 0.34f * ex, sy = dy + 0.34f * ey, sz = dz + 0.34f * ez;  // stacking site
	if(sx * sx + sy * sy + sz * sz > a.skin2) return true;
	sx = dx + (bk.x - lbk.x), sy = dy + (bk.y - lbk.y), sz = dz + (bk.z - lbk.z);  // backbone site
	return sx * sx + sy * sy + sz * sz > a.skin2;
}

__global__ void k_make_mirrors(StepArgs a) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= a.N) return;
	float3 a1, bk;
	(void) mirror_position(a, i, a.pos[i]);
	mirror_frame(a, i, a.quat[i], a1, bk);
}

// ---------------------------------------------------------------- first half step

__device__ __forceinline__ long long step_of(const ThermoArgs &t) { return *t.step_base + t.step_offset; }

// completes step sp of nucleotide i (system sy): its second half kick (CUDA_mixed.cuh:71-93)
// and its thermostat (Brownian redraw or Bussi rescaling)
template <typename V4>
__device__ __forceinline__ void complete_step(const ThermoArgs &t, int i, int sy, long long sp, const V4 &F, const V4 &T,
		double4_32a &v, double4_32a &L) {
	// the half kicks are written as FMAs here and in the first step, so that a step completed at
	// the end of a run and one completed by the next first step are the same
	const double hdt = 0.5 * t.dt;
	v.x = fma(widen(F.x), hdt, v.x);
	v.y = fma(widen(F.y), hdt, v.y);
	v.z = fma(widen(F.z), hdt, v.z);
	L.x = fma(widen(T.x), hdt, L.x);
	L.y = fma(widen(T.y), hdt, L.y);
	L.z = fma(widen(T.z), hdt, L.z);
	if(t.thermostat == 1 && sp % t.newtonian_steps == 0) brownian_redraw(t, sy, (t.id ? t.id[i] : i) - t.sys_off[sy], sp, v, L);
	else if(t.thermostat == 2 && *t.bussi_stamp == sp) bussi_rescale(t, sy, v, L);
}

// the orientation after a step of dt with angular momentum L (body frame):
// q <- q * (sin(th/2) L^, cos(th/2)), th = dt |L|, then renormalised
__device__ __forceinline__ void rotate(double4_32a &q, const double4_32a &L, double dt) {
	const double L2 = L.x * L.x + L.y * L.y + L.z * L.z;
	if(!(L2 > 0.0)) return;
	const double hd = 0.5 * dt, x2 = hd * hd * L2;  // x = th / 2
	double k, ch;
	if(x2 < 1e-5) {
		// sin(x) / x and cos(x) as Taylor series in x^2: no square root, range reduction or
		// division, which are slow in FP64.  The first omitted terms, x^6/5040 and x^8/40320,
		// are below 2e-19 for x^2 < 1e-5 (a typical step has x^2 ~ 1e-6)
		k = hd * (1.0 - x2 * (1.0 / 6.0) * (1.0 - x2 * (1.0 / 20.0)));
		ch = 1.0 - x2 * 0.5 * (1.0 - x2 * (1.0 / 12.0) * (1.0 - x2 * (1.0 / 30.0)));
	}
	else if(x2 < 1e-2) {
		// the same series to x^10 (truncation below 1e-20 for |x| < 0.1)
		k = hd * (1.0 - x2 * (1.0 / 6.0) * (1.0 - x2 * (1.0 / 20.0) * (1.0 - x2 * (1.0 / 42.0) * (1.0 - x2 * (1.0 / 72.0) * (1.0 - x2 * (1.0 / 110.0))))));
		ch = 1.0 - x2 * 0.5 * (1.0 - x2 * (1.0 / 12.0) * (1.0 - x2 * (1.0 / 30.0) * (1.0 - x2 * (1.0 / 56.0) * (1.0 - x2 * (1.0 / 90.0)))));
	}
	else {
		const double norm = sqrt(L2);
		double sh;
		sincos(hd * norm, &sh, &ch);
		k = sh / norm;
	}
	const double rx = L.x * k, ry = L.y * k, rz = L.z * k, rw = ch;
	double4_32a n;
	n.w = q.w * rw - q.x * rx - q.y * ry - q.z * rz;
	n.x = q.w * rx + q.x * rw + q.y * rz - q.z * ry;
	n.y = q.w * ry - q.x * rz + q.y * rw + q.z * rx;
	n.z = q.w * rz + q.x * ry - q.y * rx + q.z * rw;
	const double nn = n.x * n.x + n.y * n.y + n.z * n.z + n.w * n.w;
	const double d = nn - 1.0;
	// |n|^2 = 1 + d with |d| at the rounding level: 1/sqrt(1 + d) = 1 - d/2 + 3d^2/8 - ...
	const double inv = fabs(d) < 1e-6 ? 1.0 - d * (0.5 - 0.375 * d) : 1.0 / sqrt(nn);
	q = make_double4_32a(n.x * inv, n.y * inv, n.z * inv, n.w * inv);
}

// The FP32 rotation of backend_precision = float (CUDA_MD.cuh:11-25): q <- q * (sin(th/2) L^,
// cos(th/2)), th = dt |L|, in FP32; renormalised in FP32 as well (the reference's float path
// lets the norm drift)
__device__ __forceinline__ void rotate_f32(float4 &q, float3 L, float dt) {
	const float L2 = L.x * L.x + L.y * L.y + L.z * L.z;
	if(!(L2 > 0.f)) return;
	const float norm = sqrtf(L2);
	float sh, ch;
	sincosf(0.5f * dt * norm, &sh, &ch);
	const float k = sh / norm;
	const float rx = L.x * k, ry = L.y * k, rz = L.z * k, rw = ch;
	float4 n;
	n.w = q.w * rw - q.x * rx - q.y * ry - q.z * rz;
	n.x = q.w * rx + q.x * rw + q.y * rz - q.z * ry;
	n.y = q.w * ry - q.x * rz + q.y * rw + q.z * rx;
	n.z = q.w * rz + q.x * ry - q.y * rx + q.z * rw;
	const float inv = rsqrtf(n.x * n.x + n.y * n.y + n.z * n.z + n.w * n.w);
	q = make_float4(n.x * inv, n.y * inv, n.z * inv, n.w * inv);
}

__device__ __forceinline__ double4_32a widen4(float x, float y, float z, float w) {
	return make_double4_32a(widen(x), widen(y), widen(z), widen(w));
}

// a state vector rounded to FP32 (backend_precision = float keeps the state FP32-representable)
__device__ __forceinline__ double4_32a round4(const double4_32a &v) {
	return widen4(narrow(v.x), narrow(v.y), narrow(v.z), narrow(v.w));
}

// First half of step s, two warps per 32 nucleotides: warp 0 of a block the translation (second
// half kick and thermostat of step s - 1, half kick, drift, position mirror), warp 1 the
// rotation (the same for the angular momentum, rotation, frame mirror).  The chains of FP64
// operations are half as long and twice as many warps hide them; a warp never diverges on the
// kind of motion.
// (capped at 64 registers, 16 blocks per SM: measured in alternating runs, the 250k MD step
// 138.7 -> 136.9 us and the 256-system batch 263.4 -> 261.3 us against the uncapped 80)
template <typename V4, bool F32 = false>
__global__ void __launch_bounds__(64, 16) k_first_step(StepArgs a) {
	__shared__ float3 s_r32[32];
	const int lane = threadIdx.x & 31;
	const bool rot = threadIdx.x >= 32;
	const int i = blockIdx.x * 32 + lane;
	const bool live = i < a.N;
	float3 r32 = make_float3(0.f, 0.f, 0.f), fa1 = r32, fbk = r32;
	int sy = 0;
	double4_32a x, y;  // (v, r) on the translation warp, (L, q) on the rotation warp
	float4 lp, la1, lbk;
	auto load_state = [&]() {
		if(live) {
			sy = a.th.sys[i];
			x = rot ? a.angmom[i] : a.vel[i];
			y = rot ? a.quat[i] : a.pos[i];
			if(rot) {
				lp = a.list_pos[i];
				if(a.list_a1) la1 = a.list_a1[i], lbk = a.list_back[i];
			}
		}
	};
	// Inside a graph of steps (offset > 0) the kernel before this one is the previous step's
	// last, launched after the FP64 state and the list build's positions were written: they are
	// read before waiting for it, and only its outputs (the forces, the Bussi update) after.
	// Otherwise (the first step of a graph or a single step, which may follow any kernel that
	// writes the state) everything is read after the wait.
	const bool early = a.th.step_offset > 0;
	if(early) load_state();
	pdl_wait();
	pdl_trigger();
	if(!early) load_state();
	if constexpr(F32) {
		if(live) {
		// backend_precision = float (CUDA_MD.cuh:11-60,556-578): the kicks, the drift and the
		// rotation in FP32 arithmetic on the FP32-representable state (exact conversions); the
		// thermostats act in FP64 on the completed momenta, rounded back to FP32
		const long long s = step_of(a.th);
		const float dt = (float) a.dt, hdt = 0.5f * dt;
		const bool complete = *a.th.open_step == s - 1;
		const long long sp = s - 1;
		const bool brownian = complete && a.th.thermostat == 1 && sp % a.th.newtonian_steps == 0;
		const bool bussi = complete && a.th.thermostat == 2 && *a.th.bussi_stamp == sp;
		const V4 G = reinterpret_cast<const V4 *>(rot ? a.torques : a.forces)[i];
		const float gx = (float) G.x, gy = (float) G.y, gz = (float) G.z;
		float3 u = make_float3(narrow(x.x), narrow(x.y), narrow(x.z));
		if(complete) {
			u.x += gx * hdt;
			u.y += gy * hdt;
			u.z += gz * hdt;
			if(brownian || bussi) {
				x = widen4(u.x, u.y, u.z, 0.f);
				if(brownian) x = brownian_redraw_part(a.th, sy, (a.th.id ? a.th.id[i] : i) - a.th.sys_off[sy], sp, rot ? 1 : 0, x);
				else bussi_rescale_part(a.th, sy, rot ? 1 : 0, x);
				u = make_float3(narrow(x.x), narrow(x.y), narrow(x.z));
			}
		}
		u.x += gx * hdt;
		u.y += gy * hdt;
		u.z += gz * hdt;
		x = widen4(u.x, u.y, u.z, 0.f);
		if(!rot) {
			float3 r = make_float3(narrow(y.x), narrow(y.y), narrow(y.z));
			r.x += u.x * dt;
			r.y += u.y * dt;
			r.z += u.z * dt;
			const double4_32a rd = widen4(r.x, r.y, r.z, 0.f);
			a.vel[i] = x;
			a.pos[i] = rd;
			r32 = mirror_position(a, i, rd);
		}
		else {
			float4 q = make_float4(narrow(y.x), narrow(y.y), narrow(y.z), narrow(y.w));
			rotate_f32(q, u, dt);
			const double4_32a qd = widen4(q.x, q.y, q.z, q.w);
			a.angmom[i] = x;
			a.quat[i] = qd;
			mirror_frame(a, i, qd, fa1, fbk);
		}
		}
	}
	else if(live) {
		const long long s = step_of(a.th);
		const double hdt = 0.5 * a.dt;
		// the previous step's second half kick and thermostat (kept as a separate half kick, so
		// that a state is the same whether or not a run ended at that step)
		const bool complete = *a.th.open_step == s - 1;
		const long long sp = s - 1;
		const bool brownian = complete && a.th.thermostat == 1 && sp % a.th.newtonian_steps == 0;
		const bool bussi = complete && a.th.thermostat == 2 && *a.th.bussi_stamp == sp;
		const V4 G = reinterpret_cast<const V4 *>(rot ? a.torques : a.forces)[i];
		const double gx = widen(G.x), gy = widen(G.y), gz = widen(G.z);
		if(complete) {
			x.x = fma(gx, hdt, x.x);
			x.y = fma(gy, hdt, x.y);
			x.z = fma(gz, hdt, x.z);
			if(brownian) x = brownian_redraw_part(a.th, sy, (a.th.id ? a.th.id[i] : i) - a.th.sys_off[sy], sp, rot ? 1 : 0, x);
			else if(bussi) bussi_rescale_part(a.th, sy, rot ? 1 : 0, x);
		}
		x.x = fma(gx, hdt, x.x);
		x.y = fma(gy, hdt, x.y);
		x.z = fma(gz, hdt, x.z);
		if(!rot) {
			double4_32a r = y;
			r.x += x.x * a.dt;
			r.y += x.y * a.dt;
			r.z += x.z * a.dt;
			a.vel[i] = x;
			a.pos[i] = r;
			r32 = mirror_position(a, i, r);
		}
		else {
			double4_32a q = y;
			// mixed precision: the small rotation as an FP64 sum of an FP32-pair correction (as
			// accurate, far fewer FP64 operations); double precision, or a large step: FP64
			if(!(sizeof(V4) == sizeof(float4) && rotate_small(q.x, q.y, q.z, q.w, x.x, x.y, x.z, 0.5 * a.dt))) rotate(q, x, a.dt);
			a.angmom[i] = x;
			a.quat[i] = q;
			mirror_frame(a, i, q, fa1, fbk);
		}
	}
	// Verlet list staleness (CUDA_mixed.cuh:68, extended to the interaction sites for the term
	// lists), per system, on the rotation warp (the slower one) with the translation warp's FP32
	// position: the translation warp posts it and leaves (named barrier 1: arrive, no wait)
	if(!rot) {
		s_r32[lane] = r32;
		asm volatile("bar.arrive 1, 64;" ::: "memory");
		return;
	}
	asm volatile("bar.sync 1, 64;" ::: "memory");
	if(live && list_stale(a, lp, la1, lbk, s_r32[lane], fa1, fbk)) {
		a.sys_stale[sy] = 1;
		atomicOr(a.flag, 1);
	}
}

// ---------------------------------------------------------------- thermostats

// the Bussi draws of the current step for system blockIdx.x: warp 0 translational (channel 0),
// warp 1 rotational (channel 1)
__global__ void k_bussi_noise(StepArgs a) {
	const long long s = step_of(a.th);
	const int sy = blockIdx.x;
	if(s % a.th.newtonian_steps != 0 || (threadIdx.x & 31) != 0) return;
	const int w = threadIdx.x >> 5;
	if(w > 1) return;
	const int n = a.th.sys_off[sy + 1] - a.th.sys_off[sy];
	Stream rs;
	rs.init(a.th.sys_seed[sy], s, (unsigned) w);
	double sum, rr;
	bussi_draws(rs, w == 0 ? 3 * (n - 1) : 3 * n, sum, rr);
	a.th.bussi_state[16 * sy + 8 + 2 * w] = sum;
	a.th.bussi_state[16 * sy + 9 + 2 * w] = rr;
}

// ---------------------------------------------------------------- Bussi kinetic sums
//
// The update of step s needs, per system, the sums of v, |v|^2 and |L|^2 over the completed
// momenta v + h F and L + h T (h = dt / 2).  They are split as
//   sum (v + h F)^2 = sum v^2 + 2 h sum v.F + h^2 sum F^2   (and likewise for L, T):
// the FP64 sums of the half-kicked state (k_bussi_prep) depend only on the first step and run on
// a side branch of the step graph while the force kernels run (they use the FP64 pipe, which
// the FP32 force kernels leave idle); the force terms (k_bussi_sums) are FP32 products of the
// FP32 forces with the FP32-rounded momenta, summed with compensation, a correction of relative
// size h |F| / |v| to sums that stay FP64.  Both sums run over the same chunks (up to 256
// nucleotides of one system, aligned to the system's first nucleotide), so a system reduces the
// same way in a batch as alone.

__device__ __forceinline__ double shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }

// a float sum with its running error (TwoSum at every addition)
struct CompF {
	float s, e;
};
__device__ __forceinline__ CompF shfl_xor(CompF v, int m) {
	return CompF{__shfl_xor_sync(0xffffffffu, v.s, m), __shfl_xor_sync(0xffffffffu, v.e, m)};
}
__device__ __forceinline__ CompF comp_add(CompF a, CompF b) {
	const float t = a.s + b.s, bp = t - a.s;
	return CompF{t, a.e + b.e + ((a.s - (t - bp)) + (b.s - bp))};
}

// sum over a warp of 8 values per lane by a transposed butterfly (9 additions where 8
// separate reductions take 40); every lane returns the total of value (lane >> 2) & 7.  The
// order is fixed.
template <typename T, typename Add>
__device__ __forceinline__ T warp_transpose_sum8(const T (&x)[8], Add add) {
	const int lane = threadIdx.x & 31;
	const bool h16 = lane & 16, h8 = lane & 8, h4 = lane & 4;
	T w[4], u[2];
#pragma unroll
	for(int k = 0; k < 4; k++) w[k] = add(h16 ? x[k + 4] : x[k], shfl_xor(h16 ? x[k] : x[k + 4], 16));
#pragma unroll
	for(int k = 0; k < 2; k++) u[k] = add(h8 ? w[k + 2] : w[k], shfl_xor(h8 ? w[k] : w[k + 2], 8));
	T t = add(h4 ? u[1] : u[0], shfl_xor(h4 ? u[0] : u[1], 4));
	t = add(t, shfl_xor(t, 2));
	return add(t, shfl_xor(t, 1));
}

// the 8 per-thread values of a block summed in a fixed order into red[0..7] (a 256-thread block)
__device__ __forceinline__ void block_sum8(const double (&x)[8], double *red) {
	__shared__ double part[8][8];
	const double t = warp_transpose_sum8(x, [](double p, double q) { return p + q; });
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
	if((lane & 3) == 0) part[lane >> 2][w] = t;
	__syncthreads();
	if(threadIdx.x < 8) {
		double r = 0;
		for(int u = 0; u < nw; u++) r += part[threadIdx.x][u];
		red[threadIdx.x] = r;
	}
}

__device__ __forceinline__ CompF block_sum8_comp(const CompF (&x)[8]) {
	__shared__ CompF part[8][8];
	const CompF t = warp_transpose_sum8(x, comp_add);
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
	if((lane & 3) == 0) part[lane >> 2][w] = t;
	__syncthreads();
	CompF r{0.f, 0.f};
	if(threadIdx.x < 8)
		for(int u = 0; u < nw; u++) r = comp_add(r, part[threadIdx.x][u]);
	return r;
}

// the block's compensated sums of 8 values as float pairs (written by threads 0..7)
__device__ __forceinline__ void block_sum8f(const CompF (&x)[8], float2 *out) {
	const CompF r = block_sum8_comp(x);
	if(threadIdx.x < 8) out[threadIdx.x] = make_float2(r.s, r.e);
}

// the same into doubles (threads 0..7)
__device__ __forceinline__ void block_sum8(const CompF (&x)[8], double *red) {
	const CompF r = block_sum8_comp(x);
	if(threadIdx.x < 8) red[threadIdx.x] = widen(r.s) + widen(r.e);
}

// Bussi step s, after the first step: per chunk, the FP64 sums of the half-kicked v, |v|^2 and
// |L|^2 (and, in mixed precision, v and L rounded to FP32 for the force terms)
template <typename V4>
__global__ void __launch_bounds__(256) k_bussi_prep(StepArgs a) {
	const long long s = step_of(a.th);
	if(s % a.th.newtonian_steps != 0) return;
	const int c = blockIdx.x;
	const int sy = a.th.chunk_sys[c];
	const int i = a.th.chunk_first[c] + threadIdx.x;
	double x[8] = {0, 0, 0, 0, 0, 0, 0, 0};
	if(i < a.th.sys_off[sy + 1]) {
		const double4_32a v = a.vel[i], L = a.angmom[i];
		x[0] = v.x;
		x[1] = v.y;
		x[2] = v.z;
		x[3] = v.x * v.x + v.y * v.y + v.z * v.z;
		x[4] = L.x * L.x + L.y * L.y + L.z * L.z;
		if(sizeof(V4) == sizeof(float4)) {
			a.th.bussi_vf[i] = make_float4(narrow(v.x), narrow(v.y), narrow(v.z), 0.f);
			a.th.bussi_Lf[i] = make_float4(narrow(L.x), narrow(L.y), narrow(L.z), 0.f);
		}
	}
	block_sum8(x, a.th.bussi_partials + 16 * c);
	// the block that brings a system's last chunk sums them (fixed order) into the system's
	// totals, still on the side branch
	__shared__ int last;
	if(threadIdx.x < 8) __threadfence();
	__syncthreads();
	if(threadIdx.x == 0) {
		const unsigned nc = (unsigned) (a.th.sys_chunk0[sy + 1] - a.th.sys_chunk0[sy]);
		last = atomicAdd(a.th.bussi_prep_done + sy, 1u) == nc - 1u;
		if(last) a.th.bussi_prep_done[sy] = 0u;
	}
	__syncthreads();
	if(!last) return;
	__threadfence();
	const int c0 = a.th.sys_chunk0[sy], nc = a.th.sys_chunk0[sy + 1] - c0;
	double y[8] = {0, 0, 0, 0, 0, 0, 0, 0};
	for(int b = threadIdx.x; b < nc; b += blockDim.x) {
		const double *p = a.th.bussi_partials + 16 * (c0 + b);
#pragma unroll
		for(int k = 0; k < 5; k++) y[k] += __ldcg(p + k);
	}
	__syncthreads();  // the block's scratch is reused
	block_sum8(y, a.th.bussi_tot + 8 * sy);
}

// the update of system sy: the totals of the half-kicked state (k_bussi_prep) and the force
// terms of its chunks, reduced by the block in a fixed chunk order as compensated float pairs
// (the result does not depend on which block runs it); translation on thread 0 and rotation on
// thread 32 (two warps: the chains overlap)
__device__ __forceinline__ void bussi_system_update(const StepArgs &a, int sy, long long s) {
	__shared__ double tot[8];
	const int c0 = a.th.sys_chunk0[sy], nc = a.th.sys_chunk0[sy + 1] - c0;
	CompF y[8];
#pragma unroll
	for(int k = 0; k < 8; k++) y[k] = CompF{0.f, 0.f};
	for(int b = threadIdx.x; b < nc; b += blockDim.x) {
		const float2 *p = a.th.bussi_fpart + 8 * (c0 + b);
#pragma unroll
		for(int k = 0; k < 7; k++) {
			const float2 v = __ldcg(p + k);
			y[k] = comp_add(y[k], CompF{v.x, v.y});
		}
	}
	__syncthreads();  // the block's scratch is reused
	block_sum8(y, tot);
	__syncthreads();
	if(threadIdx.x != 0 && threadIdx.x != 32) return;
	const double *x = a.th.bussi_tot + 8 * sy;
	const double h = 0.5 * a.dt;
	const double sum[5] = {__ldcg(x) + h * tot[0], __ldcg(x + 1) + h * tot[1], __ldcg(x + 2) + h * tot[2],
			__ldcg(x + 3) + 2.0 * h * tot[3] + h * h * tot[4], __ldcg(x + 4) + 2.0 * h * tot[5] + h * h * tot[6]};
	bussi_update(a.th, sy, s, threadIdx.x == 0 ? 0 : 1, sum);
}

// Bussi step s, after its forces: per chunk the sums of F, v.F, |F|^2, L.T and |T|^2 (FP32
// products, compensated sums; FP64 in double precision).  The block that brings a system's last
// chunk (a per-system arrival counter) makes that system's update, so there is no separate
// update launch.
template <typename V4>
__global__ void __launch_bounds__(256) k_bussi_sums(StepArgs a) {
	pdl_wait();  // launched after the force kernels
	pdl_trigger();
	const long long s = step_of(a.th);
	if(s % a.th.newtonian_steps != 0) return;
	const int c = blockIdx.x;
	const int sy = a.th.chunk_sys[c];
	const int i = a.th.chunk_first[c] + threadIdx.x;
	const bool live = i < a.th.sys_off[sy + 1];
	if(sizeof(V4) == sizeof(float4)) {
		CompF x[8];
#pragma unroll
		for(int k = 0; k < 8; k++) x[k] = CompF{0.f, 0.f};
		if(live) {
			const float4 F = reinterpret_cast<const float4 *>(a.forces)[i], T = reinterpret_cast<const float4 *>(a.torques)[i];
			const float4 v = a.th.bussi_vf[i], L = a.th.bussi_Lf[i];
			x[0].s = F.x;
			x[1].s = F.y;
			x[2].s = F.z;
			x[3].s = v.x * F.x + v.y * F.y + v.z * F.z;
			x[4].s = F.x * F.x + F.y * F.y + F.z * F.z;
			x[5].s = L.x * T.x + L.y * T.y + L.z * T.z;
			x[6].s = T.x * T.x + T.y * T.y + T.z * T.z;
		}
		block_sum8f(x, a.th.bussi_fpart + 8 * c);
	}
	else {
		double x[8] = {0, 0, 0, 0, 0, 0, 0, 0};
		if(live) {
			const double4_32a F = reinterpret_cast<const double4_32a *>(a.forces)[i],
							  T = reinterpret_cast<const double4_32a *>(a.torques)[i];
			const double4_32a v = a.vel[i], L = a.angmom[i];
			x[0] = F.x;
			x[1] = F.y;
			x[2] = F.z;
			x[3] = v.x * F.x + v.y * F.y + v.z * F.z;
			x[4] = F.x * F.x + F.y * F.y + F.z * F.z;
			x[5] = L.x * T.x + L.y * T.y + L.z * T.z;
			x[6] = T.x * T.x + T.y * T.y + T.z * T.z;
		}
		// FP64 sums, kept as float pairs like the mixed-precision ones (hi + lo carries 48 bits)
		__shared__ double red[8];
		block_sum8(x, red);
		__syncthreads();
		if(threadIdx.x < 8) {
			float hi, lo;
			split_rn(red[threadIdx.x], hi, lo);
			a.th.bussi_fpart[8 * c + threadIdx.x] = make_float2(hi, lo);
		}
	}
	__shared__ int last;
	if(threadIdx.x < 8) __threadfence();  // the partials are visible device-wide before this block arrives
	__syncthreads();
	if(threadIdx.x == 0) {
		const unsigned nc = (unsigned) (a.th.sys_chunk0[sy + 1] - a.th.sys_chunk0[sy]);
		last = atomicAdd(a.th.bussi_done + sy, 1u) == nc - 1u;
		if(last) {
			a.th.bussi_done[sy] = 0u;  // every chunk has arrived: ready for the next step
			// the next first step applies the rescaling of step s (every system updates at the same steps)
			if(sy == 0) *a.th.bussi_stamp = s;
		}
	}
	__syncthreads();
	if(!last) return;
	__threadfence();
	bussi_system_update(a, sy, s);
}

__global__ void k_step_advance(StepArgs a, int K) {
	if(threadIdx.x == 0 && blockIdx.x == 0) *a.th.step_base += K;
}

// end of a run: the last step's second half kick and thermostat ...
template <typename V4>
__global__ void k_step_flush(StepArgs a) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	const long long sp = *a.th.step_base - 1;
	if(i >= a.N || *a.th.open_step != sp) return;
	const V4 F = reinterpret_cast<const V4 *>(a.forces)[i];
	const V4 T = reinterpret_cast<const V4 *>(a.torques)[i];
	double4_32a v = a.vel[i], L = a.angmom[i];
	complete_step(a.th, i, a.th.sys[i], sp, F, T, v, L);
	a.vel[i] = a.f32 ? round4(v) : v;
	a.angmom[i] = a.f32 ? round4(L) : L;
}

// ... after which nothing is pending
__global__ void k_step_flush_clear(StepArgs a) {
	if(threadIdx.x == 0 && blockIdx.x == 0) {
		*a.th.open_step = OXGB_NO_STEP;
		*a.th.bussi_stamp = OXGB_NO_STEP;
	}
}

// The caller's state arrays (positions, quaternions, velocities, angular momenta: 3, 4, 3 and 3
// doubles per nucleotide, the four arrays one after the other in `in`) into the FP64 state, each
// quaternion normalised (sums and products rounded in a fixed order); the lowest nucleotide whose
// quaternion cannot be normalised is kept in *bad.  With check_only nothing is written but *bad.
__global__ void k_unpack_state(StepArgs a, const double *in, int *bad, int check_only) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= a.N) return;
	const long long N = a.N;
	const double *p = in + 3 * (long long) i, *q = in + 3 * N + 4 * (long long) i, *v = in + 7 * N + 3 * (long long) i,
				 *l = in + 10 * N + 3 * (long long) i;
	const double n2 = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(q[0], q[0]), __dmul_rn(q[1], q[1])), __dmul_rn(q[2], q[2])),
			__dmul_rn(q[3], q[3]));
	double n = sqrt(n2);
	if(!(n > 0.5)) {
		atomicMin(bad, i);
		n = 1.0;
	}
	if(check_only) return;
	double4_32a P = make_double4_32a(p[0], p[1], p[2], 0.0);
	double4_32a Q = make_double4_32a(__ddiv_rn(q[0], n), __ddiv_rn(q[1], n), __ddiv_rn(q[2], n), __ddiv_rn(q[3], n));
	double4_32a V = make_double4_32a(v[0], v[1], v[2], 0.0), M = make_double4_32a(l[0], l[1], l[2], 0.0);
	if(a.f32) {  // backend_precision = float: the state FP32 from the start
		P = round4(P);
		Q = round4(Q);
		V = round4(V);
		M = round4(M);
	}
	a.pos[i] = P;
	a.quat[i] = Q;
	a.vel[i] = V;
	a.angmom[i] = M;
}

// the FP64 state into the caller's layout and order (the reverse of k_unpack_state)
__global__ void k_pack_state(StepArgs a, double *out) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= a.N) return;
	const long long N = a.N;
	const long long c = a.th.id ? a.th.id[i] : i;  // the caller's index
	double *p = out + 3 * c, *q = out + 3 * N + 4 * c, *v = out + 7 * N + 3 * c, *l = out + 10 * N + 3 * c;
	const double4_32a r = a.pos[i], o = a.quat[i], u = a.vel[i], m = a.angmom[i];
	p[0] = r.x, p[1] = r.y, p[2] = r.z;
	q[0] = o.x, q[1] = o.y, q[2] = o.z, q[3] = o.w;
	v[0] = u.x, v[1] = u.y, v[2] = u.z;
	l[0] = m.x, l[1] = m.y, l[2] = m.z;
}

// velocities and angular momenta of nucleotides lo .. hi - 1 times f (a replica exchange)
__global__ void k_scale_momenta(StepArgs a, int lo, int hi, double f) {
	const int i = lo + blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= hi) return;
	double4_32a v = a.vel[i], L = a.angmom[i];
	v.x *= f;
	v.y *= f;
	v.z *= f;
	L.x *= f;
	L.y *= f;
	L.z *= f;
	a.vel[i] = v;
	a.angmom[i] = L;
}

// per-chunk FP64 sums: potential energy (F.w / 2), translational and rotational kinetic energy
template <typename V4>
__global__ void __launch_bounds__(256) k_system_sums(StepArgs a, double *out) {
	const int c = blockIdx.x;
	const int sy = a.th.chunk_sys[c];
	const int i = a.th.chunk_first[c] + threadIdx.x;
	double acc[3] = {0, 0, 0};
	if(i < a.th.sys_off[sy + 1]) {
		const V4 F = reinterpret_cast<const V4 *>(a.forces)[i];
		const double4_32a v = a.vel[i], L = a.angmom[i];
		acc[0] = 0.5 * (double) F.w;
		acc[1] = 0.5 * (v.x * v.x + v.y * v.y + v.z * v.z);
		acc[2] = 0.5 * (L.x * L.x + L.y * L.y + L.z * L.z);
	}
	__shared__ double red[3][8];
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
	for(int k = 0; k < 3; k++) {
		double x = acc[k];
		for(int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
		if(lane == 0) red[k][w] = x;
	}
	__syncthreads();
	if(threadIdx.x < 3) {
		double x = 0;
		for(int u = 0; u < nw; u++) x += red[threadIdx.x][u];
		out[c * 4 + threadIdx.x] = x;
	}
}

__global__ void k_set_conditional(const int *flag, cudaGraphConditionalHandle h) {
	pdl_wait();  // launched after the first step, which raises the flag
	if(threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(h, *flag != 0 ? 1u : 0u);
}

// ---------------------------------------------------------------- launchers

static inline int blocks_for(int N, int tpb) { return N > 0 ? (N + tpb - 1) / tpb : 1; }

cudaError_t launch_first_step(const StepArgs &a, bool double_forces, cudaStream_t s) {
	// two-warp blocks of 32 nucleotides: the FP64 work (1/64 of the FP32 rate) spreads evenly over
	// the SMs
	if(double_forces) return launch_after(k_first_step<double4_32a>, dim3(blocks_for(a.N, 32)), dim3(64), 0, s, a);
	if(a.f32) return launch_after(k_first_step<float4, true>, dim3(blocks_for(a.N, 32)), dim3(64), 0, s, a);
	return launch_after(k_first_step<float4>, dim3(blocks_for(a.N, 32)), dim3(64), 0, s, a);
}

cudaError_t launch_bussi_noise(const StepArgs &a, cudaStream_t s) {
	k_bussi_noise<<<a.th.n_systems, 64, 0, s>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_bussi_prep(const StepArgs &a, int n_chunks, bool double_forces, cudaStream_t s) {
	if(double_forces) k_bussi_prep<double4_32a><<<n_chunks, 256, 0, s>>>(a);
	else k_bussi_prep<float4><<<n_chunks, 256, 0, s>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_bussi_reduce(const StepArgs &a, int n_chunks, bool double_forces, cudaStream_t s) {
	if(double_forces) return launch_after(k_bussi_sums<double4_32a>, dim3(n_chunks), dim3(256), 0, s, a);
	return launch_after(k_bussi_sums<float4>, dim3(n_chunks), dim3(256), 0, s, a);
}

cudaError_t launch_step_advance(const StepArgs &a, int K, cudaStream_t s) {
	k_step_advance<<<1, 32, 0, s>>>(a, K);
	return cudaGetLastError();
}

cudaError_t launch_step_flush(const StepArgs &a, bool double_forces, cudaStream_t s) {
	if(double_forces) k_step_flush<double4_32a><<<blocks_for(a.N, 256), 256, 0, s>>>(a);
	else k_step_flush<float4><<<blocks_for(a.N, 256), 256, 0, s>>>(a);
	k_step_flush_clear<<<1, 32, 0, s>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_set_conditional(const int *flag, cudaGraphConditionalHandle h, cudaStream_t s) {
	return launch_after(k_set_conditional, dim3(1), dim3(32), 0, s, flag, h);
}

cudaError_t launch_make_mirrors(const StepArgs &a, cudaStream_t s) {
	k_make_mirrors<<<blocks_for(a.N, 256), 256, 0, s>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_unpack_state(const StepArgs &a, const double *in, int *bad, bool check_only, cudaStream_t s) {
	k_unpack_state<<<blocks_for(a.N, 256), 256, 0, s>>>(a, in, bad, check_only ? 1 : 0);
	return cudaGetLastError();
}

__global__ void k_identity_order(int *id, int *slot, int N) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= N) return;
	id[i] = i;
	slot[i] = i;
}

cudaError_t launch_identity_order(int *id, int *slot, int N, cudaStream_t s) {
	k_identity_order<<<blocks_for(N, 256), 256, 0, s>>>(id, slot, N);
	return cudaGetLastError();
}

cudaError_t launch_pack_state(const StepArgs &a, double *out, cudaStream_t s) {
	k_pack_state<<<blocks_for(a.N, 256), 256, 0, s>>>(a, out);
	return cudaGetLastError();
}

cudaError_t launch_scale_momenta(const StepArgs &a, int lo, int hi, double f, cudaStream_t s) {
	if(hi > lo) k_scale_momenta<<<blocks_for(hi - lo, 256), 256, 0, s>>>(a, lo, hi, f);
	return cudaGetLastError();
}

cudaError_t launch_system_sums(const StepArgs &a, int n_chunks, bool double_forces, double *out, cudaStream_t s) {
	if(double_forces) k_system_sums<double4_32a><<<n_chunks, 256, 0, s>>>(a, out);
	else k_system_sums<float4><<<n_chunks, 256, 0, s>>>(a, out);
	return cudaGetLastError();
}

}  // namespace oxgb
