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
// first half kick; the Bussi sums and update run after the forces (k_bussi_sums) and its
// draws on a parallel branch of the step graph (k_bussi_noise).  No FP64 work is left in the force
// kernels, whose lanes are mostly idle at the epilogue.
#include "thermo.cuh"

namespace oxgb {

// ---------------------------------------------------------------- FP32 mirrors

__device__ __forceinline__ void write_mirror(const StepArgs &a, int i, const double4_32a &r, const double4_32a &q) {
	float4 hi = a.pos_hi[i], lo = a.pos_lo[i];
	hi.x = (float) r.x;
	hi.y = (float) r.y;
	hi.z = (float) r.z;
	lo.x = (float) (r.x - (double) hi.x);
	lo.y = (float) (r.y - (double) hi.y);
	lo.z = (float) (r.z - (double) hi.z);
	a.pos_hi[i] = hi;
	a.pos_lo[i] = lo;
	// body axes from the FP64 quaternion, each component rounded once
	v3<double> a1, a2, a3;
	quat_frame(q.x, q.y, q.z, q.w, a1, a2, a3);
	a.fa1[i] = make_float4((float) a1.x, (float) a1.y, (float) a1.z, 0.f);
	a.fa3[i] = make_float4((float) a3.x, (float) a3.y, (float) a3.z, 0.f);
	// grooved backbone offset (src/Particles/DNANucleotide.cpp:79) and the strand-end flag
	if(a.fback) {
		const double b1 = (double) OXM_POS_MM_BACK1, b2 = (double) OXM_POS_MM_BACK2;
		const int2 bd = a.bonds[i];
		a.fback[i] = make_float4((float) (a1.x * b1 + a2.x * b2), (float) (a1.y * b1 + a2.y * b2), (float) (a1.z * b1 + a2.z * b2),
				(bd.x < 0 || bd.y < 0) ? 1.f : 0.f);
	}
}

// true if the centre or any interaction site moved more than the skin since the last list build
__device__ __forceinline__ bool list_stale(const StepArgs &a, int i, const double4_32a &r) {
	const float4 lp = a.list_pos[i];
	const float dx = (float) r.x - lp.x, dy = (float) r.y - lp.y, dz = (float) r.z - lp.z;
	if(dx * dx + dy * dy + dz * dz > a.skin2) return true;
	if(!a.list_a1) return false;
	const float4 a1 = a.fa1[i], la1 = a.list_a1[i], bk = a.fback[i], lbk = a.list_back[i];
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
	write_mirror(a, i, a.pos[i], a.quat[i]);
}

// ---------------------------------------------------------------- first half step

__device__ __forceinline__ long long step_of(const ThermoArgs &t) { return *t.step_base + t.step_offset; }

// completes step sp of nucleotide i (system sy): its second half kick (CUDA_mixed.cuh:71-93)
// and its thermostat (Brownian redraw or Bussi rescaling)
template <typename V4>
__device__ __forceinline__ void complete_step(const ThermoArgs &t, int i, int sy, long long sp, const V4 &F, const V4 &T,
		double4_32a &v, double4_32a &L) {
	const double hdt = 0.5 * t.dt;
	v.x += (double) F.x * hdt;
	v.y += (double) F.y * hdt;
	v.z += (double) F.z * hdt;
	L.x += (double) T.x * hdt;
	L.y += (double) T.y * hdt;
	L.z += (double) T.z * hdt;
	if(t.thermostat == 1 && sp % t.newtonian_steps == 0) brownian_redraw(t, sy, i - t.sys_off[sy], sp, v, L);
	else if(t.thermostat == 2 && *t.bussi_stamp == sp) bussi_rescale(t, sy, v, L);
}

template <typename V4>
__global__ void k_first_step(StepArgs a) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= a.N) return;
	const long long s = step_of(a.th);
	const int sy = a.th.sys[i];
	const V4 F = reinterpret_cast<const V4 *>(a.forces)[i];
	const V4 T = reinterpret_cast<const V4 *>(a.torques)[i];
	const double hdt = 0.5 * a.dt;
	double4_32a v = a.vel[i], r = a.pos[i], L = a.angmom[i], q = a.quat[i];
	// the previous step's second half kick and thermostat (kept as a separate half kick, so that
	// a state is the same whether or not a run ended at that step)
	if(*a.th.open_step == s - 1) complete_step(a.th, i, sy, s - 1, F, T, v, L);
	v.x += (double) F.x * hdt;
	v.y += (double) F.y * hdt;
	v.z += (double) F.z * hdt;
	r.x += v.x * a.dt;
	r.y += v.y * a.dt;
	r.z += v.z * a.dt;
	L.x += (double) T.x * hdt;
	L.y += (double) T.y * hdt;
	L.z += (double) T.z * hdt;
	// rotation by dt|L| about L (body frame): q <- q * (sin(th/2) L^, cos(th/2))
	const double L2 = L.x * L.x + L.y * L.y + L.z * L.z;
	if(L2 > 0.0) {
		const double hd = 0.5 * a.dt, x2 = hd * hd * L2;  // x = th / 2
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
	a.vel[i] = v;
	a.pos[i] = r;
	a.angmom[i] = L;
	a.quat[i] = q;
	write_mirror(a, i, r, q);
	// Verlet list staleness (CUDA_mixed.cuh:68, extended to the interaction sites for the term
	// lists), per system
	if(list_stale(a, i, r)) {
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

// the update of system sy from its chunk sums, reduced by the block in a fixed chunk order (the
// result does not depend on which block runs it): translation on thread 0 and rotation on
// thread 32 (two warps: the chains overlap).  red is the block's shared scratch.
__device__ __forceinline__ void bussi_system_update(const StepArgs &a, int sy, long long s, double (*red)[8]) {
	const int c0 = a.th.sys_chunk0[sy], nc = a.th.sys_chunk0[sy + 1] - c0;
	double part[5] = {0, 0, 0, 0, 0};
	for(int b = threadIdx.x; b < nc; b += blockDim.x)
#pragma unroll
		for(int k = 0; k < 5; k++) part[k] += __ldcg(a.th.bussi_partials + (c0 + b) * 8 + k);
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
	for(int k = 0; k < 5; k++) {
		double x = part[k];
		for(int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
		if(lane == 0) red[k][w] = x;
	}
	__syncthreads();
	if(threadIdx.x != 0 && threadIdx.x != 32) return;
	double sum[5];
	for(int k = 0; k < 5; k++) {
		double x = 0;
		for(int u = 0; u < nw; u++) x += red[k][u];
		sum[k] = x;
	}
	bussi_update(a.th, sy, s, threadIdx.x == 0 ? 0 : 1, sum);
}

// Bussi step s, after its forces: sums of v, |v|^2 and |L|^2 over the completed velocities
// v + dt/2 F (computed here, stored by the next first step), one block per chunk of up to 256
// nucleotides of one system.  The block that finishes a system's last outstanding chunk (a
// per-system arrival counter) makes that system's update, so there is no separate update launch.
template <typename V4>
__global__ void __launch_bounds__(256) k_bussi_sums(StepArgs a) {
	const long long s = step_of(a.th);
	if(s % a.th.newtonian_steps != 0) return;
	const int c = blockIdx.x;
	const int sy = a.th.chunk_sys[c];
	const int i = a.th.chunk_first[c] + threadIdx.x;
	const double hdt = 0.5 * a.dt;
	double acc[5] = {0, 0, 0, 0, 0};
	if(i < a.th.sys_off[sy + 1]) {
		const V4 F = reinterpret_cast<const V4 *>(a.forces)[i];
		const V4 T = reinterpret_cast<const V4 *>(a.torques)[i];
		double4_32a v = a.vel[i], L = a.angmom[i];
		v.x += (double) F.x * hdt;
		v.y += (double) F.y * hdt;
		v.z += (double) F.z * hdt;
		L.x += (double) T.x * hdt;
		L.y += (double) T.y * hdt;
		L.z += (double) T.z * hdt;
		acc[0] = v.x;
		acc[1] = v.y;
		acc[2] = v.z;
		acc[3] = v.x * v.x + v.y * v.y + v.z * v.z;
		acc[4] = L.x * L.x + L.y * L.y + L.z * L.z;
	}
	__shared__ double red[5][8];
	__shared__ int last;
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
	for(int k = 0; k < 5; k++) {
		double x = acc[k];
		for(int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
		if(lane == 0) red[k][w] = x;
	}
	__syncthreads();
	if(threadIdx.x < 5) {
		double x = 0;
		for(int u = 0; u < nw; u++) x += red[threadIdx.x][u];
		a.th.bussi_partials[c * 8 + threadIdx.x] = x;
		__threadfence();  // the partial is visible device-wide before this block arrives
	}
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
	bussi_system_update(a, sy, s, red);
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
	a.vel[i] = v;
	a.angmom[i] = L;
}

// ... after which nothing is pending
__global__ void k_step_flush_clear(StepArgs a) {
	if(threadIdx.x == 0 && blockIdx.x == 0) {
		*a.th.open_step = OXGB_NO_STEP;
		*a.th.bussi_stamp = OXGB_NO_STEP;
	}
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
	if(threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(h, *flag != 0 ? 1u : 0u);
}

// ---------------------------------------------------------------- launchers

static inline int blocks_for(int N, int tpb) { return N > 0 ? (N + tpb - 1) / tpb : 1; }

cudaError_t launch_first_step(const StepArgs &a, bool double_forces, cudaStream_t s) {
	// one-warp blocks: the FP64 work (1/64 of the FP32 rate) spreads evenly over the SMs
	if(double_forces) k_first_step<double4_32a><<<blocks_for(a.N, 32), 32, 0, s>>>(a);
	else k_first_step<float4><<<blocks_for(a.N, 32), 32, 0, s>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_bussi_noise(const StepArgs &a, cudaStream_t s) {
	k_bussi_noise<<<a.th.n_systems, 64, 0, s>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_bussi_reduce(const StepArgs &a, int n_chunks, bool double_forces, cudaStream_t s) {
	if(double_forces) k_bussi_sums<double4_32a><<<n_chunks, 256, 0, s>>>(a);
	else k_bussi_sums<float4><<<n_chunks, 256, 0, s>>>(a);
	return cudaGetLastError();
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
	k_set_conditional<<<1, 32, 0, s>>>(flag, h);
	return cudaGetLastError();
}

cudaError_t launch_make_mirrors(const StepArgs &a, cudaStream_t s) {
	k_make_mirrors<<<blocks_for(a.N, 256), 256, 0, s>>>(a);
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
