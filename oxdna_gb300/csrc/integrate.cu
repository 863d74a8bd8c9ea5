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
// The second half kick is fused into the force kernel.
#include "kernels.h"

namespace oxgb {

// ---------------------------------------------------------------- Philox-4x32-10

__device__ __forceinline__ void philox(unsigned k0, unsigned k1, unsigned c0, unsigned c1, unsigned c2, unsigned c3,
		unsigned out[4]) {
	const unsigned M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
	for(int r = 0; r < 10; r++) {
		const unsigned hi0 = __umulhi(M0, c0), lo0 = M0 * c0;
		const unsigned hi1 = __umulhi(M1, c2), lo1 = M1 * c2;
		const unsigned n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
		c0 = n0;
		c1 = lo1;
		c2 = n2;
		c3 = lo0;
		k0 += W0;
		k1 += W1;
	}
	out[0] = c0;
	out[1] = c1;
	out[2] = c2;
	out[3] = c3;
}

__device__ __forceinline__ double u01(unsigned x) { return ((double) x + 1.0) * (1.0 / 4294967296.0); }

__device__ __forceinline__ void box_muller(unsigned ua, unsigned ub, double &g0, double &g1) {
	const double r = sqrt(-2.0 * log(u01(ua)));
	double s, c;
	sincos(6.283185307179586 * u01(ub), &s, &c);
	g0 = r * c;
	g1 = r * s;
}

#define RNG_BROWNIAN 0x42524f57u
#define RNG_BUSSI 0x42555353u

struct Stream {
	unsigned k0, k1, s0, s1, c, blk, idx;
	unsigned buf[4];
	__device__ void init(unsigned long long seed, long long s, unsigned channel) {
		k0 = (unsigned) seed;
		k1 = (unsigned) (seed >> 32);
		s0 = (unsigned) s;
		s1 = (unsigned) ((unsigned long long) s >> 32);
		c = RNG_BUSSI ^ channel;
		blk = 0;
		idx = 4;
	}
	__device__ double u() {
		if(idx == 4) {
			philox(k0, k1, s0, s1, c, blk++, buf);
			idx = 0;
		}
		return u01(buf[idx++]);
	}
	__device__ double gauss() {
		const double a = u(), b = u();
		return sqrt(-2.0 * log(a)) * cos(6.283185307179586 * b);
	}
};

// gamma deviate of integer order (the Numerical Recipes algorithm the reference uses)
__device__ double gamdev(Stream &st, int ia) {
	if(ia < 6) {
		double x = 1.0;
		for(int j = 1; j <= ia; j++) x *= st.u();
		return -log(x);
	}
	const double am = ia - 1, s = sqrt(2.0 * am + 1.0);
	double x = am, e, y = 0.0, v1, v2;
	// every rejection loop is bounded; each accepts with probability > 0.5, so the bounds are
	// never reached by a working random stream
	for(int guard = 0; guard < 1000; guard++) {
		bool got = false;
		for(int g2 = 0; g2 < 1000 && !got; g2++) {
			for(int g1 = 0; g1 < 1000; g1++) {
				v1 = st.u();
				v2 = 2.0 * st.u() - 1.0;
				if(v1 * v1 + v2 * v2 <= 1.0) break;
			}
			y = v2 / v1;
			x = s * y + am;
			got = x > 0.0;
		}
		if(!got) return am;
		e = (1.0 + y * y) * exp(am * log(x / am) - s * y);
		if(st.u() <= e) return x;
	}
	return am;
}

__device__ double sum_noises(Stream &st, int nn) {
	if(nn == 0) return 0.0;
	if(nn == 1) {
		const double r = st.gauss();
		return r * r;
	}
	if(nn % 2 == 0) return 2.0 * gamdev(st, nn / 2);
	const double r = st.gauss();
	return 2.0 * gamdev(st, (nn - 1) / 2) + r * r;
}

// the two draws of one kinetic-energy update (BussiThermostat::_update_K, BussiThermostat.cpp:
// 55-65): the Gaussian r, then the sum of dof - 1 squared Gaussians; they do not depend on the
// state, so they are drawn apart from (and concurrently with) the force evaluation
__device__ void bussi_draws(Stream &st, int dof, double &sum, double &rr) {
	rr = st.gauss();
	sum = sum_noises(st, dof - 1);
}

__device__ void update_K(double &K, int dof, double T, double c, double sum, double rr) {
	const double Kt = 0.5 * dof * T;
	const double dK = (1.0 - c) * (Kt * (sum + rr * rr) / dof - K) + 2.0 * rr * sqrt(K * Kt / dof * (1.0 - c) * c);
	K += dK;
}

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

template <typename V4>
__global__ void k_first_step(StepArgs a) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= a.N) return;
	const V4 F = reinterpret_cast<const V4 *>(a.forces)[i];
	const V4 T = reinterpret_cast<const V4 *>(a.torques)[i];
	const double hdt = 0.5 * a.dt;
	double4_32a v = a.vel[i], r = a.pos[i], L = a.angmom[i], q = a.quat[i];
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
		if(x2 < 1e-2) {
			// sin(x) / x and cos(x) as Taylor series in x^2 (truncation below 1e-20 for |x| < 0.1):
			// no square root, range reduction or division, which are slow in FP64
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
	// Verlet list staleness (CUDA_mixed.cuh:68, extended to the interaction sites for the term lists)
	if(list_stale(a, i, r)) atomicOr(a.flag, 1);
}

// ---------------------------------------------------------------- thermostats

__global__ void k_brownian(StepArgs a) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	const long long s = *a.step;
	if(i >= a.N || s % a.newtonian_steps != 0) return;
	unsigned o0[4], o1[4];
	const unsigned k0 = (unsigned) a.seed, k1 = (unsigned) (a.seed >> 32);
	const unsigned s0 = (unsigned) s, s1 = (unsigned) ((unsigned long long) s >> 32);
	philox(k0, k1, s0, s1, RNG_BROWNIAN, (unsigned) (2 * i), o0);
	philox(k0, k1, s0, s1, RNG_BROWNIAN, (unsigned) (2 * i + 1), o1);
	double g[6];
	box_muller(o0[2], o0[3], g[0], g[1]);
	box_muller(o1[0], o1[1], g[2], g[3]);
	box_muller(o1[2], o1[3], g[4], g[5]);
	if(u01(o0[0]) < a.pt) a.vel[i] = make_double4_32a(g[0] * a.sqrtT, g[1] * a.sqrtT, g[2] * a.sqrtT, 0.0);
	if(u01(o0[1]) < a.pr) a.angmom[i] = make_double4_32a(g[3] * a.sqrtT, g[4] * a.sqrtT, g[5] * a.sqrtT, 0.0);
}

__global__ void k_bussi_noise(StepArgs a) {
	const long long s = *a.step;
	if(s % a.newtonian_steps != 0 || (threadIdx.x & 31) != 0) return;
	// warp 0: translational (channel 0), warp 1: rotational (channel 1)
	const int w = threadIdx.x >> 5;
	if(w > 1) return;
	Stream rs;
	rs.init(a.seed, s, (unsigned) w);
	double sum, rr;
	bussi_draws(rs, w == 0 ? 3 * (a.N - 1) : 3 * a.N, sum, rr);
	a.bussi_state[8 + 2 * w] = sum;
	a.bussi_state[9 + 2 * w] = rr;
}

// per-block sums of v, v^2 and L^2; the last block to finish reduces the block sums in a fixed
// order (deterministic) and updates the running kinetic energies and the rescaling factors
__global__ void __launch_bounds__(256) k_bussi_partial(StepArgs a) {
	const long long s = *a.step;
	if(s % a.newtonian_steps != 0) return;
	double acc[5] = {0, 0, 0, 0, 0};
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		const double4_32a v = a.vel[i], L = a.angmom[i];
		acc[0] += v.x;
		acc[1] += v.y;
		acc[2] += v.z;
		acc[3] += v.x * v.x + v.y * v.y + v.z * v.z;
		acc[4] += L.x * L.x + L.y * L.y + L.z * L.z;
	}
	__shared__ double red[5][8];
	__shared__ bool last;
#pragma unroll
	for(int k = 0; k < 5; k++) {
		double x = acc[k];
		for(int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
		if((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = x;
	}
	__syncthreads();
	if(threadIdx.x < 5) {
		double x = 0;
		for(int w = 0; w < (int) (blockDim.x >> 5); w++) x += red[threadIdx.x][w];
		a.bussi_partials[blockIdx.x * 8 + threadIdx.x] = x;
		__threadfence();
	}
	__syncthreads();
	if(threadIdx.x == 0) last = atomicAdd(a.bussi_done, 1u) == gridDim.x - 1;
	__syncthreads();
	if(!last) return;
	__threadfence();
	// fixed-order reduction of the block sums: thread t takes blocks t, t + 256, ...
	double part[5] = {0, 0, 0, 0, 0};
	for(int b = threadIdx.x; b < a.bussi_blocks; b += blockDim.x)
#pragma unroll
		for(int k = 0; k < 5; k++) part[k] += __ldcg(a.bussi_partials + b * 8 + k);
#pragma unroll
	for(int k = 0; k < 5; k++) {
		double x = part[k];
		for(int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
		if((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = x;
	}
	__syncthreads();
	if(threadIdx.x != 0) return;
	double sum[5];
	for(int k = 0; k < 5; k++) {
		double x = 0;
		for(int w = 0; w < (int) (blockDim.x >> 5); w++) x += red[k][w];
		sum[k] = x;
	}
	const double N = a.N;
	const double vc[3] = {sum[0] / N, sum[1] / N, sum[2] / N};
	const double Kt_now = 0.5 * (sum[3] - N * (vc[0] * vc[0] + vc[1] * vc[1] + vc[2] * vc[2]));
	const double Kr_now = 0.5 * sum[4];
	double *st = a.bussi_state;
	update_K(st[0], 3 * (a.N - 1), a.T, a.bussi_c, __ldcg(st + 8), __ldcg(st + 9));
	update_K(st[1], 3 * a.N, a.T, a.bussi_c, __ldcg(st + 10), __ldcg(st + 11));
	st[2] = sqrt(st[0] / Kt_now);
	st[3] = sqrt(st[1] / Kr_now);
	st[4] = vc[0];
	st[5] = vc[1];
	st[6] = vc[2];
	*a.bussi_done = 0;
}

__global__ void k_bussi_apply(StepArgs a) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	const long long s = *a.step;
	if(i >= a.N || s % a.newtonian_steps != 0) return;
	const double *st = a.bussi_state;
	const double ft = st[2], fr = st[3];
	double4_32a v = a.vel[i], L = a.angmom[i];
	v.x = (v.x - st[4]) * ft + st[4];
	v.y = (v.y - st[5]) * ft + st[5];
	v.z = (v.z - st[6]) * ft + st[6];
	L.x *= fr;
	L.y *= fr;
	L.z *= fr;
	a.vel[i] = v;
	a.angmom[i] = L;
}

__global__ void k_step_advance(StepArgs a) {
	if(threadIdx.x == 0 && blockIdx.x == 0) *a.step += 1;
}

__global__ void k_set_conditional(const int *flag, cudaGraphConditionalHandle h) {
	if(threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(h, *flag != 0 ? 1u : 0u);
}

__global__ void k_kinetic(StepArgs a, double *out) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= a.N) return;
	const double4_32a v = a.vel[i], L = a.angmom[i];
	atomicAdd(out, 0.5 * (v.x * v.x + v.y * v.y + v.z * v.z));
	atomicAdd(out + 1, 0.5 * (L.x * L.x + L.y * L.y + L.z * L.z));
}

// ---------------------------------------------------------------- launchers

static inline int blocks_for(int N, int tpb) { return N > 0 ? (N + tpb - 1) / tpb : 1; }

cudaError_t launch_first_step(const StepArgs &a, bool double_forces, cudaStream_t s) {
	if(double_forces) k_first_step<double4_32a><<<blocks_for(a.N, 256), 256, 0, s>>>(a);
	else k_first_step<float4><<<blocks_for(a.N, 256), 256, 0, s>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_thermostat(const StepArgs &a, cudaStream_t s) {
	if(a.thermostat == 1) k_brownian<<<blocks_for(a.N, 256), 256, 0, s>>>(a);
	else if(a.thermostat == 2) {
		k_bussi_partial<<<a.bussi_blocks, 256, 0, s>>>(a);
		k_bussi_apply<<<blocks_for(a.N, 256), 256, 0, s>>>(a);
	}
	return cudaGetLastError();
}

cudaError_t launch_bussi_noise(const StepArgs &a, cudaStream_t s) {
	k_bussi_noise<<<1, 64, 0, s>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_step_advance(const StepArgs &a, cudaStream_t s) {
	k_step_advance<<<1, 32, 0, s>>>(a);
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

cudaError_t launch_kinetic(const StepArgs &a, double *out2, cudaStream_t s) {
	cudaError_t e = cudaMemsetAsync(out2, 0, 2 * sizeof(double), s);
	if(e != cudaSuccess) return e;
	k_kinetic<<<blocks_for(a.N, 256), 256, 0, s>>>(a, out2);
	return cudaGetLastError();
}

}  // namespace oxgb
