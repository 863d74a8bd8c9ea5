// Random streams and thermostat arithmetic of the integrator kernels (integrate.cu).
//
// Random numbers come from a counter-based Philox-4x32-10 stream keyed by (seed, step,
// particle), so runs are reproducible and graph-replayable; the oracle (oracle/dna2_oracle.c,
// oxo_philox) draws the same numbers.  The Bussi kinetic-energy update follows
// src/Backends/Thermostats/BussiThermostat.cpp:44-160 and the Brownian ("john") redraw
// src/CUDA/Thermostats/CUDABrownianThermostat.cu:15-51.
#pragma once

#include "kernels.h"

namespace oxgb {

// ---------------------------------------------------------------- Philox-4x32-10

static __device__ __forceinline__ void philox(unsigned k0, unsigned k1, unsigned c0, unsigned c1, unsigned c2, unsigned c3,
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

static __device__ __forceinline__ double u01(unsigned x) { return ((double) x + 1.0) * (1.0 / 4294967296.0); }

static __device__ __forceinline__ void box_muller(unsigned ua, unsigned ub, double &g0, double &g1) {
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
static __device__ double gamdev(Stream &st, int ia) {
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

static __device__ double sum_noises(Stream &st, int nn) {
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
static __device__ void bussi_draws(Stream &st, int dof, double &sum, double &rr) {
	rr = st.gauss();
	sum = sum_noises(st, dof - 1);
}

// K <- K + (1 - c) (K_target (sum + rr^2) / dof - K) + 2 rr sqrt(K K_target / dof (1 - c) c) with
// K_target = dof T / 2 (BussiThermostat::_update_K), written with the host-side constants
// a = (1 - c) T / 2 and b = sqrt(2 T (1 - c) c), so that the device chain is short
static __device__ __forceinline__ void update_K(double &K, double one_minus_c, double a, double b, double sum, double rr) {
	K += a * (sum + rr * rr) - one_minus_c * K + b * rr * sqrt(K);
}

// Brownian ("john") thermostat: every newtonian_steps steps each nucleotide redraws its
// velocity with probability pt and its angular momentum with probability pr from the
// Maxwell-Boltzmann distribution at T (unit mass and moment of inertia).  Keyed by the
// system's seed, the step and the index within the system.
static __device__ __noinline__ void brownian_redraw(const ThermoArgs &t, int sy, int i_local, long long s, double4_32a &v,
		double4_32a &L) {
	const double *par = t.sys_par + sy * SP_STRIDE;
	const unsigned long long seed = t.sys_seed[sy];
	unsigned o0[4], o1[4];
	const unsigned k0 = (unsigned) seed, k1 = (unsigned) (seed >> 32);
	const unsigned s0 = (unsigned) s, s1 = (unsigned) ((unsigned long long) s >> 32);
	philox(k0, k1, s0, s1, RNG_BROWNIAN, (unsigned) (2 * i_local), o0);
	philox(k0, k1, s0, s1, RNG_BROWNIAN, (unsigned) (2 * i_local + 1), o1);
	double g[6];
	box_muller(o0[2], o0[3], g[0], g[1]);
	box_muller(o1[0], o1[1], g[2], g[3]);
	box_muller(o1[2], o1[3], g[4], g[5]);
	const double sT = par[SP_SQRTT];
	if(u01(o0[0]) < par[SP_PT]) v = make_double4_32a(g[0] * sT, g[1] * sT, g[2] * sT, 0.0);
	if(u01(o0[1]) < par[SP_PR]) L = make_double4_32a(g[3] * sT, g[4] * sT, g[5] * sT, 0.0);
}

// one kind of motion of brownian_redraw (which = 0: the velocity, 1: the angular momentum), with
// the same draws; returns x, redrawn or not (by value: no stack frame for the caller)
static __device__ __noinline__ double4_32a brownian_redraw_part(const ThermoArgs &t, int sy, int i_local, long long s,
		int which, double4_32a x) {
	const double *par = t.sys_par + sy * SP_STRIDE;
	const unsigned long long seed = t.sys_seed[sy];
	unsigned o0[4], o1[4];
	const unsigned k0 = (unsigned) seed, k1 = (unsigned) (seed >> 32);
	const unsigned s0 = (unsigned) s, s1 = (unsigned) ((unsigned long long) s >> 32);
	philox(k0, k1, s0, s1, RNG_BROWNIAN, (unsigned) (2 * i_local), o0);
	philox(k0, k1, s0, s1, RNG_BROWNIAN, (unsigned) (2 * i_local + 1), o1);
	const double sT = par[SP_SQRTT];
	double g0, g1, g2, g3;
	box_muller(o1[0], o1[1], g2, g3);
	if(which == 0) {
		if(u01(o0[0]) < par[SP_PT]) {
			box_muller(o0[2], o0[3], g0, g1);
			x = make_double4_32a(g0 * sT, g1 * sT, g2 * sT, 0.0);
		}
	}
	else if(u01(o0[1]) < par[SP_PR]) {
		box_muller(o1[2], o1[3], g0, g1);
		x = make_double4_32a(g3 * sT, g0 * sT, g1 * sT, 0.0);
	}
	return x;
}

// Bussi: from the sums of v, |v|^2 and |L|^2 over system sy, the new running kinetic energy
// (with the draws of this step) and the rescaling factor of one kind of motion: which = 0
// translation (about the centre-of-mass velocity), 1 rotation.  The two run on two threads.
static __device__ void bussi_update(const ThermoArgs &t, int sy, long long s, int which, const double sum[5]) {
	const double *par = t.sys_par + sy * SP_STRIDE;
	double *st = t.bussi_state + 16 * sy;
	if(which == 0) {
		const double inv_n = par[SP_INVN];
		const double n = (double) (t.sys_off[sy + 1] - t.sys_off[sy]);
		const double vc[3] = {sum[0] * inv_n, sum[1] * inv_n, sum[2] * inv_n};
		const double Kt_now = 0.5 * (sum[3] - n * (vc[0] * vc[0] + vc[1] * vc[1] + vc[2] * vc[2]));
		update_K(st[0], par[SP_1MC], par[SP_A], par[SP_B], __ldcg(st + 8), __ldcg(st + 9));
		st[2] = sqrt(st[0]) * rsqrt(Kt_now);
		st[4] = vc[0];
		st[5] = vc[1];
		st[6] = vc[2];
	}
	else {
		const double Kr_now = 0.5 * sum[4];
		update_K(st[1], par[SP_1MC], par[SP_A], par[SP_B], __ldcg(st + 10), __ldcg(st + 11));
		st[3] = sqrt(st[1]) * rsqrt(Kr_now);
	}
}

// one kind of motion of bussi_rescale (which = 0: the velocity, 1: the angular momentum)
static __device__ __forceinline__ void bussi_rescale_part(const ThermoArgs &t, int sy, int which, double4_32a &x) {
	const double *st = t.bussi_state + 16 * sy;
	if(which == 0) {
		const double ft = __ldcg(st + 2), cx = __ldcg(st + 4), cy = __ldcg(st + 5), cz = __ldcg(st + 6);
		x.x = (x.x - cx) * ft + cx;
		x.y = (x.y - cy) * ft + cy;
		x.z = (x.z - cz) * ft + cz;
	}
	else {
		const double fr = __ldcg(st + 3);
		x.x *= fr;
		x.y *= fr;
		x.z *= fr;
	}
}

// the rescaling of the last Bussi update of system sy, applied to one nucleotide
static __device__ __forceinline__ void bussi_rescale(const ThermoArgs &t, int sy, double4_32a &v, double4_32a &L) {
	const double *st = t.bussi_state + 16 * sy;
	const double ft = __ldcg(st + 2), fr = __ldcg(st + 3), cx = __ldcg(st + 4), cy = __ldcg(st + 5), cz = __ldcg(st + 6);
	v.x = (v.x - cx) * ft + cx;
	v.y = (v.y - cy) * ft + cy;
	v.z = (v.z - cz) * ft + cz;
	L.x *= fr;
	L.y *= fr;
	L.z *= fr;
}

}  // namespace oxgb
