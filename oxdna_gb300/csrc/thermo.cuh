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

// Bussi state of system sy, 16 doubles: K_t and K_r in two slots each ([0 + u], [2 + u]) and
// the draws of a step in two slots ([8 + 4u] .. [11 + 4u]: sum_t, rr_t, sum_r, rr_r), where
// u = (step / newtonian_steps) & 1 is the parity of the update; the update at step s reads
// the slot of the previous update and writes its own, and the draws of the next step go to
// the other slot, so no kernel reads what another running kernel writes.
__device__ __forceinline__ int bussi_slot(const ThermoArgs &t, long long s) { return (int) ((s / t.newtonian_steps) & 1); }

struct BussiFactors {
	double ft, fr, cx, cy, cz;
};

// The rescaling of system sy decided by the Bussi update of step s, computed by a whole warp
// (every lane gets it): the chunk sums of the system (k_bussi_sums) in a fixed order, the new
// running kinetic energies from the draws of step s, and the factors.  The warp holding the
// system's first nucleotide (write = true) stores the new kinetic energies.
__device__ __noinline__ BussiFactors bussi_factors(const ThermoArgs &t, int sy, long long s, bool write) {
	const int lane = threadIdx.x & 31;
	const int c0 = t.sys_chunk0[sy], nc = t.sys_chunk0[sy + 1] - c0;
	double part[5] = {0, 0, 0, 0, 0};
	for(int b = lane; b < nc; b += 32)
#pragma unroll
		for(int k = 0; k < 5; k++) part[k] += t.bussi_partials[(c0 + b) * 8 + k];
#pragma unroll
	for(int k = 0; k < 5; k++)
		for(int off = 16; off > 0; off >>= 1) part[k] += __shfl_xor_sync(0xffffffffu, part[k], off);
	const double *par = t.sys_par + sy * SP_STRIDE;
	double *st = t.bussi_state + 16 * sy;
	const int u = bussi_slot(t, s);
	const double *dr = st + 8 + 4 * u;
	const double inv_n = par[SP_INVN];
	const double n = (double) (t.sys_off[sy + 1] - t.sys_off[sy]);
	BussiFactors f;
	f.cx = part[0] * inv_n;
	f.cy = part[1] * inv_n;
	f.cz = part[2] * inv_n;
	const double Kt_now = 0.5 * (part[3] - n * (f.cx * f.cx + f.cy * f.cy + f.cz * f.cz));
	const double Kr_now = 0.5 * part[4];
	double Kt = st[1 - u], Kr = st[3 - u];
	update_K(Kt, par[SP_1MC], par[SP_A], par[SP_B], dr[0], dr[1]);
	update_K(Kr, par[SP_1MC], par[SP_A], par[SP_B], dr[2], dr[3]);
	f.ft = sqrt(Kt) * rsqrt(Kt_now);
	f.fr = sqrt(Kr) * rsqrt(Kr_now);
	if(write && lane == 0) {
		st[u] = Kt;
		st[2 + u] = Kr;
	}
	return f;
}

__device__ __forceinline__ void bussi_rescale(const BussiFactors &f, double4_32a &v, double4_32a &L) {
	v.x = (v.x - f.cx) * f.ft + f.cx;
	v.y = (v.y - f.cy) * f.ft + f.cy;
	v.z = (v.z - f.cz) * f.ft + f.cz;
	L.x *= f.fr;
	L.y *= f.fr;
	L.z *= f.fr;
}

// the factors for the system of this lane's nucleotide, for a warp whose nucleotides may
// belong to several systems (the distinct systems in turn, warp-uniform); lanes past the last
// nucleotide pass sy = -1
__device__ __forceinline__ BussiFactors bussi_factors_warp(const ThermoArgs &t, int sy, int i, long long s) {
	BussiFactors mine{1.0, 1.0, 0.0, 0.0, 0.0};
	unsigned todo = __ballot_sync(0xffffffffu, sy >= 0);
	while(todo) {
		const int leader = __ffs(todo) - 1;
		const int cur = __shfl_sync(0xffffffffu, sy, leader);
		const bool first = __any_sync(0xffffffffu, sy == cur && i == t.sys_off[cur]);
		const BussiFactors f = bussi_factors(t, cur, s, first);
		if(sy == cur) mine = f;
		todo &= ~__ballot_sync(0xffffffffu, sy == cur);
	}
	return mine;
}

}  // namespace oxgb
