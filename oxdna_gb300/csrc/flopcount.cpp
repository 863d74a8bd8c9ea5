// Algorithmic work of the force kernel, counted by running the kernel's own pair physics
// (dna2_pair.cuh, FP32 instantiation) on the host with a counting scalar type.  Every add,
// subtract, multiply and divide counts one FP32 operation, an FMA two; square root, exp,
// expm1, log and acos count as one special-function operation each (reported separately).
// Used by bench.py to turn the measured force-kernel time into achieved FLOP/s.
//
// Host-only C++ (g++), built into liboxgb_tools.so.
#include <cmath>
#include <cstdint>
#include <cstring>

static double g_flops = 0, g_sfu = 0;

struct CF {
	float v;
	CF() = default;
	CF(float x) : v(x) {}
	CF(double x) : v((float) x) {}
	CF(int x) : v((float) x) {}
};
static_assert(sizeof(CF) == 4, "CF must look like a float to the kernels' precision switches");

inline CF operator+(CF a, CF b) { g_flops += 1; return CF(a.v + b.v); }
inline CF operator-(CF a, CF b) { g_flops += 1; return CF(a.v - b.v); }
inline CF operator*(CF a, CF b) { g_flops += 1; return CF(a.v * b.v); }
inline CF operator/(CF a, CF b) { g_flops += 1; return CF(a.v / b.v); }
inline CF operator-(CF a) { return CF(-a.v); }
inline CF &operator+=(CF &a, CF b) { g_flops += 1; a.v += b.v; return a; }
inline CF &operator-=(CF &a, CF b) { g_flops += 1; a.v -= b.v; return a; }
inline CF &operator*=(CF &a, CF b) { g_flops += 1; a.v *= b.v; return a; }
inline bool operator<(CF a, CF b) { return a.v < b.v; }
inline bool operator>(CF a, CF b) { return a.v > b.v; }
inline bool operator<=(CF a, CF b) { return a.v <= b.v; }
inline bool operator>=(CF a, CF b) { return a.v >= b.v; }
inline bool operator!=(CF a, CF b) { return a.v != b.v; }
inline bool operator==(CF a, CF b) { return a.v == b.v; }

namespace oxgb {
inline CF m_sqrt(CF x) { g_sfu += 1; return CF(std::sqrt(x.v)); }
inline CF m_exp(CF x) { g_sfu += 1; return CF(std::exp(x.v)); }
inline CF m_expm1(CF x) { g_sfu += 1; return CF(std::expm1(x.v)); }
inline CF m_log(CF x) { g_sfu += 1; return CF(std::log(x.v)); }
inline CF m_acos(CF x) { g_sfu += 1; return CF(std::acos(x.v)); }
inline CF m_atan2(CF y, CF x) { g_sfu += 1; return CF(std::atan2(y.v, x.v)); }
inline CF m_fabs(CF x) { return CF(std::fabs(x.v)); }
inline CF m_fma(CF a, CF b, CF c) { g_flops += 2; return CF(std::fma(a.v, b.v, c.v)); }
inline CF m_rint(CF x) { return CF(std::rint(x.v)); }
inline CF m_copysign(CF a, CF b) { return CF(std::copysign(a.v, b.v)); }
inline CF m_min(CF a, CF b) { return CF(std::fmin(a.v, b.v)); }
inline CF m_max(CF a, CF b) { return CF(std::fmax(a.v, b.v)); }
}  // namespace oxgb

#include "dna2_pair.cuh"
#include "params.h"

using namespace oxgb;

static void frame_of(const double *a1, const double *a3, int i, Nuc<CF> &n, const DNA2Table<CF> &P) {
	n.a1 = v3<CF>{CF(a1[3 * i]), CF(a1[3 * i + 1]), CF(a1[3 * i + 2])};
	n.a3 = v3<CF>{CF(a3[3 * i]), CF(a3[3 * i + 1]), CF(a3[3 * i + 2])};
	n.a2 = cross(n.a3, n.a1);
	make_sites(P, n);
}

extern "C" int oxgb_count_flops(int N, const double *pos, const double *a1, const double *a3, const int *n3, const int *n5,
		const int *type, const int *btype, double box, const int *nb, const int *nnb, int max_nb, double T, double salt,
		double skin, double *out) {
	oxgb_dna2_settings s;
	default_settings(&s, T, salt);
	DNA2Table<double> P64;
	double rcut;
	if(build_table(s, box, P64, rcut)) return 1;
	DNA2Table<float> P32;
	to_float(P64, box, P32);
	DNA2Table<CF> P;
	std::memcpy(&P, &P32, sizeof(P));
	// the algorithmic work of one force evaluation: every bond once (both nucleotides), and every
	// unordered non-bonded pair once (from its lower index), each term over the pairs its term
	// list admits (same bounds as the list build).  A pair function forms the force and the
	// torque on its first nucleotide; the partner's torque, -T_p + d x F, adds 12 FLOPs.  Work
	// the kernels repeat (Debye-Hueckel and excluded volume are evaluated from both ends of the
	// full rows) is not counted, so it shows as lost efficiency.
	const TermRadii tr = term_radii(skin);
	const double dh_bound = P64.dh_rc + 2.0 * skin + 1e-3;
	g_flops = g_sfu = 0;
	// squared distance of sites a (of p) and b (of q) of a pair with centre separation d, in
	// double and uncounted (the list build's test, not the pair's arithmetic)
	auto site_sq = [](const double *d, const v3<CF> &a, const v3<CF> &b) {
		const double x = d[0] + b.x.v - a.x.v, y = d[1] + b.y.v - a.y.v, z = d[2] + b.z.v - a.z.v;
		return x * x + y * y + z * z;
	};
	double pairs = 0, in_range = 0;
	auto load = [&](int j, Nuc<CF> &q) {
		frame_of(a1, a3, j, q, P);
		q.type = type[j];
		q.btype = btype[j];
		q.is_end = n3[j] < 0 || n5[j] < 0;
	};
	for(int i = 0; i < N; i++) {
		Nuc<CF> p;
		load(i, p);
		if(n3[i] >= 0) {
			const int j = n3[i];
			Nuc<CF> q;
			load(j, q);
			Sep<CF> sp;
			sp.hi = v3<CF>{CF(pos[3 * j] - pos[3 * i]), CF(pos[3 * j + 1] - pos[3 * i + 1]), CF(pos[3 * j + 2] - pos[3 * i + 2])};
			sp.lo = v3<CF>{CF(0.f), CF(0.f), CF(0.f)};
			BondOut<CF> b;
			bonded_both(P, p, q, sp, b);
		}
		g_flops += 9;  // the nucleotide's Debye-Hueckel torque from its summed force
		const int nn = nnb[i] < max_nb ? nnb[i] : max_nb;
		for(int k = 0; k < nn; k++) {
			const int j = nb[(long long) i * max_nb + k];
			if(j < i) continue;
			Nuc<CF> q;
			load(j, q);
			double d[3];
			for(int c = 0; c < 3; c++) {
				d[c] = pos[3 * j + c] - pos[3 * i + c];
				d[c] -= std::rint(d[c] / box) * box;
			}
			g_flops += 3 * 4;  // minimum image of the hi/lo separation
			Sep<CF> sp;
			sp.hi = v3<CF>{CF(d[0]), CF(d[1]), CF(d[2])};
			sp.lo = v3<CF>{CF(0.f), CF(0.f), CF(0.f)};
			const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
			PairOut<CF> o{};
			// Debye-Hueckel: the force of the pair; each nucleotide's torque is one cross product
			// of its backbone offset with its summed force (below)
			// each term over the pairs its list admits: Debye-Hueckel over the pairs whose backbone
			// sites are within its cutoff plus twice the skin, the excluded volume over those with a
			// site pair within that pair's cutoff plus twice the skin
			if(site_sq(d, p.back, q.back) < dh_bound * dh_bound) {
				v3<CF> fdh;
				CF edh;
				dh_sites(P, sp.plain() + q.back - p.back, p.is_end, q.is_end, fdh, edh);
			}
			if(r2 < tr.ev2) {
				const bool ev_near = site_sq(d, p.back, q.back) < tr.evs2[0] || site_sq(d, p.base, q.base) < tr.evs2[1] ||
						site_sq(d, p.back, q.base) < tr.evs2[2] || site_sq(d, p.base, q.back) < tr.evs2[2];
				if(ev_near) pair_ev<CF, false>(p, q, sp, o);
				double bb = 0, ss = 0;
				for(int c = 0; c < 3; c++) {
					const double da = a1[3 * j + c] - a1[3 * i + c];
					bb += (d[c] + 0.4 * da) * (d[c] + 0.4 * da);
					ss += (d[c] + 0.34 * da) * (d[c] + 0.34 * da);
				}
				if(bb < tr.base2) pair_base<CF, false>(P, p, q, sp, o);
				if(ss < tr.stk2) pair_stack<CF, false>(P, p, q, sp, o);
			}
			if(r2 < tr.ev2) g_flops += 12;  // the partner's torque (rigid-rotation balance)
			pairs += 1;
			if(r2 < rcut * rcut) in_range += 1;
		}
	}
	out[0] = g_flops;
	out[1] = g_sfu;
	out[2] = pairs;
	out[3] = in_range;
	return 0;
}
