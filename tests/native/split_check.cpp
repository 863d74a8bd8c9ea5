// Host check of the integer-pipe conversions and the FP32 error-free frame (split.cuh): the
// split and the widening are bit-identical to the C casts (round to nearest, like the device's
// cvt.rn), and the frame is within half an ulp of 1 of the exact frame, like the FP64 frame
// rounded once.  Built with g++ -ffp-contract=off by tests/test_split.py; exits non-zero on a
// failure.
#include "split.cuh"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

using namespace oxgb;

int main(int argc, char **argv) {
	const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
	std::mt19937_64 g(1);
	std::uniform_real_distribution<double> U(-1, 1);
	long bad = 0, fast = 0;
	auto check = [&](double r) {
		float h, l;
		const bool f = split_rn_int(r, h, l);
		const float h2 = (float) r, l2 = (float) (r - (double) h2);
		if(f) {
			fast++;
			if(f32_bits(h) != f32_bits(h2) || f32_bits(l) != f32_bits(l2)) bad++;
		}
		split_rn(r, h, l);
		if(f32_bits(h) != f32_bits(h2) || f32_bits(l) != f32_bits(l2)) bad++;
	};
	for(long i = 0; i < n; i++) check(U(g) * std::ldexp(1.0, (int) (g() % 200) - 90));
	for(long i = 0; i < n / 10; i++) {
		// exact ties between two floats and their neighbours
		const float f = (float) U(g) * 1000.f, f2 = f32_from_bits(f32_bits(f) + 1);
		const double mid = ((double) f + (double) f2) / 2;
		check(mid), check(std::nextafter(mid, 0.0)), check(std::nextafter(mid, 1e300)), check((double) f), check(-mid);
	}
	for(double r : {1.0, -1.0, 0.5, 1.0 - 1e-17, 3.0e38, 1e-22, 5e-23, 0.0, -0.0}) check(r);
	long ibad = 0;  // the conversion-free int -> float over its range
	for(long t = 0; t < n; t++) {
		const int x = (int) (g() % (2u << 29)) - (1 << 29) + 1;
		ibad += f32_bits(int_to_float(x)) != f32_bits((float) x);
	}
	for(int x : {0, 1, -1, 127, -128, 1 << 24, (1 << 24) + 1, (1 << 24) + 3, -(1 << 24) - 1, (1 << 29), -(1 << 29) + 1, (1 << 29) - 1})
		ibad += f32_bits(int_to_float(x)) != f32_bits((float) x);
	bad += ibad;
	long wbad = 0;
	for(long i = 0; i < n; i++) {
		const float f = f32_from_bits((unsigned) g());
		const double a = widen(f), b = (double) f;
		if(f64_bits(a) != f64_bits(b) && !(std::isnan(a) && std::isnan(b))) wbad++;
	}
	for(float f : {0.f, -0.f, 1e-40f, -1e-45f, 1.f, -3.4e38f}) wbad += f64_bits(widen(f)) != f64_bits((double) f);
	std::normal_distribution<double> N(0, 1);
	double worst = 0;
	for(long t = 0; t < n / 10; t++) {
		double q[4], nn = 0;
		for(int k = 0; k < 4; k++) q[k] = N(g), nn += q[k] * q[k];
		nn = std::sqrt(nn);
		for(int k = 0; k < 4; k++) q[k] /= nn;
		if(t % 7 == 0) q[g() % 4] *= 1e-6;
		const long double X = q[0], Y = q[1], Z = q[2], W = q[3];
		const long double E1[3] = {X * X - Y * Y - Z * Z + W * W, 2 * (X * Y + Z * W), 2 * (X * Z - Y * W)};
		const long double E2[3] = {2 * (X * Y - Z * W), -X * X + Y * Y - Z * Z + W * W, 2 * (Y * Z + X * W)};
		const long double E3[3] = {2 * (X * Z + Y * W), 2 * (Y * Z - X * W), -X * X - Y * Y + Z * Z + W * W};
		float qh[4], ql[4], a1[3], a3[3], bk[3];
		for(int k = 0; k < 4; k++) split_rn(q[k], qh[k], ql[k]);
		const float b1 = -0.34f, b2 = 0.3408f;
		frame_mirror(qh, ql, b1, b2, a1, a3, bk);
		for(int k = 0; k < 3; k++) {
			const long double eb = E1[k] * (long double) b1 + E2[k] * (long double) b2;
			for(long double d : {(long double) a1[k] - E1[k], (long double) a3[k] - E3[k], (long double) bk[k] - eb})
				worst = std::fmax(worst, (double) std::fabs(d) * std::ldexp(1.0, 24));
		}
	}
	// the small-rotation update against the rotation in extended precision, next to the FP64
	// formula it replaces
	double rot_err = 0, f64_err = 0;
	long rot_used = 0;
	const double hd = 0.0015;
	for(long t = 0; t < n / 10; t++) {
		double q[4], nn = 0;
		for(int k = 0; k < 4; k++) q[k] = N(g), nn += q[k] * q[k];
		nn = std::sqrt(nn);
		for(int k = 0; k < 4; k++) q[k] /= nn;
		const double sc = std::ldexp(1.0, (int) (g() % 6) - 2);  // |L| from about 0.25 to 8
		const double L[3] = {N(g) * sc, N(g) * sc, N(g) * sc};
		const long double L2 = (long double) L[0] * L[0] + (long double) L[1] * L[1] + (long double) L[2] * L[2];
		const long double nrm = sqrtl(L2), x = hd * nrm;
		const long double k = sinl(x) / nrm, ch = cosl(x);
		const long double r[4] = {L[0] * k, L[1] * k, L[2] * k, ch};  // x, y, z, w
		const long double X = q[0], Y = q[1], Z = q[2], Wq = q[3];
		long double e[4] = {Wq * r[0] + X * r[3] + Y * r[2] - Z * r[1], Wq * r[1] - X * r[2] + Y * r[3] + Z * r[0],
				Wq * r[2] + X * r[1] - Y * r[0] + Z * r[3], Wq * r[3] - X * r[0] - Y * r[1] - Z * r[2]};
		const long double en = sqrtl(e[0] * e[0] + e[1] * e[1] + e[2] * e[2] + e[3] * e[3]);
		for(int c = 0; c < 4; c++) e[c] /= en;
		double a[4] = {q[0], q[1], q[2], q[3]};
		if(!rotate_small(a[0], a[1], a[2], a[3], L[0], L[1], L[2], hd)) continue;
		rot_used++;
		// the FP64 formula: series for sin(x)/x and cos(x), product, Newton renormalisation
		const double L2d = L[0] * L[0] + L[1] * L[1] + L[2] * L[2], x2 = hd * hd * L2d;
		const double kk = hd * (1.0 - x2 * (1.0 / 6.0) * (1.0 - x2 * (1.0 / 20.0)));
		const double chd = 1.0 - x2 * 0.5 * (1.0 - x2 * (1.0 / 12.0) * (1.0 - x2 * (1.0 / 30.0)));
		const double rx = L[0] * kk, ry = L[1] * kk, rz = L[2] * kk;
		double b[4] = {q[3] * rx + q[0] * chd + q[1] * rz - q[2] * ry, q[3] * ry - q[0] * rz + q[1] * chd + q[2] * rx,
				q[3] * rz + q[0] * ry - q[1] * rx + q[2] * chd, q[3] * chd - q[0] * rx - q[1] * ry - q[2] * rz};
		const double dd = b[0] * b[0] + b[1] * b[1] + b[2] * b[2] + b[3] * b[3] - 1.0, inv = 1.0 - dd * (0.5 - 0.375 * dd);
		for(int c = 0; c < 4; c++) {
			rot_err = std::fmax(rot_err, (double) fabsl((long double) a[c] - e[c]));
			f64_err = std::fmax(f64_err, (double) fabsl((long double) (b[c] * inv) - e[c]));
		}
	}
	std::printf("split: %ld fast, %ld mismatches; widen: %ld mismatches; frame: max error %.4f x 2^-24; "
			"rotation (%ld): max error %.3g (FP64 formula %.3g)\n", fast, bad, wbad, worst, rot_used, rot_err, f64_err);
	return (bad || wbad || worst > 0.5001 || rot_used == 0 || rot_err > 2.0 * f64_err + 1e-16) ? 1 : 0;
}
