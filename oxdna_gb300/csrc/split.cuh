// Conversions between FP64 and FP32 done with integer operations.
//
// GB300 runs FP64 arithmetic and f64<->f32 conversions at about 1.8 operations per clock per
// SM (measured), against 128 FP32 or integer operations, and the first integration step is bound
// by that pipe.  The conversions it needs are exact functions of the bit patterns, so they are
// written here with integer operations, bit-identical to the hardware conversions inside the
// stated ranges (checked on the host against C casts, which round to nearest like cvt.rn):
//   split_rn:  r -> hi = (float) r, lo = (float) (r - (double) hi)
//   widen:     f -> (double) f
// Outside the ranges (zeros, denormals, huge values) they fall back to the FP64 conversions.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "oxgb_vec.cuh"

namespace oxgb {

// Products and sums that must not be contracted into FMAs (the error terms depend on their
// rounding): the _rn intrinsics on the device; host builds use -ffp-contract=off.
#ifdef __CUDA_ARCH__
#define OXGB_FMUL(a, b) __fmul_rn(a, b)
#define OXGB_FADD(a, b) __fadd_rn(a, b)
#define OXGB_FSUB(a, b) __fsub_rn(a, b)
#define OXGB_FMAF(a, b, c) __fmaf_rn(a, b, c)
#else
#define OXGB_FMUL(a, b) ((a) * (b))
#define OXGB_FADD(a, b) ((a) + (b))
#define OXGB_FSUB(a, b) ((a) - (b))
#define OXGB_FMAF(a, b, c) std::fma(a, b, c)
#endif

OXGB_HD unsigned long long f64_bits(double x) {
#ifdef __CUDA_ARCH__
	return (unsigned long long) __double_as_longlong(x);
#else
	unsigned long long u;
	std::memcpy(&u, &x, sizeof u);
	return u;
#endif
}

OXGB_HD double f64_from_bits(unsigned long long u) {
#ifdef __CUDA_ARCH__
	return __longlong_as_double((long long) u);
#else
	double x;
	std::memcpy(&x, &u, sizeof x);
	return x;
#endif
}

OXGB_HD unsigned f32_bits(float x) {
#ifdef __CUDA_ARCH__
	return __float_as_uint(x);
#else
	unsigned u;
	std::memcpy(&u, &x, sizeof u);
	return u;
#endif
}

OXGB_HD float f32_from_bits(unsigned u) {
#ifdef __CUDA_ARCH__
	return __uint_as_float(u);
#else
	float x;
	std::memcpy(&x, &u, sizeof x);
	return x;
#endif
}

// (float) x rounded to nearest for |x| < 2^29 without a conversion instruction (which runs on
// the slow FP64/conversion pipe): x = 128 q + m with q = x >> 7 (|q| < 2^22) and m = x & 127,
// each made exactly from the bits of 1.5 * 2^23 + q (or 2^23 + m) less that constant, then one
// FMA rounds 128 q + m once
OXGB_HD float int_to_float(int x) {
	const int q = x >> 7, m = x & 127;
	const float fq = OXGB_FSUB(f32_from_bits(0x4B400000u + (unsigned) q), 12582912.f);
	const float fm = OXGB_FSUB(f32_from_bits(0x4B000000u | (unsigned) m), 8388608.f);
	return OXGB_FMAF(fq, 128.f, fm);
}

// hi = r rounded to the nearest float (ties to even), lo = the exact remainder r - hi rounded
// to the nearest float; both are exact in the FP32 normal range: 2^-74 <= |r| < 2^127
// (biased FP64 exponent 949 .. 1149).  Returns false outside it.
OXGB_HD bool split_rn_int(double r, float &hi, float &lo) {
	const unsigned long long b = f64_bits(r);
	const int e = (int) ((b >> 52) & 0x7ffu);
	if(e < 949 || e > 1149) return false;
	const unsigned sign = (unsigned) (b >> 63);
	const unsigned long long mag = b & 0x7fffffffffffffffull;
	// the 29 mantissa bits a float drops, and round to nearest even on them
	const unsigned low = (unsigned) (mag & 0x1fffffffull);
	const bool up = low > 0x10000000u || (low == 0x10000000u && ((mag >> 29) & 1u));
	// exponent and top 23 mantissa bits, rebiased from 1023 to 127 (a carry of the rounding into
	// the exponent is the correctly rounded result)
	const unsigned hbits = (unsigned) ((mag >> 29) + (up ? 1u : 0u) - (896ull << 23));
	hi = f32_from_bits((sign << 31) | hbits);
	// r - hi = (low - 2^29 [if rounded up]) units of 2^(e - 1075), with the sign of r, rounded to
	// the nearest float (int_to_float) and scaled by the exact power of two
	const int li = (int) low - (up ? (1 << 29) : 0);
	const float scale = f32_from_bits((unsigned) (e - 1075 + 127) << 23);
	lo = int_to_float(sign ? -li : li) * scale;  // an exact remainder is +0, as r - hi gives
	return true;
}

// The out-of-range cases on the conversion instructions, in a function of its own: inlined, the
// compiler would compute them on every call and select (they run on the slow FP64 pipe).
#ifdef __CUDA_ARCH__
#define OXGB_COLD __device__ __noinline__
#else
#define OXGB_COLD inline
#endif

struct HiLo {
	float hi, lo;
};

OXGB_COLD HiLo split_rn_cold(double r) {
	const float hi = (float) r;
	return HiLo{hi, (float) (r - (double) hi)};
}

OXGB_COLD double widen_cold(float f) { return (double) f; }

OXGB_HD void split_rn(double r, float &hi, float &lo) {
	if(!split_rn_int(r, hi, lo)) {
		const HiLo c = split_rn_cold(r);
		hi = c.hi;
		lo = c.lo;
	}
}

// (float) r: the high part of split_rn
OXGB_HD float narrow(double r) {
	float hi, lo;
	split_rn(r, hi, lo);
	return hi;
}

// (double) f for normal floats and zeros (exact); denormals, infinities and NaNs take the
// conversion instruction
OXGB_HD double widen(double f) { return f; }

OXGB_HD double widen(float f) {
	const unsigned u = f32_bits(f);
	const unsigned e = (u >> 23) & 0xffu;
	if(e == 0u || e == 0xffu) {
		if((u & 0x7fffffffu) == 0u) return f64_from_bits((unsigned long long) (u >> 31) << 63);
		return widen_cold(f);
	}
	const unsigned long long d = ((unsigned long long) (u >> 31) << 63) | ((unsigned long long) (e + 896u) << 52) |
			((unsigned long long) (u & 0x7fffffu) << 29);
	return f64_from_bits(d);
}

// ---------------------------------------------------------------- FP32 error-free arithmetic



// a float pair s + e
struct F2 {
	float s, e;
};

// a + b = s + e exactly (TwoSum, no ordering condition)
OXGB_HD F2 two_sum(float a, float b) {
	const float s = OXGB_FADD(a, b);
	const float bp = OXGB_FSUB(s, a);
	return F2{s, OXGB_FADD(OXGB_FSUB(a, OXGB_FSUB(s, bp)), OXGB_FSUB(b, bp))};
}

// (ah + al)(bh + bl) as a pair, to a relative 2^-46 (the al bl term is dropped)
OXGB_HD F2 prod2(float ah, float al, float bh, float bl) {
	const float p = OXGB_FMUL(ah, bh);
	return F2{p, OXGB_FMAF(ah, bl, OXGB_FMAF(al, bh, OXGB_FMAF(ah, bh, -p)))};
}

// (a + b) - (c + d) of four pairs, as a pair
OXGB_HD F2 diff_of_sums2(F2 a, F2 b, F2 c, F2 d) {
	const F2 u = two_sum(a.s, b.s), v = two_sum(c.s, d.s), w = two_sum(u.s, -v.s);
	return F2{w.s, OXGB_FADD(OXGB_FADD(OXGB_FSUB(u.e, v.e), w.e), OXGB_FSUB(OXGB_FADD(a.e, b.e), OXGB_FADD(c.e, d.e)))};
}

// 2 (a +/- b) of two pairs, as a pair
OXGB_HD F2 twice_sum2(F2 a, F2 b, float sign) {
	const F2 u = two_sum(a.s, sign * b.s);
	const float e = OXGB_FADD(u.e, OXGB_FADD(a.e, sign * b.e));
	return F2{2.f * u.s, 2.f * e};
}

OXGB_HD float round2(F2 a) { return OXGB_FADD(a.s, a.e); }

// b1 x + b2 y of two pairs with float constants, as a pair (round2 rounds it)
OXGB_HD F2 lin2_pair(float b1, F2 x, float b2, F2 y) {
	const float u = OXGB_FMUL(b1, x.s), eu = OXGB_FMAF(b1, x.s, -u);
	const float v = OXGB_FMUL(b2, y.s), ev = OXGB_FMAF(b2, y.s, -v);
	const F2 w = two_sum(u, v);
	const float e = OXGB_FADD(OXGB_FADD(w.e, OXGB_FADD(eu, ev)), OXGB_FMAF(b1, x.e, OXGB_FMUL(b2, y.e)));
	return F2{w.s, e};
}

// the remainder of a pair's FP32 rounding r = round2(a): a - r (a.s - r is exact, the two being
// a few ulps apart)
OXGB_HD float rem2(F2 a, float r) { return OXGB_FADD(OXGB_FSUB(a.s, r), a.e); }

// The body axes a1, a2, a3 of the unit quaternion (x, y, z, w) = (qh + ql) given as FP32 pairs
// (split_rn), as pairs accurate to ~2^-46.  The frame is that of quat_frame.
OXGB_HD void frame_pairs(const float qh[4], const float ql[4], F2 a1[3], F2 a2[3], F2 a3[3]) {
	const F2 xx = prod2(qh[0], ql[0], qh[0], ql[0]), yy = prod2(qh[1], ql[1], qh[1], ql[1]),
			 zz = prod2(qh[2], ql[2], qh[2], ql[2]), ww = prod2(qh[3], ql[3], qh[3], ql[3]);
	const F2 xy = prod2(qh[0], ql[0], qh[1], ql[1]), xz = prod2(qh[0], ql[0], qh[2], ql[2]),
			 xw = prod2(qh[0], ql[0], qh[3], ql[3]), yz = prod2(qh[1], ql[1], qh[2], ql[2]),
			 yw = prod2(qh[1], ql[1], qh[3], ql[3]), zw = prod2(qh[2], ql[2], qh[3], ql[3]);
	a1[0] = diff_of_sums2(xx, ww, yy, zz), a1[1] = twice_sum2(xy, zw, 1.f), a1[2] = twice_sum2(xz, yw, -1.f);
	a2[0] = twice_sum2(xy, zw, -1.f), a2[1] = diff_of_sums2(yy, ww, xx, zz), a2[2] = twice_sum2(yz, xw, 1.f);
	a3[0] = twice_sum2(xz, yw, 1.f), a3[1] = twice_sum2(yz, xw, -1.f), a3[2] = diff_of_sums2(zz, ww, xx, yy);
}

// The body axes a1, a3 and the backbone offset b1 a1 + b2 a2 of the unit quaternion
// (x, y, z, w) = (qh + ql) given as FP32 pairs (split_rn), each rounded to FP32 from a pair
// accurate to ~2^-46: the same values (to within an ulp, nearly always equal) as the FP64
// frame rounded once, computed on the FP32 pipe.
OXGB_HD void frame_mirror(const float qh[4], const float ql[4], float b1, float b2, float a1[3], float a3[3], float back[3]) {
	F2 p1[3], p2[3], p3[3];
	frame_pairs(qh, ql, p1, p2, p3);
#pragma unroll
	for(int k = 0; k < 3; k++) {
		a1[k] = round2(p1[k]);
		a3[k] = round2(p3[k]);
		back[k] = round2(lin2_pair(b1, p1[k], b2, p2[k]));
	}
}

// The remainders of frame_mirror's a1 and backbone offset: a1 = a1_mirror + a1lo and back =
// back_mirror + backlo to ~2^-46 (the mirrors are recomputed here, bit-identical)
OXGB_HD void frame_remainders(const float qh[4], const float ql[4], float b1, float b2, float a1lo[3], float backlo[3]) {
	F2 p1[3], p2[3], p3[3];
	frame_pairs(qh, ql, p1, p2, p3);
#pragma unroll
	for(int k = 0; k < 3; k++) {
		a1lo[k] = rem2(p1[k], round2(p1[k]));
		const F2 bk = lin2_pair(b1, p1[k], b2, p2[k]);
		backlo[k] = rem2(bk, round2(bk));
	}
}

// frame_mirror and frame_remainders from one evaluation of the pairs
OXGB_HD void frame_mirror_rem(const float qh[4], const float ql[4], float b1, float b2, float a1[3], float a3[3], float back[3],
		float a1lo[3], float backlo[3]) {
	F2 p1[3], p2[3], p3[3];
	frame_pairs(qh, ql, p1, p2, p3);
#pragma unroll
	for(int k = 0; k < 3; k++) {
		a1[k] = round2(p1[k]);
		a3[k] = round2(p3[k]);
		const F2 bk = lin2_pair(b1, p1[k], b2, p2[k]);
		back[k] = round2(bk);
		a1lo[k] = rem2(p1[k], a1[k]);
		backlo[k] = rem2(bk, back[k]);
	}
}

// ---------------------------------------------------------------- pairs as ~48-bit numbers

// a + b of two pairs, renormalised (|e| <= ulp(s) / 2)
OXGB_HD F2 add2(F2 a, F2 b) {
	const F2 t = two_sum(a.s, b.s);
	const float e = OXGB_FADD(t.e, OXGB_FADD(a.e, b.e));
	const float s = OXGB_FADD(t.s, e);
	return F2{s, OXGB_FSUB(e, OXGB_FSUB(s, t.s))};
}

// a b of two pairs, renormalised
OXGB_HD F2 mul2(F2 a, F2 b) {
	const F2 p = prod2(a.s, a.e, b.s, b.e);
	const float s = OXGB_FADD(p.s, p.e);
	return F2{s, OXGB_FSUB(p.e, OXGB_FSUB(s, p.s))};
}

OXGB_HD F2 neg2(F2 a) { return F2{-a.s, -a.e}; }

OXGB_HD F2 split2(double x) {
	F2 r;
	split_rn(x, r.s, r.e);
	return r;
}

// The rotation of the unit quaternion q = (x, y, z, w) by the angle dt |L| about the body-frame
// angular momentum L (hd = dt / 2): q <- q (x) (sin(t/2) L^, cos(t/2)), t = dt |L|, written
// as q + c with the small correction c = q (x) (delta, eps), delta = k L, eps = cos(t/2) - 1,
// k = sin(t/2) / |L|, computed in FP32 pairs (~48 bits: |c| ~ hd |L|, so its absolute error is
// below 1e-17, under an ulp of q's FP64 components); only the final additions are FP64.  The
// norm error of q entering the step is removed with it (q (1 - d / 2), d = |q|^2 - 1), so q
// stays unit to rounding.  Returns false, leaving q alone, outside the range where this holds
// (x^2 = (hd |L|)^2 >= 1e-5, or |d| >= 1e-6): the caller then rotates in FP64.
OXGB_HD bool rotate_small(double &qx, double &qy, double &qz, double &qw, double Lx, double Ly, double Lz, double hd) {
	const double d = fma(qx, qx, fma(qy, qy, fma(qz, qz, fma(qw, qw, -1.0))));
	if(!(fabs(d) < 1e-6)) return false;
	const F2 lx = split2(Lx), ly = split2(Ly), lz = split2(Lz), h = split2(hd);
	const F2 x2 = mul2(mul2(h, h), add2(add2(mul2(lx, lx), mul2(ly, ly)), mul2(lz, lz)));
	if(!(x2.s < 1e-5f)) return false;
	// sin(x) / x = 1 - x^2 / 6 + x^4 / 120 - ..., cos(x) - 1 = -x^2 / 2 + x^4 / 24 - ...; the
	// omitted terms are below 1e-20 for x^2 < 1e-5, the x^4 terms need only FP32
	const F2 sixth = split2(1.0 / 6.0);
	const float x4 = OXGB_FMUL(x2.s, x2.s);
	const F2 sinc = add2(F2{1.f, 0.f}, add2(neg2(mul2(x2, sixth)), F2{OXGB_FMUL(x4, 1.f / 120.f), 0.f}));
	const F2 eps = add2(F2{-0.5f * x2.s, -0.5f * x2.e}, F2{OXGB_FMUL(x4, 1.f / 24.f), 0.f});
	const F2 k = mul2(h, sinc);
	const F2 dx = mul2(k, lx), dy = mul2(k, ly), dz = mul2(k, lz);
	const F2 ax = split2(qx), ay = split2(qy), az = split2(qz), aw = split2(qw);
	const F2 cw = add2(add2(mul2(aw, eps), neg2(mul2(ax, dx))), add2(neg2(mul2(ay, dy)), neg2(mul2(az, dz))));
	const F2 cx = add2(add2(mul2(aw, dx), mul2(ax, eps)), add2(mul2(ay, dz), neg2(mul2(az, dy))));
	const F2 cy = add2(add2(mul2(aw, dy), neg2(mul2(ax, dz))), add2(mul2(ay, eps), mul2(az, dx)));
	const F2 cz = add2(add2(mul2(aw, dz), mul2(ax, dy)), add2(neg2(mul2(ay, dx)), mul2(az, eps)));
	const double hs = -0.5 * d;
	qx = (fma(qx, hs, qx) + widen(cx.s)) + widen(cx.e);
	qy = (fma(qy, hs, qy) + widen(cy.s)) + widen(cy.e);
	qz = (fma(qz, hs, qz) + widen(cz.s)) + widen(cz.e);
	qw = (fma(qw, hs, qw) + widen(cw.s)) + widen(cw.e);
	return true;
}

}  // namespace oxgb
