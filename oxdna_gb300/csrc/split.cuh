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
	// r - hi = (low - 2^29 [if rounded up]) units of 2^(e - 1075), with the sign of r; the
	// integer-to-float conversion rounds to nearest and the power-of-two scale is exact
	const int li = (int) low - (up ? (1 << 29) : 0);
	const float scale = f32_from_bits((unsigned) (e - 1075 + 127) << 23);
	lo = (float) (sign ? -li : li) * scale;  // an exact remainder is +0, as r - hi gives
	return true;
}

OXGB_HD void split_rn(double r, float &hi, float &lo) {
	if(!split_rn_int(r, hi, lo)) {
		hi = (float) r;
		lo = (float) (r - (double) hi);
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
		return (double) f;
	}
	const unsigned long long d = ((unsigned long long) (u >> 31) << 63) | ((unsigned long long) (e + 896u) << 52) |
			((unsigned long long) (u & 0x7fffffu) << 29);
	return f64_from_bits(d);
}

// ---------------------------------------------------------------- FP32 error-free arithmetic

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

// b1 x + b2 y of two pairs with float constants, rounded
OXGB_HD float lin2(float b1, F2 x, float b2, F2 y) {
	const float u = OXGB_FMUL(b1, x.s), eu = OXGB_FMAF(b1, x.s, -u);
	const float v = OXGB_FMUL(b2, y.s), ev = OXGB_FMAF(b2, y.s, -v);
	const F2 w = two_sum(u, v);
	const float e = OXGB_FADD(OXGB_FADD(w.e, OXGB_FADD(eu, ev)), OXGB_FMAF(b1, x.e, OXGB_FMUL(b2, y.e)));
	return OXGB_FADD(w.s, e);
}

// The body axes a1, a3 and the backbone offset b1 a1 + b2 a2 of the unit quaternion
// (x, y, z, w) = (qh + ql) given as FP32 pairs (split_rn), each rounded to FP32 from a pair
// accurate to ~2^-46: the same values (to within an ulp, nearly always equal) as the FP64
// frame rounded once, computed on the FP32 pipe.  The frame is that of quat_frame.
OXGB_HD void frame_mirror(const float qh[4], const float ql[4], float b1, float b2, float a1[3], float a3[3], float back[3]) {
	const F2 xx = prod2(qh[0], ql[0], qh[0], ql[0]), yy = prod2(qh[1], ql[1], qh[1], ql[1]),
			 zz = prod2(qh[2], ql[2], qh[2], ql[2]), ww = prod2(qh[3], ql[3], qh[3], ql[3]);
	const F2 xy = prod2(qh[0], ql[0], qh[1], ql[1]), xz = prod2(qh[0], ql[0], qh[2], ql[2]),
			 xw = prod2(qh[0], ql[0], qh[3], ql[3]), yz = prod2(qh[1], ql[1], qh[2], ql[2]),
			 yw = prod2(qh[1], ql[1], qh[3], ql[3]), zw = prod2(qh[2], ql[2], qh[3], ql[3]);
	const F2 a1x = diff_of_sums2(xx, ww, yy, zz), a1y = twice_sum2(xy, zw, 1.f), a1z = twice_sum2(xz, yw, -1.f);
	const F2 a2x = twice_sum2(xy, zw, -1.f), a2y = diff_of_sums2(yy, ww, xx, zz), a2z = twice_sum2(yz, xw, 1.f);
	const F2 a3x = twice_sum2(xz, yw, 1.f), a3y = twice_sum2(yz, xw, -1.f), a3z = diff_of_sums2(zz, ww, xx, yy);
	a1[0] = round2(a1x), a1[1] = round2(a1y), a1[2] = round2(a1z);
	a3[0] = round2(a3x), a3[1] = round2(a3y), a3[2] = round2(a3z);
	back[0] = lin2(b1, a1x, b2, a2x);
	back[1] = lin2(b1, a1y, b2, a2y);
	back[2] = lin2(b1, a1z, b2, a2z);
}

}  // namespace oxgb
