// Small vector type and precision-dispatched math for the oxDNA2 kernels.  Everything is
// __host__ __device__ so that the same physics compiles for the GPU (float and double
// instantiations) and, for error studies, for the host.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define OXGB_HD __host__ __device__ __forceinline__
#else
#define OXGB_HD inline
#endif

namespace oxgb {

template <typename R>
struct v3 {
	R x, y, z;
};

template <typename R>
OXGB_HD v3<R> mk(R x, R y, R z) {
	return v3<R>{x, y, z};
}
template <typename R>
OXGB_HD v3<R> operator+(v3<R> a, v3<R> b) {
	return v3<R>{a.x + b.x, a.y + b.y, a.z + b.z};
}
template <typename R>
OXGB_HD v3<R> operator-(v3<R> a, v3<R> b) {
	return v3<R>{a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename R>
OXGB_HD v3<R> operator-(v3<R> a) {
	return v3<R>{-a.x, -a.y, -a.z};
}
template <typename R>
OXGB_HD v3<R> operator*(v3<R> a, R s) {
	return v3<R>{a.x * s, a.y * s, a.z * s};
}
template <typename R>
OXGB_HD v3<R> operator*(R s, v3<R> a) {
	return v3<R>{a.x * s, a.y * s, a.z * s};
}
template <typename R>
OXGB_HD void operator+=(v3<R> &a, v3<R> b) {
	a.x += b.x;
	a.y += b.y;
	a.z += b.z;
}
template <typename R>
OXGB_HD void operator-=(v3<R> &a, v3<R> b) {
	a.x -= b.x;
	a.y -= b.y;
	a.z -= b.z;
}
template <typename R>
OXGB_HD R dot(v3<R> a, v3<R> b) {
	return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename R>
OXGB_HD v3<R> cross(v3<R> a, v3<R> b) {
	return v3<R>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// math dispatch: the float overloads use CUDA's accurate single-precision functions (the
// force kernels are not compiled with fast-math), the double ones the double functions
OXGB_HD float m_sqrt(float x) { return sqrtf(x); }
OXGB_HD double m_sqrt(double x) { return sqrt(x); }
OXGB_HD float m_exp(float x) { return expf(x); }
OXGB_HD double m_exp(double x) { return exp(x); }
OXGB_HD float m_expm1(float x) { return expm1f(x); }
OXGB_HD double m_expm1(double x) { return expm1(x); }
OXGB_HD float m_log(float x) { return logf(x); }
OXGB_HD double m_log(double x) { return log(x); }
OXGB_HD float m_acos(float x) { return acosf(x); }
OXGB_HD double m_acos(double x) { return acos(x); }
OXGB_HD float m_atan2(float y, float x) { return atan2f(y, x); }
OXGB_HD double m_atan2(double y, double x) { return atan2(y, x); }
OXGB_HD float m_fabs(float x) { return fabsf(x); }
OXGB_HD double m_fabs(double x) { return fabs(x); }
OXGB_HD float m_fma(float a, float b, float c) { return fmaf(a, b, c); }
OXGB_HD double m_fma(double a, double b, double c) { return fma(a, b, c); }
OXGB_HD float m_rint(float x) { return rintf(x); }
OXGB_HD double m_rint(double x) { return rint(x); }
OXGB_HD float m_copysign(float a, float b) { return copysignf(a, b); }
OXGB_HD double m_copysign(double a, double b) { return copysign(a, b); }
OXGB_HD float m_min(float a, float b) { return fminf(a, b); }
OXGB_HD double m_min(double a, double b) { return fmin(a, b); }
OXGB_HD float m_max(float a, float b) { return fmaxf(a, b); }
OXGB_HD double m_max(double a, double b) { return fmax(a, b); }

// lab-frame axes of a unit quaternion (x, y, z, w): a1, a2, a3 are the columns of its
// rotation matrix (the convention of the reference's device code)
template <typename R>
OXGB_HD void quat_frame(R x, R y, R z, R w, v3<R> &a1, v3<R> &a2, v3<R> &a3) {
	const R xx = x * x, yy = y * y, zz = z * z, ww = w * w;
	const R xy = x * y, xz = x * z, xw = x * w, yz = y * z, yw = y * w, zw = z * w;
	a1 = v3<R>{xx - yy - zz + ww, R(2) * (xy + zw), R(2) * (xz - yw)};
	a2 = v3<R>{R(2) * (xy - zw), -xx + yy - zz + ww, R(2) * (yz + xw)};
	a3 = v3<R>{R(2) * (xz + yw), R(2) * (yz - xw), -xx - yy + zz + ww};
}

}  // namespace oxgb
