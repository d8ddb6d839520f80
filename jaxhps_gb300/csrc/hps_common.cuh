// Common device-side helpers for the HPS GB300 kernels.
//
// Scalar arithmetic is written once over four element types (f64, f32,
// complex128, complex64) through small overloads, so the batched linear
// algebra (GEMM, Gauss-Jordan inverse) and the HPS gather/scatter kernels
// are templated on the element type.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hps {

struct c64 {
  float x, y;
};
struct c128 {
  double x, y;
};

// ---- construction ---------------------------------------------------------
template <class T> __host__ __device__ inline T make_scalar(double re, double im);
template <> __host__ __device__ inline float make_scalar<float>(double re, double) { return (float)re; }
template <> __host__ __device__ inline double make_scalar<double>(double re, double) { return re; }
template <> __host__ __device__ inline c64 make_scalar<c64>(double re, double im) { return c64{(float)re, (float)im}; }
template <> __host__ __device__ inline c128 make_scalar<c128>(double re, double im) { return c128{re, im}; }

template <class T> __host__ __device__ inline T zero() { return make_scalar<T>(0.0, 0.0); }
template <class T> __host__ __device__ inline T one() { return make_scalar<T>(1.0, 0.0); }

// ---- arithmetic -----------------------------------------------------------
__device__ __forceinline__ float add(float a, float b) { return a + b; }
__device__ __forceinline__ double add(double a, double b) { return a + b; }
__device__ __forceinline__ c64 add(c64 a, c64 b) { return c64{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ c128 add(c128 a, c128 b) { return c128{a.x + b.x, a.y + b.y}; }

__device__ __forceinline__ float sub(float a, float b) { return a - b; }
__device__ __forceinline__ double sub(double a, double b) { return a - b; }
__device__ __forceinline__ c64 sub(c64 a, c64 b) { return c64{a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ c128 sub(c128 a, c128 b) { return c128{a.x - b.x, a.y - b.y}; }

__device__ __forceinline__ float mul(float a, float b) { return a * b; }
__device__ __forceinline__ double mul(double a, double b) { return a * b; }
__device__ __forceinline__ c64 mul(c64 a, c64 b) {
  return c64{fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x)};
}
__device__ __forceinline__ c128 mul(c128 a, c128 b) {
  return c128{fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x)};
}

__device__ __forceinline__ float neg(float a) { return -a; }
__device__ __forceinline__ double neg(double a) { return -a; }
__device__ __forceinline__ c64 neg(c64 a) { return c64{-a.x, -a.y}; }
__device__ __forceinline__ c128 neg(c128 a) { return c128{-a.x, -a.y}; }

// acc + a*b
__device__ __forceinline__ float fma_(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ c64 fma_(c64 a, c64 b, c64 c) {
  c.x = fmaf(a.x, b.x, c.x);
  c.x = fmaf(-a.y, b.y, c.x);
  c.y = fmaf(a.x, b.y, c.y);
  c.y = fmaf(a.y, b.x, c.y);
  return c;
}
__device__ __forceinline__ c128 fma_(c128 a, c128 b, c128 c) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
  return c;
}
// acc - a*b
__device__ __forceinline__ float fms_(float a, float b, float c) { return fmaf(-a, b, c); }
__device__ __forceinline__ double fms_(double a, double b, double c) { return fma(-a, b, c); }
__device__ __forceinline__ c64 fms_(c64 a, c64 b, c64 c) { return fma_(neg(a), b, c); }
__device__ __forceinline__ c128 fms_(c128 a, c128 b, c128 c) { return fma_(neg(a), b, c); }

// 1/a  (IEEE division; complex via conj(a)/|a|^2 with scaling)
__device__ __forceinline__ float rcp_(float a) { return 1.0f / a; }
__device__ __forceinline__ double rcp_(double a) { return 1.0 / a; }
__device__ __forceinline__ c64 rcp_(c64 a) {
  float s = fmaxf(fabsf(a.x), fabsf(a.y));
  float ar = a.x / s, ai = a.y / s;
  float d = (ar * ar + ai * ai) * s;
  return c64{ar / d, -ai / d};
}
__device__ __forceinline__ c128 rcp_(c128 a) {
  double s = fmax(fabs(a.x), fabs(a.y));
  double ar = a.x / s, ai = a.y / s;
  double d = (ar * ar + ai * ai) * s;
  return c128{ar / d, -ai / d};
}

// Pivot magnitude: |a| for reals, |re|+|im| for complex (the LAPACK
// cabs1 convention used by i?amax), computed in the element's own real
// precision (FP64 arithmetic is a small fraction of FP32 throughput on
// GB300, so single-precision kernels never touch it).
template <class T> struct MagOf;
template <> struct MagOf<float> { using type = float; };
template <> struct MagOf<c64> { using type = float; };
template <> struct MagOf<double> { using type = double; };
template <> struct MagOf<c128> { using type = double; };

__device__ __forceinline__ float pivmag(float a) { return fabsf(a); }
__device__ __forceinline__ double pivmag(double a) { return fabs(a); }
__device__ __forceinline__ float pivmag(c64 a) { return fabsf(a.x) + fabsf(a.y); }
__device__ __forceinline__ double pivmag(c128 a) { return fabs(a.x) + fabs(a.y); }

// NaN magnitudes are promoted to +inf so that a NaN pivot column is picked
// (and propagates) instead of leaving no candidate.
__device__ __forceinline__ float nan_to_inf(float m) { return (m != m) ? __int_as_float(0x7f800000) : m; }
__device__ __forceinline__ double nan_to_inf(double m) {
  return (m != m) ? __longlong_as_double(0x7ff0000000000000LL) : m;
}

// Conversions from the FP64 host-precision inputs.
template <class T> __device__ __forceinline__ T from_real(double v);
template <> __device__ __forceinline__ float from_real<float>(double v) { return (float)v; }
template <> __device__ __forceinline__ double from_real<double>(double v) { return v; }
template <> __device__ __forceinline__ c64 from_real<c64>(double v) { return c64{(float)v, 0.f}; }
template <> __device__ __forceinline__ c128 from_real<c128>(double v) { return c128{v, 0.0}; }

template <class T> __device__ __forceinline__ T from_c128(c128 v);
template <> __device__ __forceinline__ float from_c128<float>(c128 v) { return (float)v.x; }
template <> __device__ __forceinline__ double from_c128<double>(c128 v) { return v.x; }
template <> __device__ __forceinline__ c64 from_c128<c64>(c128 v) { return c64{(float)v.x, (float)v.y}; }
template <> __device__ __forceinline__ c128 from_c128<c128>(c128 v) { return v; }

// Element-type tags shared with the C ABI (see include/jaxhps_gb300.h).
enum DType : int { F64 = 0, F32 = 1, C128 = 2, C64 = 3 };

template <class T> struct DTypeOf;
template <> struct DTypeOf<double> { static constexpr int value = F64; };
template <> struct DTypeOf<float> { static constexpr int value = F32; };
template <> struct DTypeOf<c128> { static constexpr int value = C128; };
template <> struct DTypeOf<c64> { static constexpr int value = C64; };

inline size_t dtype_size(int dt) {
  switch (dt) {
    case F64: return 8;
    case F32: return 4;
    case C128: return 16;
    case C64: return 8;
    default: return 0;
  }
}

}  // namespace hps
