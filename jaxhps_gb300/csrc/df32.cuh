// Double-float ("df32") arithmetic: a value held as an unevaluated pair of
// FP32 numbers hi + lo (~48-bit significand), with products and sums formed
// by the error-free transformations TwoProd (one FMA) and TwoSum (Knuth), so
// that refinement residuals run on the FP32 pipe instead of GB300's FP64
// pipe (1/64 of the FP32 rate).  Used by the residual-update kernels.
#pragma once

#include <cuda_runtime.h>

namespace hps {

struct df32 {
  float hi, lo;
};

__device__ __forceinline__ df32 df_split(double x) {
  const float h = __double2float_rn(x);
  return df32{h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ double df_join(float s, float e) { return (double)s + (double)e; }

// (s, e) with |e| <= |s| ulp-wise; FastTwoSum on the FP32 pipe
__device__ __forceinline__ df32 df_norm(float s, float e) {
  const float h = s + e;
  return df32{h, e - (h - s)};
}

// a * b for pairs, renormalised (FP32 pipe only)
__device__ __forceinline__ df32 df_mul(df32 a, df32 b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_norm(p, e);
}

// (s, e) += a * b ; s carries the running sum, e the low-order terms
__device__ __forceinline__ void df_mac(float& s, float& e, df32 a, df32 b) {
  const float p = a.hi * b.hi;
  float pe = fmaf(a.hi, b.hi, -p);
  pe = fmaf(a.hi, b.lo, pe);
  pe = fmaf(a.lo, b.hi, pe);
  const float t = s + p;
  const float bb = t - s;
  const float err = (s - (t - bb)) + (p - bb);
  s = t;
  e += err + pe;
}

// (s, e) += (ah + al) * b for a single FP32 b: TwoProd of the high parts,
// the low part's product folded into e directly
__device__ __forceinline__ void df_mac1(float& s, float& e, float ah, float al, float b) {
  const float p = ah * b;
  const float pe = fmaf(ah, b, -p);
  e = fmaf(al, b, e);
  const float t = s + p;
  const float bb = t - s;
  const float err = (s - (t - bb)) + (p - bb);
  s = t;
  e += err + pe;
}

// (s, e) += (ah + al) * (bh + bl)
__device__ __forceinline__ void df_mac2(float& s, float& e, float ah, float al, float bh, float bl) {
  const float p = ah * bh;
  float pe = fmaf(ah, bh, -p);
  pe = fmaf(ah, bl, pe);
  pe = fmaf(al, bh, pe);
  const float t = s + p;
  const float bb = t - s;
  const float err = (s - (t - bb)) + (p - bb);
  s = t;
  e += err + pe;
}

// (xh + xl) - (yh + yl), renormalised
__device__ __forceinline__ df32 df_sub(float xh, float xl, float yh, float yl) {
  const float t = xh - yh;
  const float bb = t - xh;
  const float err = (xh - (t - bb)) + (-yh - bb);
  return df_norm(t, err + (xl - yl));
}

}  // namespace hps
