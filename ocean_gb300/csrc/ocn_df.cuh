// ocn_df.cuh -- double-float arithmetic: a value is an unevaluated sum h + l of
// two binary32 numbers with |l| <= ulp(h)/2 (about 48 significant bits).  Sums
// and products keep their rounding errors with TwoSum and an FMA-based
// TwoProduct (Dekker; Hida, Li and Bailey's QD library, "double-double"
// arithmetic restated for binary32 pairs).  Every operation is an explicit
// round-to-nearest intrinsic, so no compiler contraction changes the result.
//
// GB300 issues FP64 instructions at a small fraction of its FP32 rate; vector
// kernels that touch every element of psi run on the FP32 pipe in this format.
#pragma once

#include <cuda_runtime.h>

namespace ocn {

struct df {
  float h, l;
};

// nearest double-float of a double (two FP64 operations: set-up paths only)
__device__ __forceinline__ df df_split(double v) {
  const float h = __double2float_rn(v);
  const float l = __double2float_rn(v - (double)h);
  return {h, l};
}
__device__ __forceinline__ double df_value(df a) { return (double)a.h + (double)a.l; }

// s + e = a + b exactly
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ df quick_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// a + b
__device__ __forceinline__ df df_add(df a, df b) {
  const df s = two_sum(a.h, b.h);
  return quick_two_sum(s.h, __fadd_rn(__fadd_rn(a.l, b.l), s.l));
}
// a + b, b a binary32 number
__device__ __forceinline__ df df_add(df a, float b) {
  const df s = two_sum(a.h, b);
  return quick_two_sum(s.h, __fadd_rn(a.l, s.l));
}
__device__ __forceinline__ df df_neg(df a) { return {-a.h, -a.l}; }

// a * b
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return quick_two_sum(p, e);
}
// a * b, b a binary32 number
__device__ __forceinline__ df df_mul(df a, float b) {
  const float p = __fmul_rn(a.h, b);
  float e = __fmaf_rn(a.h, b, -p);
  e = __fmaf_rn(a.l, b, e);
  return quick_two_sum(p, e);
}
// c + a * b
__device__ __forceinline__ df df_fma(df a, df b, df c) { return df_add(c, df_mul(a, b)); }

// (sh, sl) += a * b, the running-sum form used by the dot products
__device__ __forceinline__ void df_fma(float& sh, float& sl, df a, df b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  const float s = __fadd_rn(sh, p);
  const float bb = __fsub_rn(s, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// (ah, al) += (bh, bl), renormalised
__device__ __forceinline__ void df_add(float& ah, float& al, float bh, float bl) {
  const float s = __fadd_rn(ah, bh);
  const float bb = __fsub_rn(s, ah);
  const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
  const float lo = __fadd_rn(__fadd_rn(al, bl), err);
  const float h = __fadd_rn(s, lo);
  al = __fsub_rn(lo, __fsub_rn(h, s));
  ah = h;
}

// the binary32 number nearest to a (h + l rounded once)
__device__ __forceinline__ float df_to_float(df a) { return __fadd_rn(a.h, a.l); }

__device__ __forceinline__ df df_ld(const float2* p, size_t i) {
  const float2 v = p[i];
  return {v.x, v.y};
}
__device__ __forceinline__ void df_st(float2* p, size_t i, df a) { p[i] = make_float2(a.h, a.l); }

}  // namespace ocn
