// df32.cuh — double-float arithmetic on the FP32 pipe.
//
// A value is an unevaluated sum x + y of two floats (float2 .x = high part,
// .y = low part), carrying about 44 significant bits.  Products use the
// FMA-based exact product (a*b = p + fma(a, b, -p)) and sums Knuth's
// branch-free two-sum, the error-free transformations of Dekker (1971) and
// Ogita, Rump and Oishi, "Accurate sum and dot product" (SIAM J. Sci. Comput.
// 26, 2005).  Results are not renormalised after every operation: the low part
// collects the rounding errors of the high parts, so it stays about 2^-23
// times the magnitude of the terms that went into the value, which is all the
// next product or sum needs.
//
// Every operation uses the _rn intrinsics so the compiler never contracts a
// product into a following sum (that would break the exactness of two-sum).
#pragma once
#include <cuda_runtime.h>

namespace ads {

typedef float2 dfl;

__device__ __forceinline__ dfl df_make(float h, float l) { return make_float2(h, l); }
__device__ __forceinline__ dfl df_zero() { return make_float2(0.f, 0.f); }

// a * b
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  return make_float2(p, e);
}

// a * b with b a plain float (exact in its high part)
__device__ __forceinline__ dfl df_mulf(dfl a, float b) {
  const float p = __fmul_rn(a.x, b);
  float e = __fmaf_rn(a.x, b, -p);
  e = __fmaf_rn(a.y, b, e);
  return make_float2(p, e);
}

// s + a * b with b a plain float
__device__ __forceinline__ dfl df_macf(dfl s, dfl a, float b) {
  const float p = __fmul_rn(a.x, b);
  float e = __fmaf_rn(a.x, b, -p);
  e = __fmaf_rn(a.y, b, e);
  const float t = __fadd_rn(s.x, p);
  const float bp = __fsub_rn(t, s.x);
  const float err = __fadd_rn(__fsub_rn(s.x, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  return make_float2(t, __fadd_rn(s.y, __fadd_rn(err, e)));
}

// r - a as a float: the two-sum of r and -a.x is exact, then its error and
// the low part are added, with at most two roundings
__device__ __forceinline__ float df_sub_to_float(float r, dfl a) {
  const float t = __fsub_rn(r, a.x);
  const float bp = __fsub_rn(t, r);
  const float err = __fadd_rn(__fsub_rn(r, __fsub_rn(t, bp)), __fsub_rn(-a.x, bp));
  return __fadd_rn(t, __fsub_rn(err, a.y));
}

// a + b
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  const float t = __fadd_rn(a.x, b.x);
  const float bp = __fsub_rn(t, a.x);
  const float err = __fadd_rn(__fsub_rn(a.x, __fsub_rn(t, bp)), __fsub_rn(b.x, bp));
  return make_float2(t, __fadd_rn(__fadd_rn(a.y, b.y), err));
}

// s + a * b
__device__ __forceinline__ dfl df_mac(dfl s, dfl a, dfl b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  const float t = __fadd_rn(s.x, p);
  const float bp = __fsub_rn(t, s.x);
  const float err = __fadd_rn(__fsub_rn(s.x, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  return make_float2(t, __fadd_rn(s.y, __fadd_rn(err, e)));
}

// first term of a sum (FIRST) or s + a * b: lets unrolled loops start without
// an add of zero
template <bool FIRST>
__device__ __forceinline__ dfl df_acc(dfl s, dfl a, dfl b) {
  if constexpr (FIRST) return df_mul(a, b);
  else return df_mac(s, a, b);
}

__device__ __forceinline__ dfl df_neg(dfl a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ dfl df_shfl_up(dfl v, int d) {
  return make_float2(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
}

}  // namespace ads
