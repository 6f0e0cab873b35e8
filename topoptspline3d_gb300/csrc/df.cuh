// Double-float arithmetic shared by the fine operator and the sensitivity.
#pragma once

#include <cuda_runtime.h>

namespace topo {

// ---------------------------------------------------------------------------
// Double-float ("float-float") arithmetic: a value is the unevaluated sum
// hi + lo of two floats with |lo| <= ulp(hi)/2, about 48 significant bits.
// Addition uses Knuth's error-free TwoSum on the high parts, folds in the low
// parts and renormalises with Dekker's Fast2Sum; multiplication forms the exact
// product error of the high parts with an FMA (TwoProd).  This is the sloppy
// double-double addition of Hida, Li and Bailey (2001) on floats.  All
// operations use the _rn intrinsics so the compiler cannot fuse or reorder
// them.  On GB300 the FP32 pipe is 58x the FP64 pipe, so the fine operator of
// the FP64 outer CG and the element sensitivity run in this arithmetic with
// FP64-level accuracy.
// ---------------------------------------------------------------------------
struct df {
  float hi, lo;
  __device__ __forceinline__ df() {}
  __device__ __forceinline__ df(float h, float l) : hi(h), lo(l) {}
  __device__ __forceinline__ explicit df(int v) : hi((float)v), lo(0.f) {}
};

__device__ __forceinline__ df df_fast2sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ df operator+(df a, df b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return df_fast2sum(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df operator-(df a, df b) { return a + df(-b.hi, -b.lo); }
__device__ __forceinline__ df operator*(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  return df_fast2sum(p, e);
}
__device__ __forceinline__ df& operator+=(df& a, df b) { a = a + b; return a; }
__device__ __forceinline__ bool operator!=(df a, df b) { return a.hi != b.hi || a.lo != b.lo; }
__device__ __forceinline__ df df_from(double x) {
  const float h = __double2float_rn(x);
  return df(h, __double2float_rn(x - (double)h));
}
__device__ __forceinline__ double df_to(df a) { return (double)a.hi + (double)a.lo; }

// Two double-float values in the lanes of the packed two-lane FP32 instructions
// of sm_100 and later (__fadd2_rn, __ffma2_rn, __fmul2_rn): per lane the same
// operations and roundings as the scalar forms above, so the results are
// identical, with half the instructions.
struct df2 {
  float2 hi, lo;
};
__device__ __forceinline__ float2 f2_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) {  // a - b, one rounding
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
__device__ __forceinline__ df2 df2_add(df2 a, df2 b) {
  const float2 s = f2_add(a.hi, b.hi);
  const float2 bb = f2_sub(s, a.hi);
  const float2 e = f2_add(f2_sub(a.hi, f2_sub(s, bb)), f2_sub(b.hi, bb));
  const float2 t = f2_add(e, f2_add(a.lo, b.lo));
  const float2 s2 = f2_add(s, t);
  return {s2, f2_sub(t, f2_sub(s2, s))};
}
__device__ __forceinline__ df2 df2_neg(df2 a) {
  const float2 m1 = make_float2(-1.f, -1.f);
  return {__fmul2_rn(a.hi, m1), __fmul2_rn(a.lo, m1)};
}

}  // namespace topo
