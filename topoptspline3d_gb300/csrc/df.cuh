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

}  // namespace topo
