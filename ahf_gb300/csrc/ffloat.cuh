// ffloat.cuh -- float-float ("double-single") arithmetic for the compensated
// FP32 form: a value is hi + lo with |lo| <= ulp(hi)/2, ~48 significant
// bits.  Sums use the error-free two-sum (Knuth), products the FMA-based
// two-product, so running sums of FP32 data keep ~1e-14 relative accuracy.
// The including unit is compiled with --fmad=false; every FMA below is an
// explicit __fmaf_rn.
#pragma once

#include <cuda_runtime.h>

namespace ahfgpu {

struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ffz() { return {0.f, 0.f}; }
__device__ __forceinline__ ff fff(float a) { return {a, 0.f}; }

__device__ __forceinline__ ff ff_quick(float s, float e) {
  float h = __fadd_rn(s, e);
  return {h, __fsub_rn(e, __fsub_rn(h, s))};
}

// error-free a + b
__device__ __forceinline__ ff two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

// error-free a * b
__device__ __forceinline__ ff two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  ff t = two_sum(a.lo, b.lo);
  float e = __fadd_rn(s.lo, t.hi);
  ff u = ff_quick(s.hi, e);
  e = __fadd_rn(u.lo, t.lo);
  return ff_quick(u.hi, e);
}

__device__ __forceinline__ ff ff_neg(ff a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  ff p = two_prod(a.hi, b.hi);
  float e = __fadd_rn(p.lo, __fadd_rn(__fmul_rn(a.hi, b.lo), __fmul_rn(a.lo, b.hi)));
  return ff_quick(p.hi, e);
}

__device__ __forceinline__ ff ff_mulf(ff a, float b) {
  ff p = two_prod(a.hi, b);
  float e = __fadd_rn(p.lo, __fmul_rn(a.lo, b));
  return ff_quick(p.hi, e);
}

__device__ __forceinline__ ff ff_div(ff a, ff b) {
  float q1 = __fdiv_rn(a.hi, b.hi);
  ff r = ff_sub(a, ff_mulf(b, q1));
  float q2 = __fdiv_rn(r.hi, b.hi);
  ff q = ff_quick(q1, q2);
  r = ff_sub(a, ff_mul(b, q));
  float q3 = __fdiv_rn(r.hi, b.hi);
  return ff_add(q, fff(q3));
}

__device__ __forceinline__ ff ff_sqrt(ff a) {
  if (!(a.hi > 0.f)) return ffz();
  float s = __fsqrt_rn(a.hi);
  ff r = ff_sub(a, two_prod(s, s));
  float e = __fdiv_rn(r.hi, __fmul_rn(2.f, s));
  return ff_quick(s, e);
}

__device__ __forceinline__ double ff_d(ff a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ float ff_f(ff a) { return __fadd_rn(a.hi, a.lo); }
__device__ __forceinline__ ff ff_from_d(double d) {
  float h = __double2float_rn(d);
  return {h, __double2float_rn(d - (double)h)};
}
__device__ __forceinline__ bool ff_lt(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }

}  // namespace ahfgpu
