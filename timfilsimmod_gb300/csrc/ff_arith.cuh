// ff_arith.cuh -- float-float ("double-word") arithmetic on the FP32 pipes:
// a value is the unevaluated sum h + l of two FP32 numbers (about 48
// significant bits). Built from the error-free transformations of Knuth
// (TwoSum), Dekker (Fast2Sum) and the FMA-based exact product, as in the
// double-word arithmetic of Dekker (1971) and Bailey's DSFUN library; error
// bounds in Joldes, Muller and Popescu (2017). On this GPU an FP64 warp
// instruction costs ~19 SM cycles (1.7 FP64 lanes per clock per SM) and an
// FP32 one about a quarter cycle, so a float-float operation of 4-11 FP32
// instructions is several times cheaper than one FP64 operation.
#pragma once

#include <cuda_runtime.h>

namespace tfs {
namespace ff {

// h + l, |l| <= ulp(h)/2 after normalisation (many intermediate values are
// left unnormalised: |l| a few ulp of h).
struct FF {
  float h, l;
};

// Knuth's TwoSum: s + e = a + b exactly. The _rn intrinsics are never
// contracted into FMAs, which would break the transformation.
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

// Dekker's Fast2Sum (|a| >= |b|): s + e = a + b exactly.
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// a * b; the exact product of the high words plus the cross terms (the
// product of the low words, ~2^-48 relative, is dropped); unnormalised.
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, fmaf(a.l, b.h, e));
  return {p, e};
}

// a + b, normalised (the "sloppy" double-word sum: its error is bounded
// relative to |a| + |b|, which is what the velocity sums need).
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const FF s = ff_two_sum(a.h, b.h);
  return ff_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}

// a - b for positions (unnormalised).
__device__ __forceinline__ FF ff_sub(FF a, FF b) {
  FF s = ff_two_sum(a.h, -b.h);
  s.l = __fadd_rn(s.l, __fsub_rn(a.l, b.l));
  return s;
}

// Compensated accumulation: v.h carries the running sum, v.l every rounding
// error and low word.
__device__ __forceinline__ void ff_acc(FF &v, FF t) {
  const FF s = ff_two_sum(v.h, t.h);
  v.h = s.h;
  v.l = __fadd_rn(v.l, __fadd_rn(s.l, t.l));
}

__device__ __forceinline__ FF ff_split(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}

// a * b normalised.
__device__ __forceinline__ FF ff_mul_norm(FF a, FF b) {
  const FF p = ff_mul(a, b);
  return ff_fast_two_sum(p.h, p.l);
}

__device__ __forceinline__ FF ff_neg(FF a) { return {-a.h, -a.l}; }

// 1 / b: the FP32 quotient y0 refined by one Newton step y = y0 + y0 e,
// e = 1 - b y0 formed from the exact product b.h y0 (relative error ~2^-46).
__device__ __forceinline__ FF ff_recip(FF b) {
  const float y0 = 1.0f / b.h;
  const float ph = __fmul_rn(b.h, y0);
  const float pl = fmaf(b.h, y0, -ph);
  const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, ph), pl), __fmul_rn(b.l, y0));
  return ff_fast_two_sum(y0, __fmul_rn(y0, e));
}

__device__ __forceinline__ double ff_to_double(FF a) { return (double)a.h + (double)a.l; }

}  // namespace ff
}  // namespace tfs
