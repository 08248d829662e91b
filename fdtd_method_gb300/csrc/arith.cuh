// Arithmetic policies of the FP32-arithmetic forms.
//
// A value is a pair (h, l) of floats whose sum is the field value; the
// policies differ in how much of l they carry through an update:
//
//   ArithPlain  l is always 0: plain FP32 (also the FP16 storage form).
//   ArithComp   compensated accumulation: the curl increment is one float
//               formed from differences that keep both words of each pair,
//               and it is added to the stored pair with Fast2Sum (exact
//               where the field outweighs its increment) and renormalised,
//               so the accumulated field loses nothing but its final
//               rounding.  Source terms are double-float products
//               (FMA splits).  This is the compensated form (a BF16 l word
//               keeps the pair's significand at 32 bits or more, against 24
//               for plain FP32).
//
// Every error-free step is written with __fadd_rn / __fsub_rn / __fmul_rn,
// which the compiler never contracts or reassociates.
#pragma once

#include "storage.cuh"

namespace fdtd {

// TwoSum (Knuth): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  const float ap = __fsub_rn(s, bp);
  e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}

// Double-float helpers (value = h + l): products and sums carried with an
// FP32 error term, renormalised with Fast2Sum.
__device__ __forceinline__ Pair df_renorm(float s, float e) {
  const float h = __fadd_rn(s, e);
  return Pair{h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ Pair df_mul(Pair a, Pair b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_renorm(p, e);
}

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

// Differences with one FP16 operand, rounded once to FP32 (the sm_100
// family's mixed-precision sub/fma): the same value as converting the half
// first and subtracting in FP32, without the conversion instruction.
// h - c:
__device__ __forceinline__ float sub_h_f(__half h, float c) {
  float d;
  asm("sub.rn.f32.f16 %0, %1, %2;" : "=f"(d) : "h"(__half_as_ushort(h)), "f"(c));
  return d;
}
// c - h, as h * (-1) + c (one rounding; a zero result is +0 exactly when
// c - h gives +0):
__device__ __forceinline__ float sub_f_h(float c, __half h) {
  float d;
  const unsigned short minus_one = 0xBC00u;
  asm("fma.rn.f32.f16 %0, %1, %2, %3;" : "=f"(d) : "h"(__half_as_ushort(h)), "h"(minus_one), "f"(c));
  return d;
}

// The same with a BF16 operand (the compensated form's lo words): h - c and
// c - h.
__device__ __forceinline__ float sub_bf_f(uint16_t h, float c) {
  float d;
  asm("sub.rn.f32.bf16 %0, %1, %2;" : "=f"(d) : "h"(h), "f"(c));
  return d;
}
__device__ __forceinline__ float sub_f_bf(float c, uint16_t h) {
  float d;
  const unsigned short minus_one = 0xBF80u;
  asm("fma.rn.f32.bf16 %0, %1, %2, %3;" : "=f"(d) : "h"(h), "h"(minus_one), "f"(c));
  return d;
}

struct ArithPlain {
  static constexpr bool kPairs = false;  // neighbours need only h
  // c1 (a1 - b1) - c2 (a2 - b2) with one FMA, written out so that every
  // kernel evaluates it identically.
  __device__ __forceinline__ static Pair curl(Coef c1, Pair a1, Pair b1, Coef c2, Pair a2, Pair b2) {
    return Pair{__fmaf_rn(c1.hi, __fsub_rn(a1.hi, b1.hi), -__fmul_rn(c2.hi, __fsub_rn(a2.hi, b2.hi))), 0.f};
  }
  // curl from its two differences d1 = a1 - b1, d2 = a2 - b2 (as curl forms them)
  __device__ __forceinline__ static Pair curl_d(Coef c1, float d1, Coef c2, float d2) {
    return Pair{__fmaf_rn(c1.hi, d1, -__fmul_rn(c2.hi, d2)), 0.f};
  }
  __device__ __forceinline__ static Pair add(Pair p, Pair q) { return Pair{__fadd_rn(p.hi, q.hi), 0.f}; }
  __device__ __forceinline__ static Pair twice(Pair t) { return Pair{2.f * t.hi, 0.f}; }
  __device__ __forceinline__ static Pair acc(Pair v, Pair t) { return Pair{__fadd_rn(v.hi, t.hi), 0.f}; }
  __device__ __forceinline__ static Pair acc_curl(Pair v, Pair t) { return acc(v, t); }

  // Current values: FP32.
  using Cur = float;
  __device__ __forceinline__ static Cur cur_zero() { return 0.f; }
  __device__ __forceinline__ static Cur cur_table(const SourceSet& ss, int64_t off) { return ss.tables_f[off]; }
  __device__ __forceinline__ static Cur cur_dense(float j) { return j; }
  __device__ __forceinline__ static Cur cur_mul(Cur a, Cur b) { return __fmul_rn(a, b); }
  __device__ __forceinline__ static Cur cur_add(Cur a, Cur b) { return __fadd_rn(a, b); }
  __device__ __forceinline__ static bool cur_nonzero(Cur a) { return a != 0.f; }
  // cJ * J
  __device__ __forceinline__ static Pair cur_term(Coef cj, Cur j) { return Pair{__fmul_rn(cj.hi, j), 0.f}; }
};

struct ArithComp {
  static constexpr bool kPairs = true;
  // a - b of two stored pairs as one float: the hi words and the lo words
  // are subtracted separately, so the difference keeps what the lo words hold
  // (a field's accumulated precision) and is rounded relative to itself.
  __device__ __forceinline__ static float dif(Pair a, Pair b) {
    return __fadd_rn(__fsub_rn(a.hi, b.hi), __fsub_rn(a.lo, b.lo));
  }
  // The curl increment c1 (a1 - b1) - c2 (a2 - b2) as one float (lo = 0),
  // with the coefficients' lo parts folded in.  Its rounding error is
  // relative to the increment, a small fraction of the field it is added
  // to; the accumulation (acc) is the compensated part.
  __device__ __forceinline__ static Pair curl(Coef c1, Pair a1, Pair b1, Coef c2, Pair a2, Pair b2) {
    return curl_d(c1, dif(a1, b1), c2, dif(a2, b2));
  }
  // curl from its two differences d1 = dif(a1, b1), d2 = dif(a2, b2)
  __device__ __forceinline__ static Pair curl_d(Coef c1, float d1, Coef c2, float d2) {
    const float m = __fmaf_rn(c2.hi, d2, __fmul_rn(c2.lo, d2));
    return Pair{__fmaf_rn(c1.hi, d1, __fmaf_rn(c1.lo, d1, -m)), 0.f};
  }
  __device__ __forceinline__ static Pair add(Pair p, Pair q) {
    float s, e;
    two_sum(p.hi, q.hi, s, e);
    return Pair{s, __fadd_rn(e, __fadd_rn(p.lo, q.lo))};
  }
  __device__ __forceinline__ static Pair twice(Pair t) { return Pair{2.f * t.hi, 2.f * t.lo}; }
  // Current values: double-float (hi + lo FP32 tables), so the compensated
  // form evaluates its sources without the FP64 pipe.
  using Cur = Pair;
  __device__ __forceinline__ static Cur cur_zero() { return Pair{0.f, 0.f}; }
  __device__ __forceinline__ static Cur cur_table(const SourceSet& ss, int64_t off) {
    return Pair{ss.tables_f[off], ss.tables_f[off + ss.lo_off]};
  }
  __device__ __forceinline__ static Cur cur_dense(float j) { return Pair{j, 0.f}; }
  __device__ __forceinline__ static Cur cur_mul(Cur a, Cur b) { return df_mul(a, b); }
  __device__ __forceinline__ static Cur cur_add(Cur a, Cur b) {
    const Pair s = add(a, b);
    return df_renorm(s.hi, s.lo);
  }
  __device__ __forceinline__ static bool cur_nonzero(Cur a) { return a.hi != 0.f || a.lo != 0.f; }
  __device__ __forceinline__ static Pair cur_term(Coef cj, Cur j) { return df_mul(Pair{cj.hi, cj.lo}, j); }

  // v + t, renormalised: |l| <= ulp(h)/2 afterwards.  The sum of the hi
  // words is split with Fast2Sum, exact when |v.hi| >= |t.hi| (the field
  // against its increment: every cell but those where the field crosses
  // zero, whose error then stays within an ulp of the increment).
  __device__ __forceinline__ static Pair acc(Pair v, Pair t) {
    const float s = __fadd_rn(v.hi, t.hi);
    const float e = __fsub_rn(t.hi, __fsub_rn(s, v.hi));
    const float l = __fadd_rn(__fadd_rn(v.lo, e), t.lo);
    const float h2 = __fadd_rn(s, l);
    const float l2 = __fsub_rn(l, __fsub_rn(h2, s));
    return Pair{h2, l2};
  }
  // acc for an increment whose lo word is zero (a curl term without
  // current): the same value without the addition of t.lo (it can differ
  // from acc only in the sign of a zero lo word).
  __device__ __forceinline__ static Pair acc_curl(Pair v, Pair t) {
    const float s = __fadd_rn(v.hi, t.hi);
    const float e = __fsub_rn(t.hi, __fsub_rn(s, v.hi));
    const float l = __fadd_rn(v.lo, e);
    const float h2 = __fadd_rn(s, l);
    const float l2 = __fsub_rn(l, __fsub_rn(h2, s));
    return Pair{h2, l2};
  }
};

}  // namespace fdtd
