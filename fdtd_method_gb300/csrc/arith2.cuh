// Two-cell (float2) forms of the arithmetic policies of arith.cuh and of the
// storage codecs of storage.cuh, for the fused kernel that gives each thread
// two neighbouring x cells.  Every packed operation is the IEEE operation of
// the one-cell code applied to both lanes (__fadd2_rn, __fmul2_rn,
// __ffma2_rn, sm_100+), so the two-cell kernel reproduces the one-cell
// sweeps bit for bit.
#pragma once

#include <cuda_fp16.h>

#include "arith.cuh"

namespace fdtd {

struct P2 {
  float2 hi, lo;
};

struct Coef2 {
  float2 hi, lo;
};
__device__ __forceinline__ Coef2 bcast(Coef c) {
  return Coef2{make_float2(c.hi, c.hi), make_float2(c.lo, c.lo)};
}

__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
// a - b, correctly rounded (one rounding of a + (-b)).
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }

__device__ __forceinline__ P2 make_p2(Pair a, Pair b) {
  return P2{make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)};
}
__device__ __forceinline__ Pair lane0(P2 p) { return Pair{p.hi.x, p.lo.x}; }
__device__ __forceinline__ Pair lane1(P2 p) { return Pair{p.hi.y, p.lo.y}; }

__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = add2(a, b);
  const float2 bp = sub2(s, a);
  const float2 ap = sub2(s, bp);
  e = add2(sub2(a, ap), sub2(b, bp));
}

template <class A> struct Arith2;

template <>
struct Arith2<ArithPlain> {
  // fma(c1, a1 - b1, -(c2 (a2 - b2))), as ArithPlain::curl
  __device__ __forceinline__ static P2 curl(Coef2 c1, P2 a1, P2 b1, Coef2 c2, P2 a2, P2 b2) {
    const float2 m = mul2(c2.hi, sub2(a2.hi, b2.hi));
    return P2{fma2(c1.hi, sub2(a1.hi, b1.hi), neg2(m)), make_float2(0.f, 0.f)};
  }
  __device__ __forceinline__ static P2 add(P2 p, P2 q) { return P2{add2(p.hi, q.hi), make_float2(0.f, 0.f)}; }
  __device__ __forceinline__ static P2 twice(P2 t) { return P2{mul2(t.hi, make_float2(2.f, 2.f)), t.lo}; }
  __device__ __forceinline__ static P2 acc(P2 v, P2 t) { return P2{add2(v.hi, t.hi), make_float2(0.f, 0.f)}; }
};

template <>
struct Arith2<ArithComp> {
  // ArithComp::dif and ArithComp::curl on both lanes.
  __device__ __forceinline__ static float2 dif(P2 a, P2 b) { return add2(sub2(a.hi, b.hi), sub2(a.lo, b.lo)); }
  __device__ __forceinline__ static P2 curl(Coef2 c1, P2 a1, P2 b1, Coef2 c2, P2 a2, P2 b2) {
    const float2 d1 = dif(a1, b1), d2 = dif(a2, b2);
    const float2 m = fma2(c2.hi, d2, mul2(c2.lo, d2));
    return P2{fma2(c1.hi, d1, fma2(c1.lo, d1, neg2(m))), make_float2(0.f, 0.f)};
  }
  __device__ __forceinline__ static P2 add(P2 p, P2 q) {
    float2 s, e;
    two_sum2(p.hi, q.hi, s, e);
    return P2{s, add2(e, add2(p.lo, q.lo))};
  }
  __device__ __forceinline__ static P2 twice(P2 t) {
    return P2{mul2(t.hi, make_float2(2.f, 2.f)), mul2(t.lo, make_float2(2.f, 2.f))};
  }
  __device__ __forceinline__ static P2 acc(P2 v, P2 t) {
    const float2 s = add2(v.hi, t.hi);
    const float2 e = sub2(t.hi, sub2(s, v.hi));
    const float2 l = add2(add2(v.lo, e), t.lo);
    const float2 h2 = add2(s, l);
    return P2{h2, sub2(l, sub2(h2, s))};
  }
};

// ---------------------------------------------------------------------------
// Two-cell codecs.  RawLo is the packed lo word of two cells (0 if none).

template <class S> struct Codec2;

template <>
struct Codec2<StoreF32> {
  using HiT = float;
  using Raw = float2;
  __device__ __forceinline__ static P2 decode(const StoreF32&, int, float2 h, uint32_t) {
    return P2{h, make_float2(0.f, 0.f)};
  }
  __device__ __forceinline__ static P2 quantize(const StoreF32&, int, P2 p) { return P2{p.hi, make_float2(0.f, 0.f)}; }
  // Stores both cells (8-byte aligned pair).
  __device__ __forceinline__ static void store(const StoreF32& s, int c, int64_t idx, P2 p) {
    *reinterpret_cast<float2*>(s.v[c] + idx) = p.hi;
  }
};

template <>
struct Codec2<StoreF16> {
  using HiT = __half;
  using Raw = __half2;
  // stored values, as StoreF16 (the scales travel in the coefficients)
  __device__ __forceinline__ static P2 decode(const StoreF16&, int, __half2 h, uint32_t) {
    return P2{__half22float2(h), make_float2(0.f, 0.f)};
  }
  __device__ __forceinline__ static __half2 encode(const StoreF16&, int, P2 p) { return __float22half2_rn(p.hi); }
  __device__ __forceinline__ static P2 quantize(const StoreF16& s, int c, P2 p) {
    return decode(s, c, encode(s, c, p), 0);
  }
  __device__ __forceinline__ static void store(const StoreF16& s, int c, int64_t idx, P2 p) {
    *reinterpret_cast<__half2*>(s.v[c] + idx) = encode(s, c, p);
  }
};

template <>
struct Codec2<StoreF32C> {
  using HiT = float;
  using Raw = float2;
  // BF16 lo words of the two cells: low half = cell 0, high half = cell 1.
  __device__ __forceinline__ static P2 decode(const StoreF32C&, int, float2 h, uint32_t q2) {
    return P2{h, make_float2(__uint_as_float(q2 << 16), __uint_as_float(q2 & 0xffff0000u))};
  }
  __device__ __forceinline__ static uint32_t encode(P2 p) {
    const __nv_bfloat162 b = __floats2bfloat162_rn(p.lo.x, p.lo.y);
    return *reinterpret_cast<const uint32_t*>(&b);
  }
  __device__ __forceinline__ static P2 quantize(const StoreF32C& s, int c, P2 p) {
    return decode(s, c, p.hi, encode(p));
  }
  __device__ __forceinline__ static void store(const StoreF32C& s, int c, int64_t idx, P2 p) {
    *reinterpret_cast<float2*>(s.hi[c] + idx) = p.hi;
    *reinterpret_cast<uint32_t*>(s.lo[c] + idx) = encode(p);
  }
};

}  // namespace fdtd
