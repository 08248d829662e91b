// Storage forms of the FP32-arithmetic precision paths.
//
// Every form decodes a stored value into a (hi, lo) pair of floats whose sum
// is the field value, and encodes a pair back.  The plain forms have lo == 0
// (the compiler removes every lo term); the compensated form keeps the part of
// each accumulated value that FP32 cannot hold in a narrow integer "lo" word
// scaled to the unit in the last place of hi.
#pragma once

#include <cuda_fp16.h>

#include <cstdint>

#include "common.cuh"

namespace fdtd {

struct Pair {
  float hi, lo;
};

// A coefficient split as hi + lo floats (lo == 0 for the plain forms).
struct Coef {
  float hi, lo;
};

// ---------------------------------------------------------------------------
// Plain FP32 storage.
struct StoreF32 {
  static constexpr bool kComp = false;
  using HiT = float;
  float* v[6];
  __device__ __forceinline__ Pair decode(int, float h, int8_t) const { return Pair{h, 0.f}; }
  __device__ __forceinline__ Pair load(int c, int64_t idx) const { return Pair{v[c][idx], 0.f}; }
  __device__ __forceinline__ void store(int c, int64_t idx, Pair p) const { v[c][idx] = p.hi; }
  __device__ __forceinline__ double load_f64(int c, int64_t idx) const { return (double)v[c][idx]; }
  // The value a store followed by a load returns.
  __device__ __forceinline__ Pair quantize(int, Pair p) const { return Pair{p.hi, 0.f}; }
};

// FP16 storage with a power-of-two scale per component: stored = field * 2^e.
struct StoreF16 {
  static constexpr bool kComp = false;
  using HiT = __half;
  __half* v[6];
  float scale[6];      // 2^e
  float inv_scale[6];  // 2^-e
  __device__ __forceinline__ Pair decode(int c, __half h, int8_t) const {
    return Pair{__fmul_rn(__half2float(h), inv_scale[c]), 0.f};
  }
  __device__ __forceinline__ Pair load(int c, int64_t idx) const { return decode(c, v[c][idx], 0); }
  __device__ __forceinline__ void store(int c, int64_t idx, Pair p) const {
    v[c][idx] = __float2half_rn(__fmul_rn(p.hi, scale[c]));
  }
  __device__ __forceinline__ double load_f64(int c, int64_t idx) const {
    return (double)__half2float(v[c][idx]) * (double)inv_scale[c];
  }
  __device__ __forceinline__ Pair quantize(int c, Pair p) const {
    return Pair{__fmul_rn(__half2float(__float2half_rn(__fmul_rn(p.hi, scale[c]))), inv_scale[c]), 0.f};
  }
};

// Compensated storage: FP32 hi word + signed 8-bit lo word.  lo is an
// integer multiple of 2^(E-30), E the binary exponent of hi, so with
// |lo| <= ulp(hi)/2 = 2^(E-24) the integer stays within +-64: the pair holds
// a 30-bit significand in 5 bytes.  Both scales are built from hi's exponent
// bits with integer arithmetic; for |hi| < 2^-96 the lo word reads as 0.
constexpr int kLoShift = 30;

// 2^(E-30), or 0 when that underflows.
__device__ __forceinline__ float lo_decode_scale(float hi) {
  const int s = (__float_as_int(hi) & 0x7f800000) - (kLoShift << 23);
  return __int_as_float(max(s, 0));
}
// 2^(30-E), capped at 2^127.
__device__ __forceinline__ float lo_encode_scale(float hi) {
  const int s = ((127 + 127 + kLoShift) << 23) - (__float_as_int(hi) & 0x7f800000);
  return __int_as_float(min(s, 254 << 23));
}

// Integer <-> float for |q| < 2^22 without the conversion unit: a float of
// the form 1.5 * 2^23 + q holds q in its low mantissa bits.
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;
__device__ __forceinline__ float small_int_to_float(int q) {
  return __fsub_rn(__int_as_float(kMagicBits + q), kMagic);
}
// Round-to-nearest-even of x, |x| < 2^22.
__device__ __forceinline__ int float_to_small_int(float x) {
  return __float_as_int(__fadd_rn(x, kMagic)) - kMagicBits;
}

struct StoreF32C {
  static constexpr bool kComp = true;
  using HiT = float;
  float* hi[6];
  int8_t* lo[6];
  __device__ __forceinline__ Pair decode(int, float h, int8_t q) const {
    return Pair{h, __fmul_rn(small_int_to_float(q), lo_decode_scale(h))};
  }
  __device__ __forceinline__ Pair load(int c, int64_t idx) const { return decode(c, hi[c][idx], lo[c][idx]); }
  __device__ __forceinline__ static int encode_lo(Pair p) {
    const float x = fminf(fmaxf(__fmul_rn(p.lo, lo_encode_scale(p.hi)), -127.f), 127.f);
    return float_to_small_int(x);
  }
  __device__ __forceinline__ void store(int c, int64_t idx, Pair p) const {
    hi[c][idx] = p.hi;
    lo[c][idx] = (int8_t)encode_lo(p);
  }
  __device__ __forceinline__ Pair quantize(int, Pair p) const {
    return Pair{p.hi, __fmul_rn(small_int_to_float(encode_lo(p)), lo_decode_scale(p.hi))};
  }
  __device__ __forceinline__ double load_f64(int c, int64_t idx) const {
    const Pair p = load(c, idx);
    return (double)p.hi + (double)p.lo;
  }
};

}  // namespace fdtd
