// Storage forms of the FP32-arithmetic precision paths.
//
// Every form decodes a stored value into a (hi, lo) pair of floats whose sum
// is the field value, and encodes a pair back.  The plain forms have lo == 0
// (the compiler removes every lo term); the compensated form keeps the part of
// each accumulated value that FP32 cannot hold in a BF16 "lo" word.
#pragma once

#include <cuda_bf16.h>
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
  __device__ __forceinline__ Pair decode(int, float h, uint16_t) const { return Pair{h, 0.f}; }
  __device__ __forceinline__ Pair load(int c, int64_t idx) const { return Pair{v[c][idx], 0.f}; }
  __device__ __forceinline__ void store(int c, int64_t idx, Pair p) const { v[c][idx] = p.hi; }
  // Stores already encoded words (enc_hi / enc_lo).
  __device__ __forceinline__ void store_words(int c, int64_t idx, float h, uint16_t) const { v[c][idx] = h; }
  __device__ __forceinline__ double load_f64(int c, int64_t idx) const { return (double)v[c][idx]; }
  __device__ __forceinline__ Pair to_stored(int, Pair p) const { return p; }
  // The value a store followed by a load returns.
  __device__ __forceinline__ Pair quantize(int, Pair p) const { return Pair{p.hi, 0.f}; }
  // The stored words of a value (quantize(c, p) == decode(c, enc_hi(c, p), enc_lo(p))).
  __device__ __forceinline__ float enc_hi(int, Pair p) const { return p.hi; }
  __device__ __forceinline__ uint16_t enc_lo(Pair) const { return 0; }
};

// FP16 storage with a power-of-two scale per component: stored = field * 2^e.
// The kernels compute on stored values (the scale travels in the per-term
// coefficients, CoefSet::te/tb/tj), so decode and encode are conversions
// only; load_f64 and to_stored convert from and to field values.
struct StoreF16 {
  static constexpr bool kComp = false;
  using HiT = __half;
  __half* v[6];
  float scale[6];      // 2^e
  float inv_scale[6];  // 2^-e
  // The update coefficients in stored units: te[2c+t] multiplies the t-th curl
  // difference of E component c, tb[2c+t] that of B component c, tj[c] the
  // current of E component c; each is the FP64 form's coefficient times the
  // exact power of two 2^(e_dst - e_src) between the two components' scales.
  float te[6], tb[6], tj[3];
  __device__ __forceinline__ Pair decode(int, __half h, uint16_t) const { return Pair{__half2float(h), 0.f}; }
  __device__ __forceinline__ Pair load(int c, int64_t idx) const { return decode(c, v[c][idx], 0); }
  __device__ __forceinline__ void store(int c, int64_t idx, Pair p) const { v[c][idx] = __float2half_rn(p.hi); }
  // A field value in the units the kernels compute in.
  __device__ __forceinline__ Pair to_stored(int c, Pair p) const { return Pair{__fmul_rn(p.hi, scale[c]), 0.f}; }
  __device__ __forceinline__ void store_words(int c, int64_t idx, __half h, uint16_t) const { v[c][idx] = h; }
  __device__ __forceinline__ double load_f64(int c, int64_t idx) const {
    return (double)__half2float(v[c][idx]) * (double)inv_scale[c];
  }
  __device__ __forceinline__ Pair quantize(int, Pair p) const { return Pair{__half2float(__float2half_rn(p.hi)), 0.f}; }
  __device__ __forceinline__ __half enc_hi(int, Pair p) const { return __float2half_rn(p.hi); }
  __device__ __forceinline__ uint16_t enc_lo(Pair) const { return 0; }
};

// Compensated storage: FP32 hi word + BF16 lo word.  After every update
// |lo| <= ulp(hi)/2, and lo keeps 8 significant bits of its own: the pair
// holds at least a 32-bit significand in 6 bytes.  BF16 has FP32's exponent
// range, so lo needs no scaling: decoding is one shift, encoding one
// round-to-nearest conversion.
using LoT = uint16_t;  // BF16 bit pattern

__device__ __forceinline__ float bf16_bits_to_float(uint32_t q) { return __uint_as_float(q << 16); }
__device__ __forceinline__ LoT float_to_bf16_bits(float x) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}

struct StoreF32C {
  static constexpr bool kComp = true;
  using HiT = float;
  float* hi[6];
  LoT* lo[6];
  __device__ __forceinline__ Pair decode(int, float h, LoT q) const { return Pair{h, bf16_bits_to_float(q)}; }
  __device__ __forceinline__ Pair load(int c, int64_t idx) const { return decode(c, hi[c][idx], lo[c][idx]); }
  __device__ __forceinline__ void store(int c, int64_t idx, Pair p) const {
    hi[c][idx] = p.hi;
    lo[c][idx] = float_to_bf16_bits(p.lo);
  }
  __device__ __forceinline__ void store_words(int c, int64_t idx, float h, LoT q) const {
    hi[c][idx] = h;
    lo[c][idx] = q;
  }
  __device__ __forceinline__ Pair quantize(int, Pair p) const {
    return Pair{p.hi, bf16_bits_to_float(float_to_bf16_bits(p.lo))};
  }
  __device__ __forceinline__ float enc_hi(int, Pair p) const { return p.hi; }
  __device__ __forceinline__ LoT enc_lo(Pair p) const { return float_to_bf16_bits(p.lo); }
  __device__ __forceinline__ double load_f64(int c, int64_t idx) const {
    const Pair p = load(c, idx);
    return (double)p.hi + (double)p.lo;
  }
  __device__ __forceinline__ Pair to_stored(int, Pair p) const { return p; }
};

}  // namespace fdtd
