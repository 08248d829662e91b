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
  float* v[6];
  __device__ __forceinline__ Pair load(int c, int64_t idx) const { return Pair{v[c][idx], 0.f}; }
  __device__ __forceinline__ float load_hi(int c, int64_t idx) const { return v[c][idx]; }
  __device__ __forceinline__ void store(int c, int64_t idx, Pair p) const { v[c][idx] = p.hi; }
  __device__ __forceinline__ double load_f64(int c, int64_t idx) const { return (double)v[c][idx]; }
  // The value a store followed by a load returns.
  __device__ __forceinline__ Pair quantize(int, Pair p) const { return Pair{p.hi, 0.f}; }
};

// FP16 storage with a power-of-two scale per component: stored = field * 2^e.
struct StoreF16 {
  static constexpr bool kComp = false;
  __half* v[6];
  float scale[6];      // 2^e
  float inv_scale[6];  // 2^-e
  __device__ __forceinline__ Pair load(int c, int64_t idx) const {
    return Pair{__half2float(v[c][idx]) * inv_scale[c], 0.f};
  }
  __device__ __forceinline__ float load_hi(int c, int64_t idx) const {
    return __half2float(v[c][idx]) * inv_scale[c];
  }
  __device__ __forceinline__ void store(int c, int64_t idx, Pair p) const {
    v[c][idx] = __float2half_rn(p.hi * scale[c]);
  }
  __device__ __forceinline__ double load_f64(int c, int64_t idx) const {
    return (double)__half2float(v[c][idx]) * (double)inv_scale[c];
  }
  __device__ __forceinline__ Pair quantize(int c, Pair p) const {
    return Pair{__half2float(__float2half_rn(p.hi * scale[c])) * inv_scale[c], 0.f};
  }
};

// Compensated storage: FP32 hi word + signed 8-bit lo word.  lo is an
// integer multiple of 2^(E-30), E the binary exponent of hi, so with
// |lo| <= ulp(hi)/2 = 2^(E-24) the integer stays within +-64: the pair holds
// a 30-bit significand in 5 bytes.
constexpr int kLoShift = 30;

__device__ __forceinline__ float lo_decode_scale(float hi) {
  const int eb = (__float_as_int(hi) >> 23) & 0xff;
  return (eb > kLoShift && eb < 255) ? __int_as_float((eb - kLoShift) << 23) : 0.f;
}
__device__ __forceinline__ float lo_encode_scale(float hi) {
  const int eb = (__float_as_int(hi) >> 23) & 0xff;
  return (eb > kLoShift && eb < 255) ? __int_as_float((kLoShift + 254 - eb) << 23) : 0.f;
}

struct StoreF32C {
  static constexpr bool kComp = true;
  float* hi[6];
  int8_t* lo[6];
  __device__ __forceinline__ Pair load(int c, int64_t idx) const {
    const float h = hi[c][idx];
    return Pair{h, (float)lo[c][idx] * lo_decode_scale(h)};
  }
  __device__ __forceinline__ float load_hi(int c, int64_t idx) const { return hi[c][idx]; }
  __device__ __forceinline__ static int encode_lo(Pair p) {
    const int q = __float2int_rn(p.lo * lo_encode_scale(p.hi));
    return max(-127, min(127, q));
  }
  __device__ __forceinline__ void store(int c, int64_t idx, Pair p) const {
    hi[c][idx] = p.hi;
    lo[c][idx] = (int8_t)encode_lo(p);
  }
  __device__ __forceinline__ Pair quantize(int, Pair p) const {
    return Pair{p.hi, (float)encode_lo(p) * lo_decode_scale(p.hi)};
  }
  __device__ __forceinline__ double load_f64(int c, int64_t idx) const {
    const float h = hi[c][idx];
    return (double)h + (double)((float)lo[c][idx] * lo_decode_scale(h));
  }
};

// ---------------------------------------------------------------------------
// Arithmetic on pairs.

// a - b of two stored values.  For smooth fields neighbouring hi words are
// within a factor of two of each other, so hi_a - hi_b is exact (Sterbenz) and
// adding the lo difference recovers the difference of the full values.
template <bool kComp>
__device__ __forceinline__ float diff(Pair a, Pair b) {
  if (kComp) return (a.hi - b.hi) + (a.lo - b.lo);
  return a.hi - b.hi;
}

template <bool kComp>
__device__ __forceinline__ float mulc(Coef c, float d) {
  if (kComp) return fmaf(c.hi, d, c.lo * d);
  return c.hi * d;
}

// v + t.  Compensated: TwoSum(hi, t) moves the rounding error into lo, then a
// Fast2Sum renormalises so that |lo| <= ulp(hi)/2.
template <bool kComp>
__device__ __forceinline__ Pair accumulate(Pair v, float t) {
  if (!kComp) return Pair{v.hi + t, 0.f};
  const float s = v.hi + t;
  const float bp = s - v.hi;
  const float e = (v.hi - (s - bp)) + (t - bp);
  const float l = v.lo + e;
  const float h2 = s + l;
  const float l2 = l - (h2 - s);
  return Pair{h2, l2};
}

}  // namespace fdtd
