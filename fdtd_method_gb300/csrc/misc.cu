// Conversions between FP64 host data and the storage forms, FP64 field
// diagnostics, and small helpers.
#include "engine_internal.h"

#include <algorithm>
#include <cmath>

namespace fdtd {

namespace {

constexpr int kConvThreads = 256;

inline int conv_blocks(int64_t n) {
  int64_t b = (n + kConvThreads - 1) / kConvThreads;
  if (b > 152 * 64) b = 152 * 64;  // grid-stride beyond this
  return (int)(b < 1 ? 1 : b);
}

// Splits an FP64 value into hi + lo of the compensated form.
__device__ __forceinline__ Pair split_f64(double x) {
  const float h = __double2float_rn(x);
  const float l = __double2float_rn(x - (double)h);
  return Pair{h, l};
}

// Logical flat index -> (x, y, z).
__device__ __forceinline__ void unflatten(const PLayout& L, int64_t t, int& x, int& y, int& z) {
  const int64_t plane = (int64_t)L.Ni * L.Nj;
  z = (int)(t / plane);
  const int64_t r = t - (int64_t)z * plane;
  y = (int)(r / L.Ni);
  x = (int)(r - (int64_t)y * L.Ni);
}

// Row-wise walk over the logical cells off .. off+n-1: blocks take grid rows
// (y, z) in turn, threads take consecutive x, so every warp touches a
// contiguous run of the flat FP64 array (host memory included, when the
// caller's buffer is page-locked) and no per-element division is needed.
template <class F>
__device__ __forceinline__ void for_cells_by_row(const PLayout& L, int64_t off, int64_t n, F&& f) {
  const int64_t row0 = off / L.Ni, row1 = (off + n + L.Ni - 1) / L.Ni;
  for (int64_t row = row0 + blockIdx.x; row < row1; row += gridDim.x) {
    const int z = (int)(row / L.Nj), y = (int)(row - (int64_t)z * L.Nj);
    const int64_t first = row * L.Ni;
    for (int x = threadIdx.x; x < L.Ni; x += blockDim.x) {
      const int64_t t = first + x - off;  // position in the caller's buffer
      if (t >= 0 && t < n) f(x, y, z, t);
    }
  }
}

template <class S>
__global__ void import_kernel(PLayout L, S st, int c, const double* __restrict__ src, int64_t off, int64_t n) {
  for_cells_by_row(L, off, n, [&](int x, int y, int z, int64_t t) {
    const Pair p = S::kComp ? split_f64(src[t]) : Pair{__double2float_rn(src[t]), 0.f};
    store_with_ghosts(st, L, c, x, y, z, st.to_stored(c, p));
  });
}

template <class S>
__global__ void export_kernel(PLayout L, S st, int c, double* __restrict__ dst, int64_t off, int64_t n) {
  for_cells_by_row(L, off, n, [&](int x, int y, int z, int64_t t) { dst[t] = st.load_f64(c, L.at(x, y, z)); });
}

__global__ void to_f32_kernel(const double* __restrict__ src, float* __restrict__ dst, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    dst[t] = __double2float_rn(src[t]);
}

__global__ void split_f32_kernel(const double* __restrict__ src, float* __restrict__ hi,
                                 float* __restrict__ lo, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const Pair p = split_f64(src[t]);
    hi[t] = p.hi;
    lo[t] = p.lo;
  }
}

// FP64 values of the six fields at logical cell `idx`.
struct F64Loader {
  const double* f[6];
  __device__ __forceinline__ void get(int64_t idx, double v[6]) const {
#pragma unroll
    for (int c = 0; c < 6; ++c) v[c] = f[c][idx];
  }
};
template <class S>
struct StoreLoader {
  S st;
  PLayout L;
  __device__ __forceinline__ void get(int64_t idx, double v[6]) const {
    int x, y, z;
    unflatten(L, idx, x, y, z);
    const int64_t p = L.at(x, y, z);
#pragma unroll
    for (int c = 0; c < 6; ++c) v[c] = st.load_f64(c, p);
  }
};

// Pass 1: every block accumulates its grid-stride share of the ten sums in
// FP64 and writes them to partials[block * 10 + q].
template <class Ld>
__global__ void __launch_bounds__(kDiagThreads) sums_pass1(Ld ld, int64_t cells, double* partials) {
  double acc[kDiagValues];
#pragma unroll
  for (int q = 0; q < kDiagValues; ++q) acc[q] = 0.0;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < cells;
       idx += (int64_t)gridDim.x * blockDim.x) {
    double v[6];
    ld.get(idx, v);
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      acc[c] = fma(v[c], v[c], acc[c]);
      acc[9] += isfinite(v[c]) ? 0.0 : 1.0;
    }
    acc[6] += v[1] * v[5] - v[2] * v[4];
    acc[7] += v[2] * v[3] - v[0] * v[5];
    acc[8] += v[0] * v[4] - v[1] * v[3];
  }
  __shared__ double red[kDiagThreads / 32][kDiagValues];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kDiagValues; ++q) {
    double x = acc[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < kDiagValues) {
    double x = 0.0;
    for (int w = 0; w < kDiagThreads / 32; ++w) x += red[w][threadIdx.x];
    partials[(int64_t)blockIdx.x * kDiagValues + threadIdx.x] = x;
  }
}

// Pass 2: one block folds the per-block partials into out[10].
__global__ void __launch_bounds__(kDiagThreads) sums_pass2(const double* partials, int nblocks, double* out) {
  __shared__ double red[kDiagThreads / 32][kDiagValues];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = 0; q < kDiagValues; ++q) {
    double x = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) x += partials[(int64_t)b * kDiagValues + q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < kDiagValues) {
    double x = 0.0;
    for (int w = 0; w < kDiagThreads / 32; ++w) x += red[w][threadIdx.x];
    out[threadIdx.x] = x;
  }
}

// Largest |stored value| of each FP16 component over the grid's cells: the
// rows (y, z) are taken by blocks in turn; per block the six maxima go to
// out[c] with atomicMax on the FP32 bit pattern (non-negative floats order
// as their bits; NaN is skipped by fmaxf).  out must hold zeros.
__global__ void __launch_bounds__(256) f16_absmax_kernel(PLayout L, StoreF16 st, unsigned* out) {
  float m[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  // Work items: per grid row, its 16-byte groups of 8 words (rows start on
  // 64-byte boundaries), then the words past the last whole group.
  const int64_t rows = (int64_t)L.Nj * L.Nk;
  const int groups = L.Ni / 8, per_row = groups + (L.Ni - groups * 8);
  const int64_t items = rows * per_row;
  for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < items;
       it += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = it / per_row;
    const int q = (int)(it - row * per_row);
    const int z = (int)(row / L.Nj), y = (int)(row - (int64_t)z * L.Nj);
    const int64_t base = L.at(0, y, z);
    if (q < groups) {
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const uint4 w = *reinterpret_cast<const uint4*>(st.v[c] + base + 8 * q);
        const unsigned u[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&u[k]));
          m[c] = fmaxf(m[c], fmaxf(fabsf(f.x), fabsf(f.y)));
        }
      }
    } else {
      const int x = groups * 8 + (q - groups);
#pragma unroll
      for (int c = 0; c < 6; ++c) m[c] = fmaxf(m[c], fabsf(__half2float(st.v[c][base + x])));
    }
  }
  __shared__ float red[8][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    float v = m[c];
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) red[warp][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    float v = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = fmaxf(v, red[w][threadIdx.x]);
    atomicMax(&out[threadIdx.x], __float_as_uint(v));
  }
}

// v[i] = v[i] * 2^d over n stored FP16 words (16-byte aligned), eight at a
// time through 16-byte accesses, then the words past the last group: exact
// unless a value leaves FP16's normal range.
__global__ void f16_rescale_kernel(__half* v, int64_t n, float factor) {
  const int64_t groups = n / 8;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  uint4* w = reinterpret_cast<uint4*>(v);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < groups; i += stride) {
    uint4 q = w[i];
    unsigned* u = reinterpret_cast<unsigned*>(&q);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float2 x = __half22float2(*reinterpret_cast<const __half2*>(&u[k]));
      const __half2 y = __float22half2_rn(make_float2(x.x * factor, x.y * factor));
      u[k] = *reinterpret_cast<const unsigned*>(&y);
    }
    w[i] = q;
  }
  for (int64_t i = groups * 8 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    v[i] = __float2half_rn(__half2float(v[i]) * factor);
}

}  // namespace

cudaError_t launch_f16_absmax(const PLayout& L, const StoreF16& st, unsigned* out_dev, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(out_dev, 0, 6 * sizeof(unsigned), stream);
  if (e != cudaSuccess) return e;
  const int64_t rows = (int64_t)L.Nj * L.Nk;
  const int blocks = (int)std::min<int64_t>(rows, 152 * 16);
  f16_absmax_kernel<<<blocks, 256, 0, stream>>>(L, st, out_dev);
  return cudaGetLastError();
}

cudaError_t launch_f16_rescale(__half* v, int64_t n, int shift, cudaStream_t stream) {
  if (shift == 0 || n <= 0) return cudaSuccess;
  f16_rescale_kernel<<<conv_blocks(std::max<int64_t>(n / 8, 1)), kConvThreads, 0, stream>>>(v, n,
                                                                                        std::ldexp(1.0f, shift));
  return cudaGetLastError();
}

cudaError_t launch_import(const StateView& v, int c, const double* src, int64_t off, int64_t n,
                          cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int nb = conv_blocks(n);
  switch (v.form) {
    case Form::F64:
      return cudaMemcpyAsync(v.f64[c] + off, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
    case Form::F32: import_kernel<<<nb, kConvThreads, 0, st>>>(v.L, v.s32, c, src, off, n); break;
    case Form::F32C: import_kernel<<<nb, kConvThreads, 0, st>>>(v.L, v.s32c, c, src, off, n); break;
    case Form::F16: import_kernel<<<nb, kConvThreads, 0, st>>>(v.L, v.s16, c, src, off, n); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_export(const StateView& v, int c, double* dst, int64_t off, int64_t n,
                          cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int nb = conv_blocks(n);
  switch (v.form) {
    case Form::F64:
      return cudaMemcpyAsync(dst, v.f64[c] + off, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
    case Form::F32: export_kernel<<<nb, kConvThreads, 0, st>>>(v.L, v.s32, c, dst, off, n); break;
    case Form::F32C: export_kernel<<<nb, kConvThreads, 0, st>>>(v.L, v.s32c, c, dst, off, n); break;
    case Form::F16: export_kernel<<<nb, kConvThreads, 0, st>>>(v.L, v.s16, c, dst, off, n); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_to_f32(const double* src, float* dst, int64_t n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  to_f32_kernel<<<conv_blocks(n), kConvThreads, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

cudaError_t launch_split_f32(const double* src, float* hi, float* lo, int64_t n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  split_f32_kernel<<<conv_blocks(n), kConvThreads, 0, st>>>(src, hi, lo, n);
  return cudaGetLastError();
}

int diag_blocks_for(int64_t cells, int max_blocks) {
  int64_t b = (cells + kDiagThreads * 8 - 1) / (kDiagThreads * 8);
  if (b > max_blocks) b = max_blocks;
  return (int)(b < 1 ? 1 : b);
}

cudaError_t launch_field_sums(const StateView& v, double* partials, int nblocks, double* out_dev,
                              cudaStream_t st) {
  const int64_t cells = v.g.cells;
  switch (v.form) {
    case Form::F64: {
      F64Loader ld{{v.f64[0], v.f64[1], v.f64[2], v.f64[3], v.f64[4], v.f64[5]}};
      sums_pass1<<<nblocks, kDiagThreads, 0, st>>>(ld, cells, partials);
      break;
    }
    case Form::F32:
      sums_pass1<<<nblocks, kDiagThreads, 0, st>>>(StoreLoader<StoreF32>{v.s32, v.L}, cells, partials);
      break;
    case Form::F32C:
      sums_pass1<<<nblocks, kDiagThreads, 0, st>>>(StoreLoader<StoreF32C>{v.s32c, v.L}, cells, partials);
      break;
    case Form::F16:
      sums_pass1<<<nblocks, kDiagThreads, 0, st>>>(StoreLoader<StoreF16>{v.s16, v.L}, cells, partials);
      break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  sums_pass2<<<1, kDiagThreads, 0, st>>>(partials, nblocks, out_dev);
  return cudaGetLastError();
}

}  // namespace fdtd
