// fdtd_field_sums_noalloc: the FP64 field sums of fdtd_field_sums for callers
// that cannot allocate device memory: a host application that routes every
// device allocation through its own pool allocator and forbids direct
// cudaMalloc calls (so the library cannot create a handle and its scratch);
// a monitoring loop beside a running simulation that must not call cudaMalloc,
// which can synchronise the whole device and stall the simulation's kernels;
// and a process whose device memory is already fully reserved by the solver.
//
// The caller passes the six FP64 field arrays (device addresses, the dense
// i + j*Ni + k*Ni*Nj layout of the drop-in form) and a device buffer for the
// ten results; the per-block partial sums live in a file-scope device array of
// fixed size, kNoAllocBlocks * 10 doubles (5 MiB), which every GPU that loads
// the library holds until the process exits.  Each block reduces a fixed
// span of kNoAllocCellsPerBlock cells, so the largest accepted grid is
// kNoAllocBlocks * kNoAllocCellsPerBlock = 268,435,456 cells (512^3 fits);
// larger grids are rejected with FDTD_ERR_INVALID_ARGUMENT.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (the host-side name of a __device__ array is not a
// device address); make that first call before any stream capture.  Later
// calls look it up again unless their stream is capturing (the address moves
// if the device's context was reset and the module reloaded); a capturing
// call uses the address found last.  All calls share the one array: calls
// whose kernels overlap on the GPU (different streams, no ordering between
// them) race on it.  Every slot a call reads is written by the same call
// first, so nothing needs clearing between calls.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/fdtd_gb300.h"

namespace fdtd {
void set_last_error(const std::string& msg);  // engine.cu: the text fdtd_last_error() returns
}

namespace {

constexpr int kNoAllocValues = 10;
constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocCellsPerThread = 16;
constexpr int64_t kNoAllocCellsPerBlock = (int64_t)kNoAllocThreads * kNoAllocCellsPerThread;
constexpr int kNoAllocBlocks = 65536;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kNoAllocBlocks * kNoAllocValues];

std::mutex g_setup_mutex;
double* g_partials_addr[kMaxDevices] = {nullptr};


// Pass 1: block b sums cells [b * span, (b+1) * span) into slot b.
__global__ void __launch_bounds__(kNoAllocThreads)
    noalloc_pass1(const double* __restrict__ ex, const double* __restrict__ ey, const double* __restrict__ ez,
                  const double* __restrict__ bx, const double* __restrict__ by, const double* __restrict__ bz,
                  int64_t cells, double* partials) {
  double acc[kNoAllocValues];
#pragma unroll
  for (int q = 0; q < kNoAllocValues; ++q) acc[q] = 0.0;
  const int64_t begin = (int64_t)blockIdx.x * kNoAllocCellsPerBlock;
#pragma unroll 4
  for (int s = 0; s < kNoAllocCellsPerThread; ++s) {
    const int64_t i = begin + (int64_t)s * kNoAllocThreads + threadIdx.x;
    if (i >= cells) break;
    const double v[6] = {ex[i], ey[i], ez[i], bx[i], by[i], bz[i]};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      acc[c] = fma(v[c], v[c], acc[c]);
      acc[9] += isfinite(v[c]) ? 0.0 : 1.0;
    }
    acc[6] += v[1] * v[5] - v[2] * v[4];
    acc[7] += v[2] * v[3] - v[0] * v[5];
    acc[8] += v[0] * v[4] - v[1] * v[3];
  }
  __shared__ double red[kNoAllocThreads / 32][kNoAllocValues];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kNoAllocValues; ++q) {
    double x = acc[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < kNoAllocValues) {
    double x = 0.0;
    for (int w = 0; w < kNoAllocThreads / 32; ++w) x += red[w][threadIdx.x];
    partials[(int64_t)blockIdx.x * kNoAllocValues + threadIdx.x] = x;
  }
}

// Pass 2: one block folds slots [0, nblocks) into out[10].
__global__ void __launch_bounds__(kNoAllocThreads)
    noalloc_pass2(const double* partials, int nblocks, double* out) {
  __shared__ double red[kNoAllocThreads / 32][kNoAllocValues];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = 0; q < kNoAllocValues; ++q) {
    double x = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += kNoAllocThreads) x += partials[(int64_t)b * kNoAllocValues + q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < kNoAllocValues) {
    double x = 0.0;
    for (int w = 0; w < kNoAllocThreads / 32; ++w) x += red[w][threadIdx.x];
    out[threadIdx.x] = x;
  }
}

int noalloc_fail(int code, const std::string& msg) {
  fdtd::set_last_error(msg);
  return code;
}

// Device address of the static partials on the current device: looked up on
// the device's first call and on every call outside a stream capture; a call
// on a capturing stream takes the address found last.
int partials_address(cudaStream_t st, double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(FDTD_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(FDTD_ERR_UNSUPPORTED, "device index beyond the supported range");
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(st, &cs);
  if (e != cudaSuccess)
    return noalloc_fail(FDTD_ERR_CUDA, std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(e));
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_partials_addr[dev] || cs == cudaStreamCaptureStatusNone) {
    if (cs != cudaStreamCaptureStatusNone)
      return noalloc_fail(FDTD_ERR_INVALID_ARGUMENT,
                          "the first call on a device must come before any stream capture");
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess || !p)
      return noalloc_fail(FDTD_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_partials_addr[dev] = static_cast<double*>(p);
  }
  *out = g_partials_addr[dev];
  return FDTD_OK;
}

}  // namespace

extern "C" {

int fdtd_field_sums_noalloc(const double* const fields[6], int64_t cells, double* out_device, void* stream) {
  if (!fields || !out_device) return noalloc_fail(FDTD_ERR_INVALID_ARGUMENT, "null argument");
  for (int c = 0; c < 6; ++c)
    if (!fields[c]) return noalloc_fail(FDTD_ERR_INVALID_ARGUMENT, "null field pointer");
  if (cells <= 0) return noalloc_fail(FDTD_ERR_INVALID_ARGUMENT, "cells must be positive");
  const int64_t blocks = (cells + kNoAllocCellsPerBlock - 1) / kNoAllocCellsPerBlock;
  if (blocks > kNoAllocBlocks)
    return noalloc_fail(FDTD_ERR_INVALID_ARGUMENT,
                        "grid too large for fdtd_field_sums_noalloc: at most 268435456 cells "
                        "(its fixed device scratch holds 65536 block partials); use fdtd_field_sums");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* partials = nullptr;
  if (int rc = partials_address(st, &partials)) return rc;
  noalloc_pass1<<<(unsigned)blocks, kNoAllocThreads, 0, st>>>(fields[0], fields[1], fields[2], fields[3],
                                                                fields[4], fields[5], cells, partials);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    noalloc_pass2<<<1, kNoAllocThreads, 0, st>>>(partials, (int)blocks, out_device);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return noalloc_fail(FDTD_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return FDTD_OK;
}

}  // extern "C"
