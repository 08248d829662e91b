// Throughput probe of the FP64 pipe: the peak that bounds the FP64 sweeps
// (kernels_fp64.cu), measured on the GPU the engine runs on.
//
// Every thread runs kChains independent chains x <- (x * a) + b, each step a
// DMUL and a DADD (the two instructions the bitwise FP64 sweeps issue, with
// __dmul_rn / __dadd_rn so that nothing is contracted into DFMA).  Enough
// warps are resident that the chains' latency is hidden, so the time is the
// pipe's issue rate.  The result goes to a device variable only on a
// condition that never holds for these inputs, which keeps the chains live
// without stores.
#include <cuda_runtime.h>

#include <string>

#include "handle.h"

namespace fdtd {
namespace {

constexpr int kChains = 8;
constexpr int kProbeThreads = 256;
constexpr int kProbeBlocksPerSm = 8;

__device__ double g_probe_sink;

__global__ void __launch_bounds__(kProbeThreads) fp64_chains(double a, double b, int iters) {
  double x[kChains];
#pragma unroll
  for (int q = 0; q < kChains; ++q) x[q] = 1e-3 * (threadIdx.x + q);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int q = 0; q < kChains; ++q) x[q] = __dadd_rn(__dmul_rn(x[q], a), b);
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < kChains; ++q) s += x[q];
  if (s == -1.0) g_probe_sink = s;  // a, b keep every chain in (0, 1): never taken
}

}  // namespace
}  // namespace fdtd

extern "C" int fdtd_measure_fp64_rate(double* dp_instr_per_s, double* ms_out) {
  using namespace fdtd;
  if (!dp_instr_per_s) {
    set_last_error("null output pointer");
    return FDTD_ERR_INVALID_ARGUMENT;
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const int blocks = sms * kProbeBlocksPerSm;
  const int iters = 4096;
  // x -> 0.5 x + 0.25 stays in (0, 1) from any start in [0, 1).
  if (e == cudaSuccess) fp64_chains<<<blocks, kProbeThreads>>>(0.5, 0.25, iters / 8);  // warm-up
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventRecord(e0);
  if (e == cudaSuccess) fp64_chains<<<blocks, kProbeThreads>>>(0.5, 0.25, iters);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventRecord(e1);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) {
    set_last_error(std::string("FP64 rate probe: ") + cudaGetErrorString(e));
    return FDTD_ERR_CUDA;
  }
  const double instr = 2.0 * kChains * (double)iters * (double)blocks * kProbeThreads;
  *dp_instr_per_s = instr / (ms * 1e-3);
  if (ms_out) *ms_out = ms;
  return FDTD_OK;
}
