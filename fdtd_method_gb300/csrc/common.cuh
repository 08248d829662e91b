// Shared device-side definitions of the FDTD engine.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fdtd {

// Grid extents with 64-bit plane strides (the reference uses int indices,
// include/FDTD_kokkos/kokkos_functors.h:65,129, which overflow past 2^31 cells).
struct Grid {
  int Ni, Nj, Nk;
  int64_t plane;  // Ni * Nj
  int64_t cells;  // Ni * Nj * Nk
};

// Periodic neighbour of an in-range index (include/FDTD_kokkos/kokkos_functors.h:13-20:
// -1 maps to N-1, N maps to 0).
__device__ __forceinline__ int wrap_next(int i, int n) { return (i + 1 == n) ? 0 : i + 1; }
__device__ __forceinline__ int wrap_prev(int i, int n) { return (i == 0) ? n - 1 : i - 1; }

// Source descriptor as held on the device.  The profile tables live in one
// device buffer; *_off are offsets into it.
struct DevSource {
  int comp_mask;
  int i0, j0, k0;
  int ni, nj, nk;
  int64_t gx_off, gy_off, gz_off, amp_off;
  int64_t n_amp;
};

constexpr int kMaxSources = 64;

struct SourceSet {
  int count;
  const DevSource* src;    // device array [count]
  const double* tables;    // device buffer holding every profile and amplitude table
  const float* tables_f;   // the same tables split into FP32 hi (at the same
                           // offsets) and FP32 lo parts (at offset + lo_off)
  int64_t lo_off;
};

// Offset of index v inside the periodic window [o, o+n) of an axis of length N,
// or -1 if outside.
__device__ __forceinline__ int box_offset(int v, int o, int n, int N) {
  int d = v - o;
  if (d < 0) d += N;
  return d < n ? d : -1;
}

// Sum of all sources' contributions to the three J components at (i,j,k) for
// time step `s`, formed in the order of the oracle and of the reference sample's
// SetCurrent lambda: J = J + ((amp * gx) * gy) * gz, sources in registration order.
// Returns true if any source covers the cell.  No fused multiply-add.
__device__ __forceinline__ bool source_current(const SourceSet& ss, int64_t s, int i, int j, int k,
                                               const Grid& g, double& jx, double& jy, double& jz) {
  bool any = false;
  for (int q = 0; q < ss.count; ++q) {
    const DevSource& d = ss.src[q];
    if (s >= d.n_amp) continue;
    const int dk = box_offset(k, d.k0, d.nk, g.Nk);
    if (dk < 0) continue;
    const int dj = box_offset(j, d.j0, d.nj, g.Nj);
    if (dj < 0) continue;
    const int di = box_offset(i, d.i0, d.ni, g.Ni);
    if (di < 0) continue;
    const double a = ss.tables[d.amp_off + s];
    double v = __dmul_rn(a, ss.tables[d.gx_off + di]);
    v = __dmul_rn(v, ss.tables[d.gy_off + dj]);
    v = __dmul_rn(v, ss.tables[d.gz_off + dk]);
    if (d.comp_mask & 1) jx = __dadd_rn(jx, v);
    if (d.comp_mask & 2) jy = __dadd_rn(jy, v);
    if (d.comp_mask & 4) jz = __dadd_rn(jz, v);
    any = true;
  }
  return any;
}

}  // namespace fdtd
