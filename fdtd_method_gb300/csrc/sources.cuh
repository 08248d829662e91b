// Current-source evaluation of the FP32-arithmetic kernels.  Current values
// are A::Cur: FP32 for the plain forms, double-float for the compensated one.
// A source contributes ((amp[s] gx[di]) gy[dj]) gz[dk], sources added in
// registration order (the oracle's and the reference sample's order).
#pragma once

#include "arith.cuh"
#include "layout.cuh"

namespace fdtd {

// Sources whose per-column factor a kernel keeps in registers (the first
// listed for a tile; further ones are evaluated per cell).  One: with two,
// the batched compensated sweep spilled 92 bytes per thread and ran 12 %
// slower on its workload of one pulse per domain.
constexpr int kFastSources = 1;

// jv[c] += v for the components in `mask`; a component not yet in `set`
// (bit c: jv[c] already holds current) takes v itself, which is the bits of
// 0 + v (v is a normalised value) without the addition.
template <class A>
__device__ __forceinline__ void add_current(typename A::Cur jv[3], int mask, typename A::Cur v, unsigned set) {
  if (mask & 1) jv[0] = (set & 1u) ? A::cur_add(jv[0], v) : v;
  if (mask & 2) jv[1] = (set & 2u) ? A::cur_add(jv[1], v) : v;
  if (mask & 4) jv[2] = (set & 4u) ? A::cur_add(jv[2], v) : v;
}

// Every source at logical cell (i, j, k), time step s, added to jv (whose
// components in `set` already hold current).  Returns the mask of the J
// components that received current (bit c: component c); only those get the
// current term.
template <class A>
__device__ __forceinline__ unsigned source_sum(const SourceSet& ss, int64_t s, int i, int j, int k,
                                               const PLayout& L, typename A::Cur jv[3], unsigned set) {
  unsigned any = 0;
  for (int q = 0; q < ss.count; ++q) {
    const DevSource& d = ss.src[q];
    if (s >= d.n_amp) continue;
    const int dk = box_offset(k, d.k0, d.nk, L.Nk);
    if (dk < 0) continue;
    const int dj = box_offset(j, d.j0, d.nj, L.Nj);
    if (dj < 0) continue;
    const int di = box_offset(i, d.i0, d.ni, L.Ni);
    if (di < 0) continue;
    const typename A::Cur v =
        A::cur_mul(A::cur_mul(A::cur_mul(A::cur_table(ss, d.amp_off + s), A::cur_table(ss, d.gx_off + di)),
                              A::cur_table(ss, d.gy_off + dj)),
                   A::cur_table(ss, d.gz_off + dk));
    add_current<A>(jv, d.comp_mask, v, set | any);
    any |= (unsigned)d.comp_mask;
  }
  return any;
}

// Per-column state of the first kFastSources sources: (amp gx) gy, computed
// once per launch.
template <class A>
struct ColumnSources {
  typename A::Cur xy[kFastSources];
  unsigned mask = 0;

  __device__ __forceinline__ void init(const SourceSet& ss, int x, int y, int64_t step, const PLayout& L) {
#pragma unroll
    for (int q = 0; q < kFastSources; ++q) {
      xy[q] = A::cur_zero();
      if (q < ss.count) {
        const DevSource& d = ss.src[q];
        const int di = box_offset(x, d.i0, d.ni, L.Ni);
        const int dj = box_offset(y, d.j0, d.nj, L.Nj);
        if (step < d.n_amp && di >= 0 && dj >= 0) {
          xy[q] = A::cur_mul(A::cur_mul(A::cur_table(ss, d.amp_off + step), A::cur_table(ss, d.gx_off + di)),
                             A::cur_table(ss, d.gy_off + dj));
          mask |= 1u << q;
        }
      }
    }
  }
  // Adds the contributions at plane k; returns the mask of J components that
  // received current.
  __device__ __forceinline__ unsigned eval(const SourceSet& ss, int k, const PLayout& L,
                                           typename A::Cur jv[3], unsigned set) const {
    unsigned any = 0;
#pragma unroll
    for (int q = 0; q < kFastSources; ++q) {
      if (mask & (1u << q)) {
        const DevSource& d = ss.src[q];
        const int dk = box_offset(k, d.k0, d.nk, L.Nk);
        if (dk >= 0) {
          add_current<A>(jv, d.comp_mask, A::cur_mul(xy[q], A::cur_table(ss, d.gz_off + dk)), set | any);
          any |= (unsigned)d.comp_mask;
        }
      }
    }
    return any;
  }
};

}  // namespace fdtd
