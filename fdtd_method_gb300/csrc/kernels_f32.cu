// FP32-arithmetic Yee kernels for the precision forms (plain FP32, compensated
// FP32 hi + int8 lo, FP16 with per-component scale), one sweep per half step.
// Same stencil as the FP64 drop-in (kokkos_functors.h:64-90, :128-151); FMA
// contraction is allowed here, since these forms are judged by their error
// against the FP64 result, not bit for bit.
#include "engine_internal.h"

namespace fdtd {

// Sum of the sources' contributions at (i, j, k) in FP32 (tables_f holds the
// FP32 copies of the profile and amplitude tables).
__device__ __forceinline__ bool source_current_f32(const SourceSet& ss, const float* tables_f,
                                                   int64_t s, int i, int j, int k, const Grid& g,
                                                   float& jx, float& jy, float& jz) {
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
    const float v = tables_f[d.amp_off + s] * tables_f[d.gx_off + di] * tables_f[d.gy_off + dj] *
                    tables_f[d.gz_off + dk];
    if (d.comp_mask & 1) jx += v;
    if (d.comp_mask & 2) jy += v;
    if (d.comp_mask & 4) jz += v;
    any = true;
  }
  return any;
}

template <class S, int kApplications>
__global__ void __launch_bounds__(256) b_update_f32(Grid g, S st, CoefSet cs, int kchunk,
                                                    int64_t* step_inc) {
  constexpr bool C = S::kComp;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k0 = blockIdx.z * kchunk;
  if (step_inc && i == 0 && j == 0 && k0 == 0) *step_inc += 1;
  if (i >= g.Ni || j >= g.Nj || k0 >= g.Nk) return;
  const int k1 = min(k0 + kchunk, g.Nk);
  const int64_t col = i + (int64_t)j * g.Ni;
  const int64_t col_in = wrap_next(i, g.Ni) + (int64_t)j * g.Ni;
  const int64_t col_jn = i + (int64_t)wrap_next(j, g.Nj) * g.Ni;
  const Coef cx = cs.cb[0], cy = cs.cb[1], cz = cs.cb[2];

  int64_t base = (int64_t)k0 * g.plane;
  Pair ex = st.load(0, col + base);
  Pair ey = st.load(1, col + base);
  for (int k = k0; k < k1; ++k) {
    const int64_t nbase = (int64_t)wrap_next(k, g.Nk) * g.plane;
    const Pair ex_kn = st.load(0, col + nbase);
    const Pair ey_kn = st.load(1, col + nbase);
    const Pair ez = st.load(2, col + base);
    const Pair ez_jn = st.load(2, col_jn + base);
    const Pair ez_in = st.load(2, col_in + base);
    const Pair ey_in = st.load(1, col_in + base);
    const Pair ex_jn = st.load(0, col_jn + base);

    const float tx = mulc<C>(cz, diff<C>(ey_kn, ey)) - mulc<C>(cy, diff<C>(ez_jn, ez));
    const float ty = mulc<C>(cx, diff<C>(ez_in, ez)) - mulc<C>(cz, diff<C>(ex_kn, ex));
    const float tz = mulc<C>(cy, diff<C>(ex_jn, ex)) - mulc<C>(cx, diff<C>(ey_in, ey));

    Pair bx = accumulate<C>(st.load(3, col + base), tx);
    Pair by = accumulate<C>(st.load(4, col + base), ty);
    Pair bz = accumulate<C>(st.load(5, col + base), tz);
    if (kApplications == 2) {
      bx = accumulate<C>(bx, tx);
      by = accumulate<C>(by, ty);
      bz = accumulate<C>(bz, tz);
    }
    st.store(3, col + base, bx);
    st.store(4, col + base, by);
    st.store(5, col + base, bz);

    ex = ex_kn;
    ey = ey_kn;
    base = nbase;
  }
}

template <class S, bool kDenseJ, bool kSources>
__global__ void __launch_bounds__(256) e_update_f32(Grid g, S st, const float* __restrict__ Jx,
                                                    const float* __restrict__ Jy,
                                                    const float* __restrict__ Jz, CoefSet cs,
                                                    int kchunk, SourceSet ss, const float* tables_f) {
  constexpr bool C = S::kComp;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k0 = blockIdx.z * kchunk;
  if (i >= g.Ni || j >= g.Nj || k0 >= g.Nk) return;
  const int k1 = min(k0 + kchunk, g.Nk);
  const int64_t col = i + (int64_t)j * g.Ni;
  const int64_t col_ip = wrap_prev(i, g.Ni) + (int64_t)j * g.Ni;
  const int64_t col_jp = i + (int64_t)wrap_prev(j, g.Nj) * g.Ni;
  const Coef cx = cs.ce[0], cy = cs.ce[1], cz = cs.ce[2];
  int64_t s = 0;
  if (kSources) s = *ss.step;

  int64_t base = (int64_t)k0 * g.plane;
  const int64_t pbase0 = (int64_t)wrap_prev(k0, g.Nk) * g.plane;
  Pair bx_kp = st.load(3, col + pbase0);
  Pair by_kp = st.load(4, col + pbase0);
  for (int k = k0; k < k1; ++k) {
    const Pair bx = st.load(3, col + base);
    const Pair by = st.load(4, col + base);
    const Pair bz = st.load(5, col + base);
    const Pair bz_jp = st.load(5, col_jp + base);
    const Pair bz_ip = st.load(5, col_ip + base);
    const Pair by_ip = st.load(4, col_ip + base);
    const Pair bx_jp = st.load(3, col_jp + base);

    float tx = mulc<C>(cy, diff<C>(bz, bz_jp)) - mulc<C>(cz, diff<C>(by, by_kp));
    float ty = mulc<C>(cz, diff<C>(bx, bx_kp)) - mulc<C>(cx, diff<C>(bz, bz_ip));
    float tz = mulc<C>(cx, diff<C>(by, by_ip)) - mulc<C>(cy, diff<C>(bx, bx_jp));

    bool has_j = false;
    float jx = 0.f, jy = 0.f, jz = 0.f;
    if (kDenseJ) {
      jx = Jx[col + base];
      jy = Jy[col + base];
      jz = Jz[col + base];
      has_j = true;
    }
    if (kSources) has_j |= source_current_f32(ss, tables_f, s, i, j, k, g, jx, jy, jz);
    if (has_j) {
      tx += mulc<C>(cs.cj, jx);
      ty += mulc<C>(cs.cj, jy);
      tz += mulc<C>(cs.cj, jz);
    }
    st.store(0, col + base, accumulate<C>(st.load(0, col + base), tx));
    st.store(1, col + base, accumulate<C>(st.load(1, col + base), ty));
    st.store(2, col + base, accumulate<C>(st.load(2, col + base), tz));

    bx_kp = bx;
    by_kp = by;
    base += g.plane;
  }
}

// ---------------------------------------------------------------------------
// Launchers.

static dim3 f32_grid(const Grid& g, int kchunk) {
  return dim3((g.Ni + 31) / 32, (g.Nj + 7) / 8, (g.Nk + kchunk - 1) / kchunk);
}

template <class S>
cudaError_t launch_b_f32(const Grid& g, const S& st, const CoefSet& cs, int applications,
                         int64_t* step_inc, cudaStream_t stream) {
  const int kchunk = 16;
  dim3 block(32, 8), grid = f32_grid(g, kchunk);
  if (applications == 2)
    b_update_f32<S, 2><<<grid, block, 0, stream>>>(g, st, cs, kchunk, step_inc);
  else
    b_update_f32<S, 1><<<grid, block, 0, stream>>>(g, st, cs, kchunk, step_inc);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_e_f32(const Grid& g, const S& st, const float* const J[3], bool dense_j,
                         const CoefSet& cs, const SourceSet& ss, const float* tables_f,
                         cudaStream_t stream) {
  const int kchunk = 16;
  dim3 block(32, 8), grid = f32_grid(g, kchunk);
  const bool src = ss.count > 0;
#define FDTD_E32(DJ, SRC) \
  e_update_f32<S, DJ, SRC><<<grid, block, 0, stream>>>(g, st, J[0], J[1], J[2], cs, kchunk, ss, tables_f)
  if (dense_j && src) FDTD_E32(true, true);
  else if (dense_j) FDTD_E32(true, false);
  else if (src) FDTD_E32(false, true);
  else FDTD_E32(false, false);
#undef FDTD_E32
  return cudaGetLastError();
}

template cudaError_t launch_b_f32<StoreF32>(const Grid&, const StoreF32&, const CoefSet&, int,
                                            int64_t*, cudaStream_t);
template cudaError_t launch_b_f32<StoreF32C>(const Grid&, const StoreF32C&, const CoefSet&, int,
                                             int64_t*, cudaStream_t);
template cudaError_t launch_b_f32<StoreF16>(const Grid&, const StoreF16&, const CoefSet&, int,
                                            int64_t*, cudaStream_t);
template cudaError_t launch_e_f32<StoreF32>(const Grid&, const StoreF32&, const float* const[3],
                                            bool, const CoefSet&, const SourceSet&, const float*,
                                            cudaStream_t);
template cudaError_t launch_e_f32<StoreF32C>(const Grid&, const StoreF32C&, const float* const[3],
                                             bool, const CoefSet&, const SourceSet&, const float*,
                                             cudaStream_t);
template cudaError_t launch_e_f32<StoreF16>(const Grid&, const StoreF16&, const float* const[3],
                                            bool, const CoefSet&, const SourceSet&, const float*,
                                            cudaStream_t);

}  // namespace fdtd
