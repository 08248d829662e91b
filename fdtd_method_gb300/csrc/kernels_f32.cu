// FP32-arithmetic Yee sweeps of the precision forms (plain FP32, compensated
// FP32 hi + BF16 lo, FP16 with per-component scale), on the padded layout of
// layout.cuh: one z-marching sweep per update, in place, one thread per
// (x, y) column (B half step, E step, B double half step) — 18 values moved
// per cell-step.  x/y neighbours come from the ghost cells; z wraps by index.
//
// Same stencil as the FP64 drop-in (kokkos_functors.h:64-90 E, :128-151 B);
// the arithmetic comes from the policies in arith.cuh.  These sweeps run the
// split pipeline of a handle without its second copy, z slabs' split
// schedule and the batch's pending half; the fused sweeps (kernels_fused1.cu,
// kernels_fused.cu, kernels_tblock.cu) evaluate the same arithmetic and
// reproduce them bit for bit.
#include "arith.cuh"
#include "engine_internal.h"
#include "sources.cuh"

namespace fdtd {

// B update of column (i, j), planes k0 .. min(k0+kchunk, kend)-1: reads E
// and B from `st`, writes B to `out` (the same storage for the in-place sweeps).
template <class S, class A, int kApplications>
__device__ __forceinline__ void b_column(const PLayout& L, const S& st, const S& out, const CoefSet& cs, int i, int j,
                                         int k0, int kchunk, int kend) {
  if (i >= L.Ni || j >= L.Nj || k0 >= kend) return;
  const int k1 = min(k0 + kchunk, kend);
  const int64_t col = L.at(i, j, 0), col_in = L.at(i + 1, j, 0), col_jn = L.at(i, j + 1, 0);

  Pair ex = st.load(0, col + (int64_t)k0 * L.pplane);
  Pair ey = st.load(1, col + (int64_t)k0 * L.pplane);
  for (int k = k0; k < k1; ++k) {
    const int64_t base = (int64_t)k * L.pplane;
    const int64_t nbase = (int64_t)wrap_next(k, L.Nk) * L.pplane;
    const Pair ex_kn = st.load(0, col + nbase);
    const Pair ey_kn = st.load(1, col + nbase);
    const Pair ez = st.load(2, col + base);
    Pair tx = A::curl(bcoef<S>(cs, st, 0, 0), ey_kn, ey, bcoef<S>(cs, st, 0, 1), st.load(2, col_jn + base), ez);
    Pair ty = A::curl(bcoef<S>(cs, st, 1, 0), st.load(2, col_in + base), ez, bcoef<S>(cs, st, 1, 1), ex_kn, ex);
    Pair tz = A::curl(bcoef<S>(cs, st, 2, 0), st.load(0, col_jn + base), ex, bcoef<S>(cs, st, 2, 1), st.load(1, col_in + base), ey);
    if (kApplications == 2) {
      tx = A::twice(tx);
      ty = A::twice(ty);
      tz = A::twice(tz);
    }
    store_with_ghosts(out, L, 3, i, j, k, A::acc_curl(st.load(3, col + base), tx));
    store_with_ghosts(out, L, 4, i, j, k, A::acc_curl(st.load(4, col + base), ty));
    store_with_ghosts(out, L, 5, i, j, k, A::acc_curl(st.load(5, col + base), tz));
    ex = ex_kn;
    ey = ey_kn;
  }
}

template <class S, class A, int kApplications>
__global__ void __launch_bounds__(256) b_sweep(PLayout L, S st, S out, CoefSet cs, int kchunk, int kbeg, int kend) {
  b_column<S, A, kApplications>(L, st, out, cs, blockIdx.x * blockDim.x + threadIdx.x,
                                blockIdx.y * blockDim.y + threadIdx.y, kbeg + blockIdx.z * kchunk, kchunk, kend);
}

// One B half step of every domain of a batch (the pending one, applied before
// a write): block b belongs to the domain d with block_start[d] <= b <
// block_start[d+1].
template <class S, class A>
__global__ void __launch_bounds__(256) b_sweep_batch(const BatchDomain<S>* __restrict__ doms,
                                                     const int64_t* __restrict__ block_start, int n_dom, int parity) {
  const int64_t b = blockIdx.x;
  int lo = 0, hi = n_dom;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (block_start[mid] <= b) lo = mid;
    else hi = mid;
  }
  const BatchDomain<S>& d = doms[lo];
  const int64_t local = b - block_start[lo];
  const int nbx = (d.L.Ni + 31) / 32, nby = (d.L.Nj + 7) / 8;
  const int bx = (int)(local % nbx), by = (int)((local / nbx) % nby), bz = (int)(local / ((int64_t)nbx * nby));
  b_column<S, A, 1>(d.L, d.s[parity], d.s[parity], d.cs, bx * 32 + threadIdx.x, by * 8 + threadIdx.y,
                    bz * kBatchBChunk, kBatchBChunk, d.L.Nk);
}

template <class S, class A, bool kDenseJ, bool kSources>
__global__ void __launch_bounds__(256) e_sweep(PLayout L, S st, const float* __restrict__ Jx,
                                               const float* __restrict__ Jy,
                                               const float* __restrict__ Jz, CoefSet cs, int kchunk,
                                               int kbeg, int kend, SourceSet ss, int64_t step) {
  using T = typename A::Cur;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k0 = kbeg + blockIdx.z * kchunk;
  if (i >= L.Ni || j >= L.Nj || k0 >= kend) return;
  const int k1 = min(k0 + kchunk, kend);
  const int64_t col = L.at(i, j, 0), col_ip = L.at(i - 1, j, 0), col_jp = L.at(i, j - 1, 0);
  const int64_t dcol = i + (int64_t)j * L.Ni;  // dense current index
  const int64_t dplane = (int64_t)L.Ni * L.Nj;

  const int64_t pbase0 = (int64_t)wrap_prev(k0, L.Nk) * L.pplane;
  Pair bx_kp = st.load(3, col + pbase0);
  Pair by_kp = st.load(4, col + pbase0);
  for (int k = k0; k < k1; ++k) {
    const int64_t base = (int64_t)k * L.pplane;
    const Pair bx = st.load(3, col + base);
    const Pair by = st.load(4, col + base);
    const Pair bz = st.load(5, col + base);
    Pair tx = A::curl(ecoef<S>(cs, st, 0, 0), bz, st.load(5, col_jp + base), ecoef<S>(cs, st, 0, 1), by, by_kp);
    Pair ty = A::curl(ecoef<S>(cs, st, 1, 0), bx, bx_kp, ecoef<S>(cs, st, 1, 1), bz, st.load(5, col_ip + base));
    Pair tz = A::curl(ecoef<S>(cs, st, 2, 0), by, st.load(4, col_ip + base), ecoef<S>(cs, st, 2, 1), bx, st.load(3, col_jp + base));
    T jv[3] = {A::cur_zero(), A::cur_zero(), A::cur_zero()};
    unsigned has = 0;  // J components that carry current here
    if (kDenseJ) {
      const int64_t d = dcol + (int64_t)k * dplane;
      jv[0] = A::cur_dense(Jx[d]);
      jv[1] = A::cur_dense(Jy[d]);
      jv[2] = A::cur_dense(Jz[d]);
      has = 7u;
    }
    if (kSources) has |= source_sum<A>(ss, step, i, j, k, L, jv, has);
    if (has & 1u) tx = A::add(tx, A::cur_term(jcoef<S>(cs, st, 0), jv[0]));
    if (has & 2u) ty = A::add(ty, A::cur_term(jcoef<S>(cs, st, 1), jv[1]));
    if (has & 4u) tz = A::add(tz, A::cur_term(jcoef<S>(cs, st, 2), jv[2]));
    store_with_ghosts(st, L, 0, i, j, k, (has & 1u) ? A::acc(st.load(0, col + base), tx) : A::acc_curl(st.load(0, col + base), tx));
    store_with_ghosts(st, L, 1, i, j, k, (has & 2u) ? A::acc(st.load(1, col + base), ty) : A::acc_curl(st.load(1, col + base), ty));
    store_with_ghosts(st, L, 2, i, j, k, (has & 4u) ? A::acc(st.load(2, col + base), tz) : A::acc_curl(st.load(2, col + base), tz));
    bx_kp = bx;
    by_kp = by;
  }
}

// ---------------------------------------------------------------------------
// Launchers.

template <class S> struct ArithOf { using type = ArithPlain; };
template <> struct ArithOf<StoreF32C> { using type = ArithComp; };

static dim3 sweep_grid(const PLayout& L, int kbeg, int kend, int kchunk) {
  return dim3((L.Ni + 31) / 32, (L.Nj + 7) / 8, (kend - kbeg + kchunk - 1) / kchunk);
}

template <class S>
cudaError_t launch_b_f32(const PLayout& L, const S& st, const CoefSet& cs, int applications, int kbeg, int kend,
                         cudaStream_t stream) {
  using A = typename ArithOf<S>::type;
  if (kbeg < 0 || kend > L.Nk) return cudaErrorInvalidValue;
  if (kend <= kbeg) return cudaSuccess;
  const int kchunk = 16;
  dim3 block(32, 8), grid = sweep_grid(L, kbeg, kend, kchunk);
  if (applications == 2) b_sweep<S, A, 2><<<grid, block, 0, stream>>>(L, st, st, cs, kchunk, kbeg, kend);
  else b_sweep<S, A, 1><<<grid, block, 0, stream>>>(L, st, st, cs, kchunk, kbeg, kend);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_b_f32_into(const PLayout& L, const S& st, const S& out, const CoefSet& cs, int kbeg, int kend,
                              cudaStream_t stream) {
  using A = typename ArithOf<S>::type;
  if (kbeg < 0 || kend > L.Nk) return cudaErrorInvalidValue;
  if (kend <= kbeg) return cudaSuccess;
  const int kchunk = 16;
  dim3 block(32, 8), grid = sweep_grid(L, kbeg, kend, kchunk);
  b_sweep<S, A, 1><<<grid, block, 0, stream>>>(L, st, out, cs, kchunk, kbeg, kend);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_e_f32(const PLayout& L, const S& st, const float* const J[3], bool dense_j,
                         const CoefSet& cs, const SourceSet& ss, int64_t step, int kbeg, int kend,
                         cudaStream_t stream) {
  using A = typename ArithOf<S>::type;
  if (kbeg < 0 || kend > L.Nk) return cudaErrorInvalidValue;
  if (kend <= kbeg) return cudaSuccess;
  const int kchunk = 16;
  dim3 block(32, 8), grid = sweep_grid(L, kbeg, kend, kchunk);
  const bool src = ss.count > 0;
#define FDTD_E32(DJ, SRC) \
  e_sweep<S, A, DJ, SRC><<<grid, block, 0, stream>>>(L, st, J[0], J[1], J[2], cs, kchunk, kbeg, kend, ss, step)
  if (dense_j && src) FDTD_E32(true, true);
  else if (dense_j) FDTD_E32(true, false);
  else if (src) FDTD_E32(false, true);
  else FDTD_E32(false, false);
#undef FDTD_E32
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_b_f32_batch(const void* doms, const int64_t* block_start, int n_dom, int64_t n_blocks,
                               int parity, cudaStream_t stream) {
  using A = typename ArithOf<S>::type;
  if (n_blocks <= 0) return cudaSuccess;
  if (n_blocks > 0x7fffffff) return cudaErrorInvalidValue;
  b_sweep_batch<S, A><<<(unsigned)n_blocks, dim3(32, 8), 0, stream>>>(static_cast<const BatchDomain<S>*>(doms),
                                                                     block_start, n_dom, parity);
  return cudaGetLastError();
}

#define FDTD_INSTANTIATE(S)                                                                            \
  template cudaError_t launch_b_f32<S>(const PLayout&, const S&, const CoefSet&, int, int, int, cudaStream_t); \
  template cudaError_t launch_b_f32_into<S>(const PLayout&, const S&, const S&, const CoefSet&, int, int,      \
                                            cudaStream_t);                                                    \
  template cudaError_t launch_b_f32_batch<S>(const void*, const int64_t*, int, int64_t, int, cudaStream_t); \
  template cudaError_t launch_e_f32<S>(const PLayout&, const S&, const float* const[3], bool,         \
                                       const CoefSet&, const SourceSet&, int64_t, int, int, cudaStream_t);
FDTD_INSTANTIATE(StoreF32)
FDTD_INSTANTIATE(StoreF32C)
FDTD_INSTANTIATE(StoreF16)
#undef FDTD_INSTANTIATE

}  // namespace fdtd
