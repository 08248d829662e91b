// FP32-arithmetic Yee kernels of the precision forms (plain FP32,
// compensated FP32 hi + int8 lo, FP16 with per-component scale).
//
// Same stencil as the FP64 drop-in (kokkos_functors.h:64-90 E, :128-151 B);
// the arithmetic comes from the policies in arith.cuh.
//
// Two pipelines compute identical values (the tests check bit equality):
//  * split: one z-marching sweep per update (B half step, E step, B double
//    half step) — 18 values moved per cell-step;
//  * fused: one sweep per step.  Between the first and last half step of a
//    run the scheme is E <- E + c curl B followed by B <- B + 2 (c/2) curl E,
//    so one kernel does both on a 2-D tile of columns marching along z:
//    12 values moved per cell-step (read E, B; write E, B).
#include "arith.cuh"
#include "engine_internal.h"

namespace fdtd {

template <class A>
__device__ __forceinline__ Pair curl_term(Coef c1, Pair a1, Pair b1, Coef c2, Pair a2, Pair b2) {
  return A::curl(c1, a1, b1, c2, a2, b2);
}

// Current values are FP64 for the compensated form (its error budget is
// below FP32 rounding) and FP32 for the plain forms.
template <class A> struct CurT { using T = float; };
template <> struct CurT<ArithComp> { using T = double; };

template <class A>
__device__ __forceinline__ Pair current_term(const CoefSet& cs, typename CurT<A>::T j);
template <>
__device__ __forceinline__ Pair current_term<ArithPlain>(const CoefSet& cs, float j) {
  return Pair{__fmul_rn(cs.cj.hi, j), 0.f};
}
template <>
__device__ __forceinline__ Pair current_term<ArithComp>(const CoefSet& cs, double j) {
  const double s = __dmul_rn(cs.cj64, j);
  const float h = __double2float_rn(s);
  return Pair{h, __double2float_rn(s - (double)h)};
}

template <class T> __device__ __forceinline__ const T* table_of(const SourceSet& ss);
template <> __device__ __forceinline__ const double* table_of<double>(const SourceSet& ss) { return ss.tables; }
template <> __device__ __forceinline__ const float* table_of<float>(const SourceSet& ss) { return ss.tables_f; }

// Sum over every source at (i, j, k) for time step s: ((amp gx) gy) gz.
template <class T>
__device__ __forceinline__ bool source_sum(const SourceSet& ss, int64_t s, int i, int j, int k,
                                           const Grid& g, T jv[3]) {
  const T* tb = table_of<T>(ss);
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
    const T v = mul_rn(mul_rn(mul_rn(tb[d.amp_off + s], tb[d.gx_off + di]), tb[d.gy_off + dj]),
                       tb[d.gz_off + dk]);
    if (d.comp_mask & 1) jv[0] = add_rn(jv[0], v);
    if (d.comp_mask & 2) jv[1] = add_rn(jv[1], v);
    if (d.comp_mask & 4) jv[2] = add_rn(jv[2], v);
    any = true;
  }
  return any;
}

// ---------------------------------------------------------------------------
// Split pipeline.

template <class S, class A, int kApplications>
__global__ void __launch_bounds__(256) b_sweep(Grid g, S st, CoefSet cs, int kchunk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k0 = blockIdx.z * kchunk;
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
    Pair tx = curl_term<A>(cz, ey_kn, ey, cy, st.load(2, col_jn + base), ez);
    Pair ty = curl_term<A>(cx, st.load(2, col_in + base), ez, cz, ex_kn, ex);
    Pair tz = curl_term<A>(cy, st.load(0, col_jn + base), ex, cx, st.load(1, col_in + base), ey);
    if (kApplications == 2) {
      tx = A::twice(tx);
      ty = A::twice(ty);
      tz = A::twice(tz);
    }
    st.store(3, col + base, A::acc(st.load(3, col + base), tx));
    st.store(4, col + base, A::acc(st.load(4, col + base), ty));
    st.store(5, col + base, A::acc(st.load(5, col + base), tz));
    ex = ex_kn;
    ey = ey_kn;
    base = nbase;
  }
}

template <class S, class A, bool kDenseJ, bool kSources>
__global__ void __launch_bounds__(256) e_sweep(Grid g, S st, const float* __restrict__ Jx,
                                               const float* __restrict__ Jy,
                                               const float* __restrict__ Jz, CoefSet cs, int kchunk,
                                               SourceSet ss, int64_t step) {
  using T = typename CurT<A>::T;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k0 = blockIdx.z * kchunk;
  if (i >= g.Ni || j >= g.Nj || k0 >= g.Nk) return;
  const int k1 = min(k0 + kchunk, g.Nk);
  const int64_t col = i + (int64_t)j * g.Ni;
  const int64_t col_ip = wrap_prev(i, g.Ni) + (int64_t)j * g.Ni;
  const int64_t col_jp = i + (int64_t)wrap_prev(j, g.Nj) * g.Ni;
  const Coef cx = cs.ce[0], cy = cs.ce[1], cz = cs.ce[2];

  int64_t base = (int64_t)k0 * g.plane;
  const int64_t pbase0 = (int64_t)wrap_prev(k0, g.Nk) * g.plane;
  Pair bx_kp = st.load(3, col + pbase0);
  Pair by_kp = st.load(4, col + pbase0);
  for (int k = k0; k < k1; ++k) {
    const Pair bx = st.load(3, col + base);
    const Pair by = st.load(4, col + base);
    const Pair bz = st.load(5, col + base);
    Pair tx = curl_term<A>(cy, bz, st.load(5, col_jp + base), cz, by, by_kp);
    Pair ty = curl_term<A>(cz, bx, bx_kp, cx, bz, st.load(5, col_ip + base));
    Pair tz = curl_term<A>(cx, by, st.load(4, col_ip + base), cy, bx, st.load(3, col_jp + base));
    T jv[3] = {0, 0, 0};
    bool has_j = false;
    if (kDenseJ) {
      jv[0] = Jx[col + base];
      jv[1] = Jy[col + base];
      jv[2] = Jz[col + base];
      has_j = true;
    }
    if (kSources) has_j |= source_sum<T>(ss, step, i, j, k, g, jv);
    if (has_j) {
      tx = A::add(tx, current_term<A>(cs, jv[0]));
      ty = A::add(ty, current_term<A>(cs, jv[1]));
      tz = A::add(tz, current_term<A>(cs, jv[2]));
    }
    st.store(0, col + base, A::acc(st.load(0, col + base), tx));
    st.store(1, col + base, A::acc(st.load(1, col + base), ty));
    st.store(2, col + base, A::acc(st.load(2, col + base), tz));
    bx_kp = bx;
    by_kp = by;
    base += g.plane;
  }
}

// ---------------------------------------------------------------------------
// Fused pipeline: E step + B (double) half step in one sweep.
//
// The sweep reads the state from `st` and writes the new state to `out` (a
// second copy of the fields; the engine swaps the two after each step):
// tiles read halo columns and the first plane of the next z chunk, which
// their neighbours update in the same launch, so an in-place update would race.
//
// A CTA owns a tile of (32-2) x (TY-2) interior columns plus a one-column
// halo on every side, one thread per column, and marches the planes
// k0..k1 of its z chunk.  In iteration t it
//   1. loads E(t), B(t) of its column and publishes B(t) in shared memory;
//   2. computes E'(t) = E + c curl B (needs B at i-1, j-1 from shared memory
//      and B(t-1) carried in registers) on interior and high-halo columns;
//   3. computes B'(t-1) = B(t-1) + apps (c/2) curl E' (needs E'(t-1) at
//      i+1, j+1 from shared memory, E'(t) in registers) on interior columns;
//   4. stores E'(t) (t < k1) and B'(t-1); publishes E'(t).
// Plane k1 (the next chunk's first) is read and its E' computed but not
// stored; plane k0-1 contributes only B(k0-1) of the own column.
// Low-halo columns (i = x0-1 or j = y0-1) only load B.

constexpr int kFusedTX = 32;
constexpr int kFusedMaxFastSources = 4;

template <class S, class A, int TY, int kApps, bool kDenseJ, int kSrc>
__global__ void __launch_bounds__(kFusedTX* TY) fused_step(Grid g, S st, S out, CoefSet cs, int kchunk,
                                                          const float* __restrict__ Jx,
                                                          const float* __restrict__ Jy,
                                                          const float* __restrict__ Jz,
                                                          SourceSet ss, int64_t step) {
  constexpr int TX = kFusedTX;
  constexpr int NV = A::kPairs ? 2 : 1;
  using T = typename CurT<A>::T;
  __shared__ float sB[3][NV][TY][TX];
  __shared__ float sE[2][3][NV][TY][TX];

  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x0 = blockIdx.x * (TX - 2), y0 = blockIdx.y * (TY - 2);
  const int nx = min(TX - 2, g.Ni - x0), ny = min(TY - 2, g.Nj - y0);
  const int ox = tx - 1, oy = ty - 1;
  const bool off = ox > nx || oy > ny;
  const bool do_e = !off && ox >= 0 && oy >= 0;
  const bool inner = do_e && ox < nx && oy < ny;
  int x = x0 + ox, y = y0 + oy;
  x = x < 0 ? x + g.Ni : (x >= g.Ni ? x - g.Ni : x);
  y = y < 0 ? y + g.Nj : (y >= g.Nj ? y - g.Nj : y);
  if (off) x = y = 0;
  const int64_t col = x + (int64_t)y * g.Ni;
  const int k0 = blockIdx.z * kchunk;
  const int k1 = min(k0 + kchunk, g.Nk);

  // Sources: the per-column factor amp * gx * gy, once per launch.
  T sxy[kFusedMaxFastSources];
  int nsrc = 0;
  if (kSrc == 1) {
    nsrc = ss.count;
#pragma unroll
    for (int q = 0; q < kFusedMaxFastSources; ++q) {
      sxy[q] = 0;
      if (q < nsrc && do_e) {
        const DevSource& d = ss.src[q];
        const int di = box_offset(x, d.i0, d.ni, g.Ni);
        const int dj = box_offset(y, d.j0, d.nj, g.Nj);
        if (step < d.n_amp && di >= 0 && dj >= 0) {
          const T* tb = table_of<T>(ss);
          sxy[q] = mul_rn(mul_rn(tb[d.amp_off + step], tb[d.gx_off + di]), tb[d.gy_off + dj]);
        }
      }
    }
  }

  auto put = [&](float* a, Pair v) {
    a[0] = v.hi;
    if (NV == 2) a[TY * TX] = v.lo;
  };
  auto get = [&](const float* a) { return Pair{a[0], NV == 2 ? a[TY * TX] : 0.f}; };

  Pair pbx{0.f, 0.f}, pby{0.f, 0.f}, pbz{0.f, 0.f};
  Pair pex{0.f, 0.f}, pey{0.f, 0.f}, pez{0.f, 0.f};
  if (do_e) {
    const int64_t b0 = (int64_t)wrap_prev(k0, g.Nk) * g.plane;
    pbx = st.load(3, col + b0);
    pby = st.load(4, col + b0);
  }

  for (int t = k0; t <= k1; ++t) {
    const int kk = (t == g.Nk) ? 0 : t;
    const int64_t base = (int64_t)kk * g.plane;
    const int cur = t & 1;
    Pair bx{0.f, 0.f}, by{0.f, 0.f}, bz{0.f, 0.f}, ex{0.f, 0.f}, ey{0.f, 0.f}, ez{0.f, 0.f};
    if (!off) {
      bx = st.load(3, col + base);
      by = st.load(4, col + base);
      bz = st.load(5, col + base);
      put(&sB[0][0][ty][tx], bx);
      put(&sB[1][0][ty][tx], by);
      put(&sB[2][0][ty][tx], bz);
    }
    if (do_e) {
      ex = st.load(0, col + base);
      ey = st.load(1, col + base);
      ez = st.load(2, col + base);
    }
    __syncthreads();

    Pair nex{0.f, 0.f}, ney{0.f, 0.f}, nez{0.f, 0.f};
    if (do_e) {
      const Pair bz_jp = get(&sB[2][0][ty - 1][tx]);
      const Pair bz_ip = get(&sB[2][0][ty][tx - 1]);
      const Pair by_ip = get(&sB[1][0][ty][tx - 1]);
      const Pair bx_jp = get(&sB[0][0][ty - 1][tx]);
      Pair qx = curl_term<A>(cs.ce[1], bz, bz_jp, cs.ce[2], by, pby);
      Pair qy = curl_term<A>(cs.ce[2], bx, pbx, cs.ce[0], bz, bz_ip);
      Pair qz = curl_term<A>(cs.ce[0], by, by_ip, cs.ce[1], bx, bx_jp);
      T jv[3] = {0, 0, 0};
      bool has_j = false;
      if (kDenseJ) {
        jv[0] = Jx[col + base];
        jv[1] = Jy[col + base];
        jv[2] = Jz[col + base];
        has_j = true;
      }
      if (kSrc == 1) {
#pragma unroll
        for (int q = 0; q < kFusedMaxFastSources; ++q) {
          if (q < nsrc && sxy[q] != T(0)) {
            const DevSource& d = ss.src[q];
            const int dk = box_offset(kk, d.k0, d.nk, g.Nk);
            if (dk >= 0) {
              const T v = mul_rn(sxy[q], table_of<T>(ss)[d.gz_off + dk]);
              if (d.comp_mask & 1) jv[0] = add_rn(jv[0], v);
              if (d.comp_mask & 2) jv[1] = add_rn(jv[1], v);
              if (d.comp_mask & 4) jv[2] = add_rn(jv[2], v);
              has_j = true;
            }
          }
        }
      } else if (kSrc == 2) {
        has_j |= source_sum<T>(ss, step, x, y, kk, g, jv);
      }
      if (has_j) {
        qx = A::add(qx, current_term<A>(cs, jv[0]));
        qy = A::add(qy, current_term<A>(cs, jv[1]));
        qz = A::add(qz, current_term<A>(cs, jv[2]));
      }
      // E' as its storage form will hold it, so that the B' update sees the
      // same values the split sweeps reload from memory.
      nex = st.quantize(0, A::acc(ex, qx));
      ney = st.quantize(1, A::acc(ey, qy));
      nez = st.quantize(2, A::acc(ez, qz));
    }

    if (t > k0 && inner) {
      const int prv = cur ^ 1;
      const Pair ez_jn = get(&sE[prv][2][0][ty + 1][tx]);
      const Pair ez_in = get(&sE[prv][2][0][ty][tx + 1]);
      const Pair ey_in = get(&sE[prv][1][0][ty][tx + 1]);
      const Pair ex_jn = get(&sE[prv][0][0][ty + 1][tx]);
      Pair ux = curl_term<A>(cs.cb[2], ney, pey, cs.cb[1], ez_jn, pez);
      Pair uy = curl_term<A>(cs.cb[0], ez_in, pez, cs.cb[2], nex, pex);
      Pair uz = curl_term<A>(cs.cb[1], ex_jn, pex, cs.cb[0], ey_in, pey);
      if (kApps == 2) {
        ux = A::twice(ux);
        uy = A::twice(uy);
        uz = A::twice(uz);
      }
      const int64_t pb = (int64_t)(t - 1) * g.plane;
      out.store(3, col + pb, A::acc(pbx, ux));
      out.store(4, col + pb, A::acc(pby, uy));
      out.store(5, col + pb, A::acc(pbz, uz));
    }
    if (t < k1 && inner) {
      out.store(0, col + base, nex);
      out.store(1, col + base, ney);
      out.store(2, col + base, nez);
    }
    if (do_e) {
      put(&sE[cur][0][0][ty][tx], nex);
      put(&sE[cur][1][0][ty][tx], ney);
      put(&sE[cur][2][0][ty][tx], nez);
    }
    pbx = bx;
    pby = by;
    pbz = bz;
    pex = nex;
    pey = ney;
    pez = nez;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Launchers.

template <class S> struct ArithOf { using type = ArithPlain; };
template <> struct ArithOf<StoreF32C> { using type = ArithComp; };

static dim3 sweep_grid(const Grid& g, int kchunk) {
  return dim3((g.Ni + 31) / 32, (g.Nj + 7) / 8, (g.Nk + kchunk - 1) / kchunk);
}

template <class S>
cudaError_t launch_b_f32(const Grid& g, const S& st, const CoefSet& cs, int applications,
                         cudaStream_t stream) {
  using A = typename ArithOf<S>::type;
  const int kchunk = 16;
  dim3 block(32, 8), grid = sweep_grid(g, kchunk);
  if (applications == 2) b_sweep<S, A, 2><<<grid, block, 0, stream>>>(g, st, cs, kchunk);
  else b_sweep<S, A, 1><<<grid, block, 0, stream>>>(g, st, cs, kchunk);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_e_f32(const Grid& g, const S& st, const float* const J[3], bool dense_j,
                         const CoefSet& cs, const SourceSet& ss, int64_t step, cudaStream_t stream) {
  using A = typename ArithOf<S>::type;
  const int kchunk = 16;
  dim3 block(32, 8), grid = sweep_grid(g, kchunk);
  const bool src = ss.count > 0;
#define FDTD_E32(DJ, SRC) \
  e_sweep<S, A, DJ, SRC><<<grid, block, 0, stream>>>(g, st, J[0], J[1], J[2], cs, kchunk, ss, step)
  if (dense_j && src) FDTD_E32(true, true);
  else if (dense_j) FDTD_E32(true, false);
  else if (src) FDTD_E32(false, true);
  else FDTD_E32(false, false);
#undef FDTD_E32
  return cudaGetLastError();
}

template <class S, int TY>
static cudaError_t launch_fused_ty(const Grid& g, const S& st, const S& out, const float* const J[3],
                                   bool dense_j, const CoefSet& cs, const SourceSet& ss, int64_t step,
                                   int applications, int kchunk, cudaStream_t stream) {
  using A = typename ArithOf<S>::type;
  dim3 block(kFusedTX, TY);
  dim3 grid((g.Ni + kFusedTX - 3) / (kFusedTX - 2), (g.Nj + TY - 3) / (TY - 2),
            (g.Nk + kchunk - 1) / kchunk);
  const int src = ss.count == 0 ? 0 : (ss.count <= kFusedMaxFastSources ? 1 : 2);
#define FDTD_FUSED(APPS, DJ, SRC)                                                                 \
  fused_step<S, A, TY, APPS, DJ, SRC><<<grid, block, 0, stream>>>(g, st, out, cs, kchunk, J[0], \
                                                                  J[1], J[2], ss, step)
#define FDTD_FUSED_SRC(APPS, DJ)              \
  if (src == 0) FDTD_FUSED(APPS, DJ, 0);      \
  else if (src == 1) FDTD_FUSED(APPS, DJ, 1); \
  else FDTD_FUSED(APPS, DJ, 2);
  if (applications == 2) {
    if (dense_j) { FDTD_FUSED_SRC(2, true) } else { FDTD_FUSED_SRC(2, false) }
  } else {
    if (dense_j) { FDTD_FUSED_SRC(1, true) } else { FDTD_FUSED_SRC(1, false) }
  }
#undef FDTD_FUSED_SRC
#undef FDTD_FUSED
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_fused_f32(const Grid& g, const S& st, const S& out, const float* const J[3],
                             bool dense_j, const CoefSet& cs, const SourceSet& ss, int64_t step,
                             int applications, const FusedConfig& cfg, cudaStream_t stream) {
  const int kchunk = cfg.kchunk > 0 ? cfg.kchunk : 64;
  switch (cfg.tile_y) {
    case 8: return launch_fused_ty<S, 8>(g, st, out, J, dense_j, cs, ss, step, applications, kchunk, stream);
    default: return launch_fused_ty<S, 16>(g, st, out, J, dense_j, cs, ss, step, applications, kchunk, stream);
  }
}

#define FDTD_INSTANTIATE(S)                                                                         \
  template cudaError_t launch_b_f32<S>(const Grid&, const S&, const CoefSet&, int, cudaStream_t);  \
  template cudaError_t launch_e_f32<S>(const Grid&, const S&, const float* const[3], bool,         \
                                       const CoefSet&, const SourceSet&, int64_t, cudaStream_t);   \
  template cudaError_t launch_fused_f32<S>(const Grid&, const S&, const S&, const float* const[3], \
                                           bool,                                                   \
                                           const CoefSet&, const SourceSet&, int64_t, int,         \
                                           const FusedConfig&, cudaStream_t);
FDTD_INSTANTIATE(StoreF32)
FDTD_INSTANTIATE(StoreF32C)
FDTD_INSTANTIATE(StoreF16)
#undef FDTD_INSTANTIATE

}  // namespace fdtd
