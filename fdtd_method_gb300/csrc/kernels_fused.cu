// Fused step kernel of the FP32-arithmetic forms: one sweep per step.
//
// Between the first and the last B half step of a run the scheme is
//   E <- E + c curl B ;  B <- B + 2 (c/2) curl E
// (the trailing B half step of one update_fields and the leading one of the
// next see the same E), so one kernel does both updates on a tile of columns
// marching along z: 12 values move per cell-step (read E, B; write E, B),
// against 18 for the split sweeps of kernels_f32.cu, whose arithmetic it
// reproduces bit for bit.
//
// A CTA owns an interior tile of 64 x RY columns at (x0, y0) and marches the
// planes k0..k1 of its z chunk.  Each plane of all six components reaches
// shared memory as one TMA box per array (rows y0-1 .. y0+RY, columns
// x0-4 .. x0+67 of the FP32 words, x0-8 .. x0+71 of the BF16 lo words,
// x0-8 .. x0+71 of FP16 words), kStages planes ahead, through an mbarrier ring.
// Every thread owns two neighbouring x cells and works on both with packed
// float2 instructions (arith2.cuh).  Warps 0..RY are box rows 1..RY+1 (row
// RY+1 computes E' only, for its neighbours); warp RY+1 computes E' on column
// x0+64 (the x halo) for rows 1..RY.  In iteration t every thread
//   1. computes E'(t) = E + c curl B of its cells (B at i-1, j-1 from the
//      box, B(t-1) carried in registers);
//   2. computes B'(t-1) = B(t-1) + apps (c/2) curl E' on interior cells
//      (E'(t-1) at i+1, j+1 from shared memory, E'(t) in registers);
//   3. stores E'(t) (t < k1) and B'(t-1), publishes E'(t); the CTA
//      synchronises once and thread 0 refills the freed ring slot.
// The sweep reads the state from `st` and writes the new state to `out`:
// neighbouring tiles read what a tile writes, so an in-place update would race.
#include "arith2.cuh"
#include "engine_internal.h"
#include "sources.cuh"
#include "tma.cuh"

namespace fdtd {

namespace {

constexpr int kStages = 3;
constexpr int kTileX = 64;
constexpr int kLoOff = 8;  // BF16 lo box starts 8 columns left of the tile
constexpr int kEC = 68;  // columns of the E' exchange rows (64 + halo, padded)

template <class S> struct BoxOf;
template <> struct BoxOf<StoreF32> { static constexpr int kW = 72, kOff = 4, kLoW = 0; };
template <> struct BoxOf<StoreF32C> { static constexpr int kW = 72, kOff = 4, kLoW = 80; };
template <> struct BoxOf<StoreF16> { static constexpr int kW = 80, kOff = 8, kLoW = 0; };

template <class S, int RY>
struct SmemPlan {
  using HiT = typename Codec2<S>::HiT;
  static constexpr int ROWS = RY + 2;
  static constexpr int W = BoxOf<S>::kW;
  static constexpr int LW = BoxOf<S>::kLoW;
  static constexpr int NV = S::kComp ? 2 : 1;
  static constexpr int kHiBytes = 6 * ROWS * W * (int)sizeof(HiT);
  static constexpr int kLoBytes = 6 * ROWS * LW * (int)sizeof(LoT);
  static constexpr int kStageBytes = (kHiBytes + kLoBytes + 127) / 128 * 128;
  static constexpr int kEBytes = 2 * 3 * NV * ROWS * kEC * 4;
  static constexpr int kTotal = kStages * kStageBytes + kEBytes + kStages * 8;
  static constexpr uint32_t kTx = kHiBytes + kLoBytes;
};

template <class S> struct ArithFor { using type = ArithPlain; };
template <> struct ArithFor<StoreF32C> { using type = ArithComp; };

// Stores the pair of cells at (x, x+1) (x even; cell 1 only if in1) and
// their ghost copies.
template <class S>
__device__ __forceinline__ void store_pair(const S& st, const PLayout& L, int c, int x, int y, int z, P2 v,
                                           bool in1) {
  using C2 = Codec2<S>;
  auto put = [&](int yy) {
    if (in1) C2::store(st, c, L.at(x, yy, z), v);
    else st.store(c, L.at(x, yy, z), lane0(v));
  };
  put(y);
  const bool yl = (y == 0), yh = (y == L.Nj - 1);
  if (yl) put(L.Nj);
  if (yh) put(-1);
  // x ghosts: cell 0 may be x = 0 or Ni-1, cell 1 may be Ni-1
  if (x == 0 || x == L.Ni - 1) {
    const Pair a = lane0(v);
    const int xg = (x == 0) ? L.Ni : -1;
    st.store(c, L.at(xg, y, z), a);
    if (yl) st.store(c, L.at(xg, L.Nj, z), a);
    if (yh) st.store(c, L.at(xg, -1, z), a);
    if (x == 0 && x == L.Ni - 1) {  // Ni == 1: both ghost columns
      st.store(c, L.at(-1, y, z), a);
      if (yl) st.store(c, L.at(-1, L.Nj, z), a);
      if (yh) st.store(c, L.at(-1, -1, z), a);
    }
  }
  if (in1 && x + 1 == L.Ni - 1) {
    const Pair b = lane1(v);
    st.store(c, L.at(-1, y, z), b);
    if (yl) st.store(c, L.at(-1, L.Nj, z), b);
    if (yh) st.store(c, L.at(-1, -1, z), b);
  }
}

template <class S, class A, int RY, int kApps, bool kDenseJ, int kSrc>
__global__ void __launch_bounds__(32 * (RY + 2))
    fused2(PLayout L, S st, S out, const __grid_constant__ TmaMaps maps, CoefSet cs, int kchunk,
           const float* __restrict__ Jx, const float* __restrict__ Jy, const float* __restrict__ Jz,
           SourceSet ss, int64_t step, WaitCtl wc) {
  using SP = SmemPlan<S, RY>;
  using C2 = Codec2<S>;
  using A2 = Arith2<A>;
  using HiT = typename C2::HiT;
  using Raw = typename C2::Raw;
  using T = typename A::Cur;
  constexpr int ROWS = SP::ROWS, W = SP::W, LW = SP::LW, NV = SP::NV, OFF = BoxOf<S>::kOff;
  extern __shared__ __align__(128) unsigned char smem[];
  float* sE = reinterpret_cast<float*>(smem + kStages * SP::kStageBytes);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kStages * SP::kStageBytes + SP::kEBytes);

  const int lane = threadIdx.x, w = threadIdx.y;
  const int x0 = blockIdx.x * kTileX, y0 = blockIdx.y * RY;
  const int nx = min(kTileX, L.Ni - x0), ny = min(RY, L.Nj - y0);
  const bool halo = (w == RY + 1);
  const int r = halo ? lane + 1 : w + 1;  // box row
  const int c0 = halo ? kTileX : 2 * lane;  // tile column of the first cell
  const bool row_ok = halo ? (lane < ny && nx == kTileX) : (r <= ny + 1);
  const bool e0 = row_ok && c0 <= nx;
  const bool e1 = row_ok && !halo && c0 + 1 <= nx;
  const bool active = e0 || e1;
  const bool in0 = !halo && r <= ny && c0 < nx;
  const bool in1 = !halo && r <= ny && c0 + 1 < nx;
  const int xu = x0 + c0, yu = y0 + r - 1;  // unwrapped; x = Ni, y = Nj are ghost copies of 0
  const int xl0 = xu >= L.Ni ? xu - L.Ni : xu;
  const int xl1 = xu + 1 >= L.Ni ? xu + 1 - L.Ni : xu + 1;
  const int yl = yu >= L.Nj ? yu - L.Nj : yu;
  const int k0 = blockIdx.z * kchunk;
  const int k1 = min(k0 + kchunk, L.Nk);
  const bool producer = (w == 0 && lane == 0);

  int issued = 0;  // fills issued (the producer's count)
  auto issue = [&](int t) {
    if (wc.withhold) return;
    ++issued;
    const int slot = (t - k0) % kStages;
    const int kk = (t == L.Nk) ? 0 : t;
    unsigned char* base = smem + slot * SP::kStageBytes;
    mbar_arrive_expect_tx(&bar[slot], SP::kTx);
    for (int c = 0; c < 6; ++c)
      tma_load_3d(base + c * ROWS * W * sizeof(HiT), &maps.hi[c], x0 + kPadX - OFF, y0 - 1 + kPadY, kk, &bar[slot]);
    if (S::kComp)
      for (int c = 0; c < 6; ++c)
        tma_load_3d(base + SP::kHiBytes + c * ROWS * LW * sizeof(LoT), &maps.lo[c], x0 + kPadX - kLoOff, y0 - 1 + kPadY, kk,
                    &bar[slot]);
  };

  if (producer) {
    for (int s = 0; s < kStages; ++s) mbar_init(&bar[s], 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (producer)
    for (int t = k0; t <= k1 && t < k0 + kStages; ++t) issue(t);

  ColumnSources<A> src0, src1;
  if (kSrc == 1) {
    if (e0) src0.init(ss, xl0, yl, step, L);
    if (e1) src1.init(ss, xl1, yl, step, L);
  }

  const P2 zero{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
  P2 pbx = zero, pby = zero, pbz = zero, pex = zero, pey = zero, pez = zero;
  {
    // B(k0-1) of the cells that compute E' (x <= Ni, y <= Nj: cells or ghosts)
    const int kp = wrap_prev(k0, L.Nk);
    if (e0) {
      pbx.hi.x = st.load(3, L.at(xu, yu, kp)).hi;
      pbx.lo.x = st.load(3, L.at(xu, yu, kp)).lo;
      pby.hi.x = st.load(4, L.at(xu, yu, kp)).hi;
      pby.lo.x = st.load(4, L.at(xu, yu, kp)).lo;
    }
    if (e1) {
      pbx.hi.y = st.load(3, L.at(xu + 1, yu, kp)).hi;
      pbx.lo.y = st.load(3, L.at(xu + 1, yu, kp)).lo;
      pby.hi.y = st.load(4, L.at(xu + 1, yu, kp)).hi;
      pby.lo.y = st.load(4, L.at(xu + 1, yu, kp)).lo;
    }
  }

  // E' exchange: sE[buf][comp][v][row][col]
  auto se_at = [&](int buf, int c, int v, int row, int col) -> float* {
    return sE + ((((buf * 3 + c) * NV + v) * ROWS + row) * kEC + col);
  };
  auto se_get2 = [&](int buf, int c, int row, int col) -> P2 {
    const float2 h = *reinterpret_cast<const float2*>(se_at(buf, c, 0, row, col));
    const float2 l = NV == 2 ? *reinterpret_cast<const float2*>(se_at(buf, c, NV - 1, row, col)) : make_float2(0.f, 0.f);
    return P2{h, l};
  };
  auto se_get1 = [&](int buf, int c, int row, int col) -> Pair {
    return Pair{*se_at(buf, c, 0, row, col), NV == 2 ? *se_at(buf, c, NV - 1, row, col) : 0.f};
  };

  for (int t = k0; t <= k1; ++t) {
    const int slot = (t - k0) % kStages;
    const int cur = t & 1;
    const bool timed_out = !mbar_wait_bounded(&bar[slot], ((t - k0) / kStages) & 1, wc);
    const HiT* H = reinterpret_cast<const HiT*>(smem + slot * SP::kStageBytes);
    const LoT* Lo = reinterpret_cast<const LoT*>(smem + slot * SP::kStageBytes + SP::kHiBytes);
    auto ld2 = [&](int c, int row, int col) -> P2 {  // cells col, col+1 (col even)
      const Raw h = *reinterpret_cast<const Raw*>(H + (c * ROWS + row) * W + col + OFF);
      const uint32_t q = S::kComp ? *reinterpret_cast<const uint32_t*>(Lo + (c * ROWS + row) * LW + col + kLoOff) : 0u;
      return C2::decode(st, c, h, q);
    };
    auto ld1 = [&](int c, int row, int col) -> Pair {
      const HiT h = H[(c * ROWS + row) * W + col + OFF];
      const LoT q = S::kComp ? Lo[(c * ROWS + row) * LW + col + kLoOff] : LoT(0);
      return st.decode(c, h, q);
    };

    P2 bx = zero, by = zero, bz = zero, nex = zero, ney = zero, nez = zero;
    if (active) {
      const int kk = (t == L.Nk) ? 0 : t;
      bx = ld2(3, r, c0);
      by = ld2(4, r, c0);
      bz = ld2(5, r, c0);
      const P2 ex = ld2(0, r, c0), ey = ld2(1, r, c0), ez = ld2(2, r, c0);
      const P2 bz_jp = ld2(5, r - 1, c0), bx_jp = ld2(3, r - 1, c0);
      const P2 bz_ip = make_p2(ld1(5, r, c0 - 1), lane0(bz));
      const P2 by_ip = make_p2(ld1(4, r, c0 - 1), lane0(by));
      P2 qx = A2::curl(bcast(ecoef<S>(cs, st, 0, 0)), bz, bz_jp, bcast(ecoef<S>(cs, st, 0, 1)), by, pby);
      P2 qy = A2::curl(bcast(ecoef<S>(cs, st, 1, 0)), bx, pbx, bcast(ecoef<S>(cs, st, 1, 1)), bz, bz_ip);
      P2 qz = A2::curl(bcast(ecoef<S>(cs, st, 2, 0)), by, by_ip, bcast(ecoef<S>(cs, st, 2, 1)), bx, bx_jp);
      if (kDenseJ || kSrc != 0) {
        T j0[3] = {A::cur_zero(), A::cur_zero(), A::cur_zero()};
        T j1[3] = {A::cur_zero(), A::cur_zero(), A::cur_zero()};
        unsigned h0 = 0, h1 = 0;
        if (kDenseJ) {
          const int64_t plane = (int64_t)kk * L.Ni * L.Nj, row = (int64_t)yl * L.Ni;
          const int64_t d0 = xl0 + row + plane, d1 = xl1 + row + plane;
          if (e0) {
            j0[0] = A::cur_dense(Jx[d0]);
            j0[1] = A::cur_dense(Jy[d0]);
            j0[2] = A::cur_dense(Jz[d0]);
            h0 = 7u;
          }
          if (e1) {
            j1[0] = A::cur_dense(Jx[d1]);
            j1[1] = A::cur_dense(Jy[d1]);
            j1[2] = A::cur_dense(Jz[d1]);
            h1 = 7u;
          }
        }
        if (kSrc == 1) {
          if (e0) h0 |= src0.eval(ss, kk, L, j0, h0);
          if (e1) h1 |= src1.eval(ss, kk, L, j1, h1);
        } else if (kSrc == 2) {
          if (e0) h0 |= source_sum<A>(ss, step, xl0, yl, kk, L, j0, h0);
          if (e1) h1 |= source_sum<A>(ss, step, xl1, yl, kk, L, j1, h1);
        }
        if (h0 || h1) {
          // per lane, exactly the one-cell update: add cJ J only where current flows
          P2* q[3] = {&qx, &qy, &qz};
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const Pair t0 = A::cur_term(jcoef<S>(cs, st, c), j0[c]), t1 = A::cur_term(jcoef<S>(cs, st, c), j1[c]);
            const P2 s = A2::add(*q[c], make_p2(t0, t1));
            if (h0 >> c & 1u) {
              q[c]->hi.x = s.hi.x;
              q[c]->lo.x = s.lo.x;
            }
            if (h1 >> c & 1u) {
              q[c]->hi.y = s.hi.y;
              q[c]->lo.y = s.lo.y;
            }
          }
        }
      }
      // E' as its storage form will hold it (what the split sweeps reload).
      nex = C2::quantize(st, 0, A2::acc(ex, qx));
      ney = C2::quantize(st, 1, A2::acc(ey, qy));
      nez = C2::quantize(st, 2, A2::acc(ez, qz));

      if (in0 && t > k0) {
        const int prv = cur ^ 1;
        const P2 ez_jn = se_get2(prv, 2, r + 1, c0), ex_jn = se_get2(prv, 0, r + 1, c0);
        const P2 ez_in = make_p2(lane1(pez), se_get1(prv, 2, r, c0 + 2));
        const P2 ey_in = make_p2(lane1(pey), se_get1(prv, 1, r, c0 + 2));
        P2 ux = A2::curl(bcast(bcoef<S>(cs, st, 0, 0)), ney, pey, bcast(bcoef<S>(cs, st, 0, 1)), ez_jn, pez);
        P2 uy = A2::curl(bcast(bcoef<S>(cs, st, 1, 0)), ez_in, pez, bcast(bcoef<S>(cs, st, 1, 1)), nex, pex);
        P2 uz = A2::curl(bcast(bcoef<S>(cs, st, 2, 0)), ex_jn, pex, bcast(bcoef<S>(cs, st, 2, 1)), ey_in, pey);
        if (kApps == 2) {
          ux = A2::twice(ux);
          uy = A2::twice(uy);
          uz = A2::twice(uz);
        }
        store_pair(out, L, 3, xu, yu, t - 1, A2::acc(pbx, ux), in1);
        store_pair(out, L, 4, xu, yu, t - 1, A2::acc(pby, uy), in1);
        store_pair(out, L, 5, xu, yu, t - 1, A2::acc(pbz, uz), in1);
      }
      if (in0 && t < k1) {
        store_pair(out, L, 0, xu, yu, t, nex, in1);
        store_pair(out, L, 1, xu, yu, t, ney, in1);
        store_pair(out, L, 2, xu, yu, t, nez, in1);
      }
      const P2* ne[3] = {&nex, &ney, &nez};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        *reinterpret_cast<float2*>(se_at(cur, c, 0, r, c0)) = ne[c]->hi;
        if (NV == 2) *reinterpret_cast<float2*>(se_at(cur, c, NV - 1, r, c0)) = ne[c]->lo;
      }
    }
    pbx = bx;
    pby = by;
    pbz = bz;
    pex = nex;
    pey = ney;
    pez = nez;
    if (__syncthreads_or(timed_out)) {
      // a wait gave up: stop, after the producer has waited (bounded) for the
      // fills still in flight
      if (producer)
        for (int f = t - k0; f < issued; ++f) mbar_wait_bounded(&bar[f % kStages], (f / kStages) & 1, wc, 2);
      return;
    }
    if (producer && t + kStages <= k1) issue(t + kStages);
  }
}

template <class S, int RY, int APPS, bool DJ, int SRC>
cudaError_t launch_one(dim3 grid, const PLayout& L, const S& st, const S& out, const TmaMaps& maps,
                       const CoefSet& cs, int kchunk, const float* const J[3], const SourceSet& ss,
                       int64_t step, const WaitCtl& wc, cudaStream_t stream) {
  using A = typename ArithFor<S>::type;
  auto kern = fused2<S, A, RY, APPS, DJ, SRC>;
  const int bytes = SmemPlan<S, RY>::kTotal;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  kern<<<grid, dim3(32, RY + 2), bytes, stream>>>(L, st, out, maps, cs, kchunk, J[0], J[1], J[2], ss, step,
                                                  wc);
  return cudaGetLastError();
}

template <class S, int RY>
cudaError_t launch_ry(const PLayout& L, const S& st, const S& out, const TmaMaps& maps,
                      const float* const J[3], bool dense_j, const CoefSet& cs, const SourceSet& ss,
                      int64_t step, int applications, int kchunk, const WaitCtl& wc, cudaStream_t stream) {
  dim3 grid((L.Ni + kTileX - 1) / kTileX, (L.Nj + RY - 1) / RY, (L.Nk + kchunk - 1) / kchunk);
  const int src = ss.count == 0 ? 0 : (ss.count <= kFastSources ? 1 : 2);
#define FDTD_F(APPS, DJ, SRC) \
  return launch_one<S, RY, APPS, DJ, SRC>(grid, L, st, out, maps, cs, kchunk, J, ss, step, wc, stream)
#define FDTD_FS(APPS, DJ)            \
  if (src == 0) FDTD_F(APPS, DJ, 0); \
  if (src == 1) FDTD_F(APPS, DJ, 1); \
  FDTD_F(APPS, DJ, 2);
  if (applications == 2) {
    if (dense_j) { FDTD_FS(2, true) } else { FDTD_FS(2, false) }
  } else {
    if (dense_j) { FDTD_FS(1, true) } else { FDTD_FS(1, false) }
  }
#undef FDTD_FS
#undef FDTD_F
}

}  // namespace

template <class S>
cudaError_t launch_fused_f32(const PLayout& L, const S& st, const S& out, const void* maps,
                             const float* const J[3], bool dense_j, const CoefSet& cs,
                             const SourceSet& ss, int64_t step, int applications,
                             const FusedConfig& cfg, const WaitCtl& wc, cudaStream_t stream) {
  const int kchunk = cfg.kchunk > 0 ? cfg.kchunk : 32;
  const TmaMaps& m = *static_cast<const TmaMaps*>(maps);
  if (cfg.tile_y == 6)
    return launch_ry<S, 6>(L, st, out, m, J, dense_j, cs, ss, step, applications, kchunk, wc, stream);
  return launch_ry<S, 14>(L, st, out, m, J, dense_j, cs, ss, step, applications, kchunk, wc, stream);
}

template <class S>
int fused_box_width() { return BoxOf<S>::kW; }
int fused_lo_box_width() { return BoxOf<StoreF32C>::kLoW; }

#define FDTD_INSTANTIATE(S)                                                                          \
  template cudaError_t launch_fused_f32<S>(const PLayout&, const S&, const S&, const void*,         \
                                           const float* const[3], bool, const CoefSet&,             \
                                           const SourceSet&, int64_t, int, const FusedConfig&,      \
                                           const WaitCtl&,                                          \
                                           cudaStream_t);                                           \
  template int fused_box_width<S>();
FDTD_INSTANTIATE(StoreF32)
FDTD_INSTANTIATE(StoreF32C)
FDTD_INSTANTIATE(StoreF16)
#undef FDTD_INSTANTIATE

}  // namespace fdtd
