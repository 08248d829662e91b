// Fused step kernel, one cell per thread (the variant for storage forms whose
// arithmetic is light enough that occupancy matters more than packed math).
// Same algorithm and results as kernels_fused.cu (two cells per thread); see
// there for the description of the sweep.  Tiles are 32 x RY cells (RY = 6,
// 14 or 30; 30 makes a 1024-thread CTA, one per SM).
#include "arith.cuh"
#include "engine_internal.h"
#include "sources.cuh"
#include "tma.cuh"

namespace fdtd {

template <class S> struct ArithOf1 { using type = ArithPlain; };
template <> struct ArithOf1<StoreF32C> { using type = ArithComp; };

template <class A>
__device__ __forceinline__ Pair curl_term(Coef c1, Pair a1, Pair b1, Coef c2, Pair a2, Pair b2) {
  return A::curl(c1, a1, b1, c2, a2, b2);
}

// Fused pipeline.
//
// A CTA owns an interior tile of 32 x RY columns at (x0, y0) and marches the
// planes k0..k1 of its z chunk, reading each plane of all six components as
// one TMA box per array (rows y0-1 .. y0+RY, columns x0-4 .. x0+35 for FP32
// words, x0-8 .. x0+39 for the BF16 lo words, x0-8 .. x0+39 for FP16),
// NS planes ahead through an mbarrier ring.  Warps 0..RY are rows 1..RY+1 of
// the box (row RY+1 computes E' only, for its neighbours); warp RY+1 computes
// E' on column x0+nx (the x halo) for rows 1..RY.  In iteration t every
// thread
//   1. computes E'(t) = E + c curl B of its cell (B at i-1, j-1 from the
//      box, B(t-1) carried in registers);
//   2. computes B'(t-1) = B(t-1) + apps (c/2) curl E' (E'(t-1) at i+1, j+1
//      from shared memory, E'(t) in registers) on interior cells;
//   3. stores E'(t) (t < k1) and B'(t-1), publishes E'(t), and the CTA
//      synchronises once; thread 0 then refills the freed ring slot.
// The sweep reads the state from `st` and writes the new state to `out`:
// neighbouring tiles read what a tile writes, so an in-place update would race.

constexpr int kStages1 = 3;

template <class S> struct Box1;
template <> struct Box1<StoreF32> { static constexpr int kW = 40, kOff = 4, kLoW = 0; };
template <> struct Box1<StoreF32C> { static constexpr int kW = 40, kOff = 4, kLoW = 48; };
template <> struct Box1<StoreF16> { static constexpr int kW = 48, kOff = 8, kLoW = 0; };
constexpr int kLoOff1 = 8;  // BF16 lo box starts 8 columns left of the tile

template <class S, int RY>
struct Smem1 {
  using HiT = typename S::HiT;
  static constexpr int ROWS = RY + 2;
  static constexpr int W = Box1<S>::kW;
  static constexpr int LW = Box1<S>::kLoW;
  static constexpr int NV = S::kComp ? 2 : 1;
  static constexpr int kHiBytes = 6 * ROWS * W * (int)sizeof(HiT);
  static constexpr int kLoBytes = 6 * ROWS * LW * (int)sizeof(LoT);
  static constexpr int kStageBytes = (kHiBytes + kLoBytes + 127) / 128 * 128;
  static constexpr int kEBytes = 2 * 3 * NV * ROWS * 33 * 4;
  static constexpr int kTotal = kStages1 * kStageBytes + kEBytes + kStages1 * 8;
  static constexpr uint32_t kTx = kHiBytes + kLoBytes;
};

template <class S, class A, int RY, int kApps, bool kDenseJ, int kSrc>
__global__ void __launch_bounds__(32 * (RY + 2))
    fused1(PLayout L, S st, S out, const __grid_constant__ TmaMaps maps, CoefSet cs, int kchunk,
              const float* __restrict__ Jx, const float* __restrict__ Jy,
              const float* __restrict__ Jz, SourceSet ss, int64_t step, int* err) {
  using SM = Smem1<S, RY>;
  using HiT = typename S::HiT;
  using T = typename A::Cur;
  constexpr int ROWS = SM::ROWS, W = SM::W, LW = SM::LW, NV = SM::NV, OFF = Box1<S>::kOff;
  constexpr int NS = kStages1;
  constexpr int EC = 33;  // columns of the E' exchange (32 interior + the x halo)
  extern __shared__ __align__(128) unsigned char smem[];
  float* sE = reinterpret_cast<float*>(smem + NS * SM::kStageBytes);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + NS * SM::kStageBytes + SM::kEBytes);
  auto hi_of = [&](int slot) { return reinterpret_cast<const HiT*>(smem + slot * SM::kStageBytes); };
  auto lo_of = [&](int slot) {
    return reinterpret_cast<const LoT*>(smem + slot * SM::kStageBytes + SM::kHiBytes);
  };
  // sE[buf][c][v][row][col]
  auto se = [&](int buf, int c, int v, int row, int col) -> float& {
    return sE[(((buf * 3 + c) * NV + v) * ROWS + row) * EC + col];
  };

  const int lane = threadIdx.x, w = threadIdx.y;
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * RY;
  const int nx = min(32, L.Ni - x0), ny = min(RY, L.Nj - y0);
  const bool halo = (w == RY + 1);
  const int r = halo ? lane + 1 : w + 1;   // box row
  const int cx = halo ? nx : lane;          // column within the tile (0..32)
  const bool active = halo ? (lane < ny) : (r <= ny + 1 && lane < nx);
  const bool interior = !halo && r <= ny && lane < nx;
  // logical coordinates of the cell (x = Ni and y = Nj are the ghost copies of 0)
  const int xu = x0 + cx, yu = y0 + r - 1;
  const int xl = xu >= L.Ni ? xu - L.Ni : xu, yl = yu >= L.Nj ? yu - L.Nj : yu;
  const int k0 = blockIdx.z * kchunk;
  const int k1 = min(k0 + kchunk, L.Nk);
  const bool producer = (w == 0 && lane == 0);

  auto issue = [&](int t) {
    const int slot = (t - k0) % NS;
    const int kk = (t == L.Nk) ? 0 : t;
    unsigned char* base = smem + slot * SM::kStageBytes;
    mbar_arrive_expect_tx(&bar[slot], SM::kTx);
    for (int c = 0; c < 6; ++c)
      tma_load_3d(base + c * ROWS * W * sizeof(HiT), &maps.hi[c], x0 + kPadX - OFF, y0, kk, &bar[slot]);
    if (S::kComp)
      for (int c = 0; c < 6; ++c)
        tma_load_3d(base + SM::kHiBytes + c * ROWS * LW * sizeof(LoT), &maps.lo[c], x0 + kPadX - kLoOff1, y0, kk,
                    &bar[slot]);
  };

  if (producer) {
    for (int s = 0; s < NS; ++s) mbar_init(&bar[s], 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (producer)
    for (int t = k0; t <= k1 && t < k0 + NS; ++t) issue(t);

  // Sources: per-column factor (amp gx) gy, once per launch.
  T sxy[kFastSources];
  unsigned smask = 0;
#pragma unroll
  for (int q = 0; q < kFastSources; ++q) sxy[q] = A::cur_zero();
  if (kSrc == 1 && active) {
#pragma unroll
    for (int q = 0; q < kFastSources; ++q) {
      if (q < ss.count) {
        const DevSource& d = ss.src[q];
        const int di = box_offset(xl, d.i0, d.ni, L.Ni);
        const int dj = box_offset(yl, d.j0, d.nj, L.Nj);
        if (step < d.n_amp && di >= 0 && dj >= 0) {
          sxy[q] = A::cur_mul(A::cur_mul(A::cur_table(ss, d.amp_off + step), A::cur_table(ss, d.gx_off + di)),
                              A::cur_table(ss, d.gy_off + dj));
          smask |= 1u << q;
        }
      }
    }
  }

  Pair pbx{0.f, 0.f}, pby{0.f, 0.f}, pbz{0.f, 0.f};
  Pair pex{0.f, 0.f}, pey{0.f, 0.f}, pez{0.f, 0.f};
  if (active) {
    const int64_t b0 = L.at(xu, yu, wrap_prev(k0, L.Nk));
    pbx = st.load(3, b0);
    pby = st.load(4, b0);
  }

  // Output of an interior cell: its own position and, on the grid's edges,
  // its ghost copies.
  const int64_t obase = L.at(xl, yl, 0);
  const bool edge = interior && (xl == 0 || xl == L.Ni - 1 || yl == 0 || yl == L.Nj - 1);
  auto put = [&](int c, int z, Pair v) {
    out.store(c, obase + (int64_t)z * L.pplane, v);
    if (edge) store_ghost_copies(out, L, c, xl, yl, z, v);
  };

  int slot = 0;
  uint32_t phase = 0;
  for (int t = k0; t <= k1; ++t) {
    const int cur = t & 1;
    mbar_wait_bounded(&bar[slot], phase, err);
    const HiT* H = hi_of(slot);
    const LoT* Lo = lo_of(slot);
    auto val = [&](int c, int row, int col) -> Pair {
      const HiT h = H[(c * ROWS + row) * W + col + OFF];
      const LoT q = S::kComp ? Lo[(c * ROWS + row) * LW + col + kLoOff1] : LoT(0);
      return st.decode(c, h, q);
    };

    Pair bx{0.f, 0.f}, by{0.f, 0.f}, bz{0.f, 0.f}, nex{0.f, 0.f}, ney{0.f, 0.f}, nez{0.f, 0.f};
    if (active) {
      const int kk = (t == L.Nk) ? 0 : t;
      bx = val(3, r, cx);
      by = val(4, r, cx);
      bz = val(5, r, cx);
      const Pair ex = val(0, r, cx), ey = val(1, r, cx), ez = val(2, r, cx);
      Pair qx = curl_term<A>(cs.ce[1], bz, val(5, r - 1, cx), cs.ce[2], by, pby);
      Pair qy = curl_term<A>(cs.ce[2], bx, pbx, cs.ce[0], bz, val(5, r, cx - 1));
      Pair qz = curl_term<A>(cs.ce[0], by, val(4, r, cx - 1), cs.ce[1], bx, val(3, r - 1, cx));
      T jv[3] = {A::cur_zero(), A::cur_zero(), A::cur_zero()};
      bool has_j = false;
      if (kDenseJ) {
        const int64_t d = xl + (int64_t)yl * L.Ni + (int64_t)kk * L.Ni * L.Nj;
        jv[0] = A::cur_dense(Jx[d]);
        jv[1] = A::cur_dense(Jy[d]);
        jv[2] = A::cur_dense(Jz[d]);
        has_j = true;
      }
      if (kSrc == 1) {
#pragma unroll
        for (int q = 0; q < kFastSources; ++q) {
          if (smask & (1u << q)) {
            const DevSource& d = ss.src[q];
            const int dk = box_offset(kk, d.k0, d.nk, L.Nk);
            if (dk >= 0) {
              add_current<A>(jv, d.comp_mask, A::cur_mul(sxy[q], A::cur_table(ss, d.gz_off + dk)));
              has_j = true;
            }
          }
        }
      } else if (kSrc == 2) {
        has_j |= source_sum<A>(ss, step, xl, yl, kk, L, jv);
      }
      if (has_j) {
        qx = A::add(qx, A::cur_term(cs.cj, jv[0]));
        qy = A::add(qy, A::cur_term(cs.cj, jv[1]));
        qz = A::add(qz, A::cur_term(cs.cj, jv[2]));
      }
      // E' as its storage form will hold it (what the split sweeps reload).
      nex = st.quantize(0, A::acc(ex, qx));
      ney = st.quantize(1, A::acc(ey, qy));
      nez = st.quantize(2, A::acc(ez, qz));

      if (interior && t > k0) {
        const int prv = cur ^ 1;
        auto eget = [&](int c, int row, int col) {
          return Pair{se(prv, c, 0, row, col), NV == 2 ? se(prv, c, NV - 1, row, col) : 0.f};
        };
        Pair ux = curl_term<A>(cs.cb[2], ney, pey, cs.cb[1], eget(2, r + 1, cx), pez);
        Pair uy = curl_term<A>(cs.cb[0], eget(2, r, cx + 1), pez, cs.cb[2], nex, pex);
        Pair uz = curl_term<A>(cs.cb[1], eget(0, r + 1, cx), pex, cs.cb[0], eget(1, r, cx + 1), pey);
        if (kApps == 2) {
          ux = A::twice(ux);
          uy = A::twice(uy);
          uz = A::twice(uz);
        }
        put(3, t - 1, A::acc(pbx, ux));
        put(4, t - 1, A::acc(pby, uy));
        put(5, t - 1, A::acc(pbz, uz));
      }
      if (interior && t < k1) {
        put(0, t, nex);
        put(1, t, ney);
        put(2, t, nez);
      }
      se(cur, 0, 0, r, cx) = nex.hi;
      se(cur, 1, 0, r, cx) = ney.hi;
      se(cur, 2, 0, r, cx) = nez.hi;
      if (NV == 2) {
        se(cur, 0, NV - 1, r, cx) = nex.lo;
        se(cur, 1, NV - 1, r, cx) = ney.lo;
        se(cur, 2, NV - 1, r, cx) = nez.lo;
      }
    }
    pbx = bx;
    pby = by;
    pbz = bz;
    pex = nex;
    pey = ney;
    pez = nez;
    __syncthreads();
    if (producer && t + NS <= k1) issue(t + NS);
    if (++slot == NS) {
      slot = 0;
      phase ^= 1u;
    }
  }
}

// ---------------------------------------------------------------------------

template <class S, int RY, int APPS, bool DJ, int SRC>
static cudaError_t launch1_one(dim3 grid, const PLayout& L, const S& st, const S& out,
                                    const TmaMaps& maps, const CoefSet& cs, int kchunk,
                                    const float* const J[3], const SourceSet& ss, int64_t step,
                                    int* err, cudaStream_t stream) {
  using A = typename ArithOf1<S>::type;
  auto kern = fused1<S, A, RY, APPS, DJ, SRC>;
  const int bytes = Smem1<S, RY>::kTotal;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  kern<<<grid, dim3(32, RY + 2), bytes, stream>>>(L, st, out, maps, cs, kchunk, J[0], J[1], J[2], ss,
                                                  step, err);
  return cudaGetLastError();
}

template <class S, int RY>
static cudaError_t launch1_ry(const PLayout& L, const S& st, const S& out, const TmaMaps& maps,
                                   const float* const J[3], bool dense_j, const CoefSet& cs,
                                   const SourceSet& ss, int64_t step, int applications, int kchunk,
                                   int* err, cudaStream_t stream) {
  dim3 grid((L.Ni + 31) / 32, (L.Nj + RY - 1) / RY, (L.Nk + kchunk - 1) / kchunk);
  const int src = ss.count == 0 ? 0 : (ss.count <= kFastSources ? 1 : 2);
#define FDTD_F(APPS, DJ, SRC) \
  return launch1_one<S, RY, APPS, DJ, SRC>(grid, L, st, out, maps, cs, kchunk, J, ss, step, err, stream)
#define FDTD_FS(APPS, DJ)        \
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

template <class S>
cudaError_t launch_fused1_f32(const PLayout& L, const S& st, const S& out, const void* maps,
                             const float* const J[3], bool dense_j, const CoefSet& cs,
                             const SourceSet& ss, int64_t step, int applications,
                             const FusedConfig& cfg, int* err, cudaStream_t stream) {
  const int kchunk = cfg.kchunk > 0 ? cfg.kchunk : 32;
  const TmaMaps& m = *static_cast<const TmaMaps*>(maps);
  if (cfg.tile_y == 6)
    return launch1_ry<S, 6>(L, st, out, m, J, dense_j, cs, ss, step, applications, kchunk, err, stream);
  if (cfg.tile_y == 30)
    return launch1_ry<S, 30>(L, st, out, m, J, dense_j, cs, ss, step, applications, kchunk, err, stream);
  return launch1_ry<S, 14>(L, st, out, m, J, dense_j, cs, ss, step, applications, kchunk, err, stream);
}


template <class S>
int fused1_box_width() { return Box1<S>::kW; }
int fused1_lo_box_width() { return Box1<StoreF32C>::kLoW; }

#define FDTD_INSTANTIATE(S)                                                                           \
  template cudaError_t launch_fused1_f32<S>(const PLayout&, const S&, const S&, const void*,         \
                                            const float* const[3], bool, const CoefSet&,             \
                                            const SourceSet&, int64_t, int, const FusedConfig&, int*, \
                                            cudaStream_t);                                           \
  template int fused1_box_width<S>();
FDTD_INSTANTIATE(StoreF32)
FDTD_INSTANTIATE(StoreF32C)
FDTD_INSTANTIATE(StoreF16)
#undef FDTD_INSTANTIATE

}  // namespace fdtd
