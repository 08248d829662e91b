// Fused step kernel, one cell per thread: the default step of the
// FP32-arithmetic forms.  One sweep advances one update_fields step; the
// arithmetic is that of the split sweeps (kernels_f32.cu, the reference's
// functors kokkos_functors.h:64-90 E and :128-151 B), reproduced bit for bit.
// The sweep is B-first: `apps` B half steps (the trailing half of the
// previous step, which was left pending, and the leading half of this one),
// then the E step, marching z downward.  A run of n steps is n of these with
// the last trailing half left pending; every reader of B applies it
// (engine.cu), so n update_fields calls cost n sweeps.  It adds the same
// terms in the same order as the split sweeps (and the two-cell E-first
// kernel, kernels_fused.cu), so all agree bit for bit.
//
// A CTA owns a tile of 32 x RY cells at (x0, y0) (RY = 6, 14 or 30) and
// marches the planes of its z chunk.  Warps 0..RY-1 are the tile rows; warps
// RY and RY+1 compute B' on the tile's halo row and halo column (the row
// below and the column left of the tile, which the E update reads at j-1 and
// i-1).
//
// Data movement, per plane:
//   in   one 3-D TMA box per stored array (hi words: columns x0-4 .. x0+35,
//        BF16 lo and FP16 words: x0-8 .. x0+39; each component's rows are the
//        ones its stencil reads), NS planes ahead through an mbarrier ring;
//   out  both updated fields are written to shared staging boxes of 32 x RY
//        in their stored encoding; one thread stores them with TMA through
//        tensor maps of the grid rows (the copy engine clips rows past the
//        grid; a tile narrower than 32 columns stores with plain stores).
//        The first and last tile columns store the same boxes into the x
//        margins as well, which fills the ghost columns with bulk copies
//        where the alignment allows; the remaining ghost copies (ghost
//        rows, corners, unaligned columns) are plain stores.
// The B' staging box doubles as the exchange plane from which the next
// iteration reads B' at the tile's neighbouring cells; it has two extra
// rows, holding the halo row's and the halo column's values.
//
// Iteration t (planes k1-1 down to k0-1):
//   1. B'(t) = B + apps (c/2) curl E of the thread's cell (E at i+1, j+1 from
//      the box, E(t+1) carried in registers);
//   2. on interior cells (t < k1-1), E'(t+1) = E(t+1) + c curl B' + J
//      (B'(t+1) at i-1, j-1 from the exchange plane, B'(t) in registers).
// Each iteration ends with one CTA barrier; lane 0 of the halo-column warp
// then stores the staged boxes and refills the freed ring slot.
// The sweep reads the state from `st` and writes the new state to `out`:
// neighbouring tiles read what a tile writes, so an in-place update would race.
#include "arith.cuh"
#include "engine_internal.h"
#include "sources.cuh"
#include "tma.cuh"

#include <type_traits>

namespace fdtd {

template <class S> struct ArithOf1 { using type = ArithPlain; };
template <> struct ArithOf1<StoreF32C> { using type = ArithComp; };

// Ring stages per storage form.  Three for the FP32 words (the compensated
// form's 21.6 KB stages of a 14-row tile leave room for no more at two CTAs
// per SM; plain FP32 measured 1-14 % slower with four or six), four for the
// FP16 words (8 KB stages; 0.8 % faster than three, and flat up to eight).
template <class S>
constexpr int kStages1 = sizeof(typename S::HiT) == 2 ? 4 : 3;
constexpr int kLoOff1 = 8;  // BF16 lo boxes start 8 columns left of the tile

// Box widths (elements) and the left offset of the boxes that hold the
// column left of the tile.  kW / kLoW reach the column right of the tile
// (x0+32); the B-first sweep's Ex and B boxes need no column right of the
// tile and take the narrower kWs / kLoWs (one 32-byte sector less per row).
// Every start and width keeps rows on 16-byte boundaries.
template <class S> struct Box1;
template <> struct Box1<StoreF32> { static constexpr int kW = 40, kWs = 36, kOff = 4, kLoW = 0, kLoWs = 0; };
template <> struct Box1<StoreF32C> { static constexpr int kW = 40, kWs = 36, kOff = 4, kLoW = 48, kLoWs = 40; };
template <> struct Box1<StoreF16> { static constexpr int kW = 48, kWs = 40, kOff = 8, kLoW = 0, kLoWs = 0; };

constexpr int round128(int b) { return (b + 127) / 128 * 128; }

// A field component as a compile-time constant, and a loop over the six.
template <int c>
using Comp = std::integral_constant<int, c>;
template <class F>
__device__ __forceinline__ void for_each_comp(F&& f) {
  f(Comp<0>{});
  f(Comp<1>{});
  f(Comp<2>{});
  f(Comp<3>{});
  f(Comp<4>{});
  f(Comp<5>{});
}

// CTAs per SM the register budget is sized for: one 1024-thread CTA for
// 30-row tiles, otherwise two; three for the step sweep of FP16 words in
// 14-row tiles (40 registers and about 100 bytes of spill, but 48 warps per
// SM to cover the issue-bound loop: 0.826 against 0.926 ms at 512^3; four
// CTAs, or three for FP32 words, ran 10-27 % slower).
template <int RY, class S = void>
constexpr int kMinCtas1 = RY == 30 ? 1 : (std::is_same<S, StoreF16>::value && RY == 14 ? 3 : 2);

// Ring-stage layout of the per-component tile boxes (see Plan1): byte offset
// of each hi and lo box, box rows, first box row and x shift per component.
// Computed once at compile time into a table, so that every shared-memory
// offset in the kernel folds to an immediate.
struct BoxTable {
  int hi[7], lo[7];    // byte offsets ([6]: end of the hi / lo boxes)
  int rows[6], row0[6], xoff[6], lxoff[6];
  int w[6], lw[6];     // box widths (elements)
  unsigned tx;         // bytes the six (twelve) copies write
  int stage;           // stage size, 128-byte multiple
};

constexpr BoxTable box_table(int RY, int W, int Ws, int LW, int LWs, int HS, int LS, bool lo, int off, int lo_off) {
  BoxTable b{};
  int at = 0;
  unsigned tx = 0;
  for (int c = 0; c < 6; ++c) {
    // every box starts at the row below and the column left of the tile
    // (the halo warps' cells); Ex and Ez also hold the row above (B'z and
    // B'x read them at j+1), Ey and Ez the column right of it (B'z and B'y
    // read them at i+1).  Box row 0 is y0-1.
    b.rows[c] = (c == 0 || c == 2) ? RY + 2 : RY + 1;
    b.row0[c] = 0;
    b.xoff[c] = off;
    b.lxoff[c] = lo_off;
    const bool right = (c == 1 || c == 2);
    b.w[c] = right ? W : Ws;
    b.lw[c] = right ? LW : LWs;
  }
  for (int c = 0; c < 6; ++c) {
    b.hi[c] = at;
    at = (at + b.rows[c] * b.w[c] * HS + 127) / 128 * 128;
    tx += (unsigned)(b.rows[c] * b.w[c] * HS);
  }
  b.hi[6] = at;
  for (int c = 0; c < 6; ++c) {
    b.lo[c] = at;
    if (lo) {
      at = (at + b.rows[c] * b.lw[c] * LS + 127) / 128 * 128;
      tx += (unsigned)(b.rows[c] * b.lw[c] * LS);
    }
  }
  b.lo[6] = at;
  b.tx = tx;
  b.stage = at;
  return b;
}

// Shared-memory plan (byte offsets) of the sweep.
template <class S, int RY>
struct Plan1 {
  using HiT = typename S::HiT;
  static constexpr bool kLo = S::kComp;
  static constexpr int ROWS = RY + 2;
  static constexpr int W = Box1<S>::kW, LW = Box1<S>::kLoW, OFF = Box1<S>::kOff;
  static constexpr int Ws = Box1<S>::kWs, LWs = Box1<S>::kLoWs;
  static constexpr int HS = (int)sizeof(HiT), LS = (int)sizeof(LoT);
  // Ring stage: 6 hi boxes, then 6 lo boxes.  Each component's box holds
  // only the halos its stencil reads (box_table).  Every box starts on a
  // 128-byte boundary, as tensor copies require.
  // Per-component scalars of the table (device code may use scalar
  // constants, not the table object).
  static constexpr BoxTable box() { return box_table(RY, W, Ws, LW, LWs, HS, LS, kLo, OFF, kLoOff1); }
  template <int c> static constexpr int kHiAt = box().hi[c];
  template <int c> static constexpr int kLoAt = box().lo[c];
  template <int c> static constexpr int kRow0 = box().row0[c];
  template <int c> static constexpr int kXOff = box().xoff[c];
  template <int c> static constexpr int kLXOff = box().lxoff[c];
  template <int c> static constexpr int kW = box().w[c];
  template <int c> static constexpr int kLW = box().lw[c];
  static constexpr uint32_t kTx = box().tx;
  static constexpr int kStage = box().stage;
  // Exchange / staging buffer of B': per component RY+2 rows of 32 (rows
  // 0..RY-1 the tile, row RY the halo row, row RY+1 the halo column by row),
  // hi words then lo words.
  static constexpr int kXComp = (RY + 2) * 32;  // elements per component
  static constexpr int kXHi = 0;
  static constexpr int kXLo = round128(3 * kXComp * HS);
  static constexpr int kXBytes = kXLo + (kLo ? round128(3 * kXComp * LS) : 0);
  // Staging buffer of E': per component RY rows of 32, hi words then lo
  // words.
  static constexpr int kBComp = RY * 32;
  static constexpr int kBLo = round128(3 * kBComp * HS);
  static constexpr int kBBytes = kBLo + (kLo ? round128(3 * kBComp * LS) : 0);
  static constexpr int kRing = 0;
  static constexpr int kNS = kStages1<S>;
  static constexpr int kExch = kNS * kStage;
  static constexpr int kBst = kExch + 2 * kXBytes;
  static constexpr int kBar = kBst + 2 * kBBytes;
  static constexpr int kList = kBar + kNS * 8;
  static constexpr int kTotal = kList + 4 * (kMaxSources + 1);
  // The box the B-first sweep's halo column reads starts one column left of
  // the tile, inside every box's left offset.
  static_assert(OFF >= 1 && (!kLo || kLoOff1 >= 1), "the boxes need the left halo column");
  static_assert(Ws - OFF >= 32 && (!kLo || LWs - kLoOff1 >= 32) && W - OFF >= 33 && (!kLo || LW - kLoOff1 >= 33),
                "boxes must reach the tile's last column (and the one right of it)");
  static_assert((Ws * HS) % 16 == 0 && (W * HS) % 16 == 0 && (LWs * LS) % 16 == 0 && (LW * LS) % 16 == 0,
                "box rows must be whole 16-byte units");
  static_assert(box().hi[1] % 128 == 0 && box().hi[5] % 128 == 0 && box().lo[0] % 128 == 0 &&
                    box().lo[5] % 128 == 0,
                "ring boxes must start on 128-byte boundaries");
  static_assert(kStage % 128 == 0 && kTx <= (uint32_t)kStage, "ring stage layout");
  static_assert((kXComp * HS) % 128 == 0 && (kXComp * LS) % 128 == 0, "staging boxes must stay 128-byte aligned");
  static_assert((kBComp * HS) % 128 == 0 && (kBComp * LS) % 128 == 0, "staging boxes must stay 128-byte aligned");
};

// Whether the periodic window [o, o+n) of an axis of length N meets the m
// consecutive cells a, a+1, .. (taken mod N).
__device__ __forceinline__ bool window_meets(int o, int n, int N, int a, int m) {
  int s = a - o;
  if (s < 0) s += N;
  return s < n || s + m > N;
}

// One tile: columns bx*32 .., rows by*RY .., planes bz*kchunk .. of one
// domain, with the CTA's shared memory `smem` (barriers initialised).  `ring`
// counts the ring fills the CTA has consumed so far (it carries the slot and
// phase from tile to tile); on return the copy-engine leader has waited for the tile's
// stores to read their staging, and the caller synchronises before the next
// tile writes staging again.
//
// fused1_tile lists the sources that can reach the tile, then runs the plane
// loop, fused1b_planes, compiled with (kSrc) or without source evaluation.
// On a wait that gives up (any thread), every thread leaves the plane loop
// after the iteration's barrier; the copy-engine leader then waits for the
// tile's loads still in flight and its committed stores (drain_tile), and the
// function returns false.
template <int NS>
__device__ __forceinline__ void drain_tile(uint64_t* bar, uint32_t ring, int first, int issued, const WaitCtl& wc) {
  for (int f = first; f < issued; ++f) {
    const uint32_t g = ring + (uint32_t)f;
    mbar_wait_bounded(&bar[g % NS], (g / NS) & 1u, wc, 2);
  }
  bulk_wait_all();
}

// The sweep of one tile (see the file comment): planes k1-1 down to k0-1.
// kE false: the B half steps alone (planes k1-1 down to k0, no E step and no
// halo cells; E is only read, so `out` may be `st`).  kEdge false: a tile
// that touches no face of the grid (no ghost rows or columns to write, 32
// full columns), compiled without that code.
template <class S, class A, int RY, int kApps, bool kDenseJ, bool kSrc, bool kE = true, bool kEdge = true>
__device__ __forceinline__ bool fused1b_planes(const PLayout& L, const S& st, const S& out, const StepMaps& maps,
                                               const CoefSet& cs, int bx, int by, int bz, int kchunk, int2 zr,
                                               const float* __restrict__ Jx, const float* __restrict__ Jy,
                                               const float* __restrict__ Jz, const SourceSet& ss, int64_t step,
                                               const WaitCtl& wc, unsigned char* smem, uint32_t& ring, int nsrc) {
  using P = Plan1<S, RY>;
  using HiT = typename S::HiT;
  using T = typename A::Cur;
  constexpr int NS = P::kNS;
  constexpr bool kHalfWords = std::is_same<S, StoreF16>::value;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + P::kBar);
  int* list = reinterpret_cast<int*>(smem + P::kList);

  const int lane = threadIdx.x, w = threadIdx.y;
  const int x0 = bx * 32, y0 = by * RY;
  const int nx = kEdge ? min(32, L.Ni - x0) : 32, ny = kEdge ? min(RY, L.Nj - y0) : RY;
  const bool hrow = (w == RY), hcol = (w == RY + 1);
  // Box row (0: y0-1) and tile column (-1: x0-1) of the thread's cell.  Lanes
  // of the halo-column warp past the tile's rows are clamped onto its last
  // row: they compute but never publish.
  const int r = hrow ? 0 : hcol ? min(lane, RY - 1) + 1 : w + 1;
  const int cx = hcol ? -1 : lane;
  const bool active =
      (kE || (!hrow && !hcol)) && (hrow ? (lane < nx) : hcol ? (lane < ny) : (w < ny && lane < nx));
  const bool interior = !hrow && !hcol && w < ny && lane < nx;
  // unwrapped coordinates (x = -1 and y = -1 are the ghost copies of Ni-1 and
  // Nj-1); interior cells have 0 <= x < Ni, 0 <= y < Nj
  const int xu = x0 + cx, yu = y0 + r - 1;
  const int k0 = zr.x + bz * kchunk;
  const int k1 = min(k0 + kchunk, zr.y);
  const int n_it = kE ? k1 - k0 + 1 : k1 - k0;
  const bool leader = (w == RY + 1 && lane == 0);
  const int slot0 = (int)(ring % NS);
  const uint32_t phase0 = (ring / NS) & 1u;
  const bool tile_edge = kEdge && (x0 == 0 || x0 + nx == L.Ni || y0 == 0 || y0 + ny == L.Nj);
  const bool tma_out = !kEdge || (nx == 32);
  auto ghost_r = [&]() { return P::kLo && tma_out && x0 == 0 && L.Ni % 8 == 0; };
  auto ghost_l = [&]() { return P::kLo && tma_out && x0 + 32 == L.Ni; };
  const bool edge_cell = interior && (yu == 0 || yu == L.Nj - 1);

  // Exchange offsets: where the thread publishes B', and (interior cells)
  // where it finds B' at (i-1) and (j-1).
  const int xo_own = hrow ? RY * 32 + lane : hcol ? (RY + 1) * 32 + (r - 1) : w * 32 + lane;
  const int xo_left = (lane == 0) ? (RY + 1) * 32 + w : w * 32 + lane - 1;
  const int xo_down = (w == 0) ? RY * 32 + lane : (w - 1) * 32 + lane;
  const int bo_own = w * 32 + lane;

  // Iteration it handles plane t = k1-1-it (t = -1 is plane Nk-1) from ring
  // fill `it` of the tile.
  int issued = 0;
  auto issue = [&](int it) {
    if (wc.withhold) return;
    ++issued;
    const int t = k1 - 1 - it;
    const int kk = t < 0 ? L.Nk - 1 : t;
    const int slot = (slot0 + it) % NS;
    unsigned char* base = smem + P::kRing + slot * P::kStage;
    mbar_arrive_expect_tx(&bar[slot], P::kTx);
    for_each_comp([&](auto cc) {
      constexpr int c = decltype(cc)::value;
      tma_load_3d(base + P::template kHiAt<c>, &maps.ld.hi[c], x0 + kPadX - P::template kXOff<c>, y0 - 1 + kPadY,
                  kk, &bar[slot]);
      if (P::kLo)
        tma_load_3d(base + P::template kLoAt<c>, &maps.ld.lo[c], x0 + kPadX - P::template kLXOff<c>,
                    y0 - 1 + kPadY, kk, &bar[slot]);
    });
  };
  if (leader)
    for (int it = 0; it < n_it && it < NS; ++it) issue(it);

  // Per-column factor (amp gx) gy of the first kFastSources listed sources.
  T sxy[kFastSources];
  unsigned smask = 0;
#pragma unroll
  for (int q = 0; q < kFastSources; ++q) {
    sxy[q] = A::cur_zero();
    if (kSrc && q < nsrc) {
      const DevSource& d = ss.src[list[q]];
      const int di = box_offset(xu, d.i0, d.ni, L.Ni);
      const int dj = box_offset(yu, d.j0, d.nj, L.Nj);
      if (interior && di >= 0 && dj >= 0) {
        sxy[q] = A::cur_mul(A::cur_mul(A::cur_table(ss, d.amp_off + step), A::cur_table(ss, d.gx_off + di)),
                            A::cur_table(ss, d.gy_off + dj));
        smask |= 1u << q;
      }
    }
  }

  // E(t+1) of the thread's cell (its z neighbour above), then B'(t+1).
  Pair pex{0.f, 0.f}, pey{0.f, 0.f}, pez{0.f, 0.f};
  Pair pbx{0.f, 0.f}, pby{0.f, 0.f}, pbz{0.f, 0.f};
  if (active) {
    const int64_t e0 = L.at(xu, yu, k1 == L.Nk ? 0 : k1);
    pex = st.load(0, e0);
    pey = st.load(1, e0);
  }

  int slot = slot0;
  uint32_t phase = phase0;
  for (int it = 0; it < n_it; ++it) {
    const int t = k1 - 1 - it;
    const int cur = it & 1;
    const bool timed_out = !mbar_wait_bounded(&bar[slot], phase, wc);
    const unsigned char* stage = smem + P::kRing + slot * P::kStage;
    const HiT* H = reinterpret_cast<const HiT*>(stage);
    const LoT* Q = reinterpret_cast<const LoT*>(stage);
    // component c at (dr rows, dc columns) from the thread's cell (box row r,
    // tile column cx); each component's box has its own width
    auto V = [&](auto cc, int dr, int dc) -> Pair {
      constexpr int c = decltype(cc)::value;
      const HiT h = H[P::template kHiAt<c> / P::HS + (r + dr - P::template kRow0<c>) * P::template kW<c> +
                      P::template kXOff<c> + cx + dc];
      const LoT q = P::kLo ? Q[P::template kLoAt<c> / P::LS + (r + dr - P::template kRow0<c>) * P::template kLW<c> +
                               P::template kLXOff<c> + cx + dc]
                           : LoT(0);
      return st.decode(c, h, q);
    };

    // 1. B'(t), in the operation order of the B sweep (kernels_f32.cu b_column)
    const Pair ex = V(Comp<0>{}, 0, 0), ey = V(Comp<1>{}, 0, 0), ez = V(Comp<2>{}, 0, 0);
    Pair ux, uy, uz;
    if constexpr (kHalfWords) {
      // FP16 words: a neighbour that enters one difference only enters it
      // unconverted (sub_h_f: the same FP32 difference)
      auto VH = [&](auto cc, int dr, int dc) -> HiT {
        constexpr int c = decltype(cc)::value;
        return H[P::template kHiAt<c> / P::HS + (r + dr - P::template kRow0<c>) * P::template kW<c> +
                 P::template kXOff<c> + cx + dc];
      };
      ux = A::curl_d(bcoef<S>(cs, st, 0, 0), __fsub_rn(pey.hi, ey.hi), bcoef<S>(cs, st, 0, 1),
                     sub_h_f(VH(Comp<2>{}, 1, 0), ez.hi));
      uy = A::curl_d(bcoef<S>(cs, st, 1, 0), sub_h_f(VH(Comp<2>{}, 0, 1), ez.hi), bcoef<S>(cs, st, 1, 1),
                     __fsub_rn(pex.hi, ex.hi));
      uz = A::curl_d(bcoef<S>(cs, st, 2, 0), sub_h_f(VH(Comp<0>{}, 1, 0), ex.hi), bcoef<S>(cs, st, 2, 1),
                     sub_h_f(VH(Comp<1>{}, 0, 1), ey.hi));
    } else if constexpr (S::kComp) {
      // compensated words: the same for a neighbour's BF16 lo word (sub_bf_f)
      auto VN = [&](auto cc, int dr, int dc, const Pair& own) -> float {
        constexpr int c = decltype(cc)::value;
        const int row = r + dr - P::template kRow0<c>;
        const float h = H[P::template kHiAt<c> / P::HS + row * P::template kW<c> + P::template kXOff<c> + cx + dc];
        const LoT q = Q[P::template kLoAt<c> / P::LS + row * P::template kLW<c> + P::template kLXOff<c> + cx + dc];
        return __fadd_rn(__fsub_rn(h, own.hi), sub_bf_f(q, own.lo));
      };
      ux = A::curl_d(bcoef<S>(cs, st, 0, 0), A::dif(pey, ey), bcoef<S>(cs, st, 0, 1), VN(Comp<2>{}, 1, 0, ez));
      uy = A::curl_d(bcoef<S>(cs, st, 1, 0), VN(Comp<2>{}, 0, 1, ez), bcoef<S>(cs, st, 1, 1), A::dif(pex, ex));
      uz = A::curl_d(bcoef<S>(cs, st, 2, 0), VN(Comp<0>{}, 1, 0, ex), bcoef<S>(cs, st, 2, 1), VN(Comp<1>{}, 0, 1, ey));
    } else {
      ux = A::curl(bcoef<S>(cs, st, 0, 0), pey, ey, bcoef<S>(cs, st, 0, 1), V(Comp<2>{}, 1, 0), ez);
      uy = A::curl(bcoef<S>(cs, st, 1, 0), V(Comp<2>{}, 0, 1), ez, bcoef<S>(cs, st, 1, 1), pex, ex);
      uz = A::curl(bcoef<S>(cs, st, 2, 0), V(Comp<0>{}, 1, 0), ex, bcoef<S>(cs, st, 2, 1), V(Comp<1>{}, 0, 1), ey);
    }
    if (kApps == 2) {
      ux = A::twice(ux);
      uy = A::twice(uy);
      uz = A::twice(uz);
    }
    const Pair ax = A::acc_curl(V(Comp<3>{}, 0, 0), ux), ay = A::acc_curl(V(Comp<4>{}, 0, 0), uy),
               az = A::acc_curl(V(Comp<5>{}, 0, 0), uz);
    // B' in its stored words; the E update uses the value they hold.
    const HiT bhx = st.enc_hi(3, ax), bhy = st.enc_hi(4, ay), bhz = st.enc_hi(5, az);
    const LoT blx = st.enc_lo(ax), bly = st.enc_lo(ay), blz = st.enc_lo(az);
    const Pair nbx = st.decode(3, bhx, blx), nby = st.decode(4, bhy, bly), nbz = st.decode(5, bhz, blz);

    unsigned char* xb = smem + P::kExch + cur * P::kXBytes;
    if (active) {
      HiT* xh = reinterpret_cast<HiT*>(xb + P::kXHi) + xo_own;
      xh[0] = bhx;
      xh[P::kXComp] = bhy;
      xh[2 * P::kXComp] = bhz;
      if (P::kLo) {
        LoT* xq = reinterpret_cast<LoT*>(xb + P::kXLo) + xo_own;
        xq[0] = blx;
        xq[P::kXComp] = bly;
        xq[2 * P::kXComp] = blz;
      }
    }

    // 2. E'(t+1), in the operation order of the E sweep (kernels_f32.cu e_sweep)
    Pair nex{0.f, 0.f}, ney{0.f, 0.f}, nez{0.f, 0.f};
    unsigned char* eb = smem + P::kBst + cur * P::kBBytes;
    const bool e_step = kE && it > 0;  // plane t+1 lies in the chunk
    if (e_step && interior) {
      const int ke = t + 1;  // < k1 <= Nk
      const unsigned char* pb = smem + P::kExch + (cur ^ 1) * P::kXBytes;
      const HiT* ph = reinterpret_cast<const HiT*>(pb + P::kXHi);
      const LoT* pq = reinterpret_cast<const LoT*>(pb + P::kXLo);
      auto Bn = [&](int c, int off) -> Pair {  // B'(t+1), component 3 + c
        return st.decode(3 + c, ph[c * P::kXComp + off], P::kLo ? pq[c * P::kXComp + off] : LoT(0));
      };
      Pair qx, qy, qz;
      if constexpr (kHalfWords) {
        auto BH = [&](int c, int off) -> HiT { return ph[c * P::kXComp + off]; };  // B'(t+1) word
        qx = A::curl_d(ecoef<S>(cs, st, 0, 0), sub_f_h(pbz.hi, BH(2, xo_down)), ecoef<S>(cs, st, 0, 1),
                       __fsub_rn(pby.hi, nby.hi));
        qy = A::curl_d(ecoef<S>(cs, st, 1, 0), __fsub_rn(pbx.hi, nbx.hi), ecoef<S>(cs, st, 1, 1),
                       sub_f_h(pbz.hi, BH(2, xo_left)));
        qz = A::curl_d(ecoef<S>(cs, st, 2, 0), sub_f_h(pby.hi, BH(1, xo_left)), ecoef<S>(cs, st, 2, 1),
                       sub_f_h(pbx.hi, BH(0, xo_down)));
      } else if constexpr (S::kComp) {
        // own pair minus a neighbour's B'(t+1) words (sub_f_bf on the lo word)
        auto DN = [&](const Pair& own, int c, int off) -> float {
          return __fadd_rn(__fsub_rn(own.hi, ph[c * P::kXComp + off]), sub_f_bf(own.lo, pq[c * P::kXComp + off]));
        };
        qx = A::curl_d(ecoef<S>(cs, st, 0, 0), DN(pbz, 2, xo_down), ecoef<S>(cs, st, 0, 1), A::dif(pby, nby));
        qy = A::curl_d(ecoef<S>(cs, st, 1, 0), A::dif(pbx, nbx), ecoef<S>(cs, st, 1, 1), DN(pbz, 2, xo_left));
        qz = A::curl_d(ecoef<S>(cs, st, 2, 0), DN(pby, 1, xo_left), ecoef<S>(cs, st, 2, 1), DN(pbx, 0, xo_down));
      } else {
        qx = A::curl(ecoef<S>(cs, st, 0, 0), pbz, Bn(2, xo_down), ecoef<S>(cs, st, 0, 1), pby, nby);
        qy = A::curl(ecoef<S>(cs, st, 1, 0), pbx, nbx, ecoef<S>(cs, st, 1, 1), pbz, Bn(2, xo_left));
        qz = A::curl(ecoef<S>(cs, st, 2, 0), pby, Bn(1, xo_left), ecoef<S>(cs, st, 2, 1), pbx, Bn(0, xo_down));
      }
      unsigned has = 0;  // E components that received current (their increment has a lo word)
      if (kDenseJ || kSrc) {
        T jv[3] = {A::cur_zero(), A::cur_zero(), A::cur_zero()};
        if (kDenseJ) {
          const int64_t d = xu + (int64_t)yu * L.Ni + (int64_t)ke * L.Ni * L.Nj;
          jv[0] = A::cur_dense(Jx[d]);
          jv[1] = A::cur_dense(Jy[d]);
          jv[2] = A::cur_dense(Jz[d]);
          has = 7u;
        }
#pragma unroll
        for (int q = 0; q < kFastSources; ++q) {
          if (kSrc && q < nsrc) {
            const DevSource& d = ss.src[list[q]];
            const int dk = box_offset(ke, d.k0, d.nk, L.Nk);  // the same for the whole tile
            if (dk >= 0 && (smask >> q & 1u)) {
              add_current<A>(jv, d.comp_mask, A::cur_mul(sxy[q], A::cur_table(ss, d.gz_off + dk)), has);
              has |= (unsigned)d.comp_mask;
            }
          }
        }
        for (int i = kFastSources; kSrc && i < nsrc; ++i) {
          const DevSource& d = ss.src[list[i]];
          const int dk = box_offset(ke, d.k0, d.nk, L.Nk);
          if (dk < 0) continue;
          const int di = box_offset(xu, d.i0, d.ni, L.Ni);
          const int dj = box_offset(yu, d.j0, d.nj, L.Nj);
          if (di >= 0 && dj >= 0) {
            add_current<A>(jv, d.comp_mask,
                           A::cur_mul(A::cur_mul(A::cur_mul(A::cur_table(ss, d.amp_off + step),
                                                            A::cur_table(ss, d.gx_off + di)),
                                                 A::cur_table(ss, d.gy_off + dj)),
                                      A::cur_table(ss, d.gz_off + dk)),
                           has);
            has |= (unsigned)d.comp_mask;
          }
        }
        if (has & 1u) qx = A::add(qx, A::cur_term(jcoef<S>(cs, st, 0), jv[0]));
        if (has & 2u) qy = A::add(qy, A::cur_term(jcoef<S>(cs, st, 1), jv[1]));
        if (has & 4u) qz = A::add(qz, A::cur_term(jcoef<S>(cs, st, 2), jv[2]));
      }
      nex = (has & 1u) ? A::acc(pex, qx) : A::acc_curl(pex, qx);
      ney = (has & 2u) ? A::acc(pey, qy) : A::acc_curl(pey, qy);
      nez = (has & 4u) ? A::acc(pez, qz) : A::acc_curl(pez, qz);
      HiT* eh = reinterpret_cast<HiT*>(eb) + bo_own;
      eh[0] = st.enc_hi(0, nex);
      eh[P::kBComp] = st.enc_hi(1, ney);
      eh[2 * P::kBComp] = st.enc_hi(2, nez);
      if (P::kLo) {
        LoT* eq = reinterpret_cast<LoT*>(eb + P::kBLo) + bo_own;
        eq[0] = st.enc_lo(nex);
        eq[P::kBComp] = st.enc_lo(ney);
        eq[2 * P::kBComp] = st.enc_lo(nez);
      }
    }
    if (kEdge && !tma_out && interior) {
      const int64_t o = L.at(xu, yu, 0);
      if (t >= k0) {
        out.store(3, o + (int64_t)t * L.pplane, nbx);
        out.store(4, o + (int64_t)t * L.pplane, nby);
        out.store(5, o + (int64_t)t * L.pplane, nbz);
      }
      if (e_step) {
        out.store(0, o + (int64_t)(t + 1) * L.pplane, nex);
        out.store(1, o + (int64_t)(t + 1) * L.pplane, ney);
        out.store(2, o + (int64_t)(t + 1) * L.pplane, nez);
      }
    }
    // Ghost copies of edge cells (their tiles only).
    if (tile_edge && edge_cell) {
      if (t >= k0) {
        store_ghost_rows(out, L, true, true, 3, xu, yu, t, nbx);
        store_ghost_rows(out, L, true, true, 4, xu, yu, t, nby);
        store_ghost_rows(out, L, true, true, 5, xu, yu, t, nbz);
      }
      if (e_step) {
        store_ghost_rows(out, L, true, true, 0, xu, yu, t + 1, nex);
        store_ghost_rows(out, L, true, true, 1, xu, yu, t + 1, ney);
        store_ghost_rows(out, L, true, true, 2, xu, yu, t + 1, nez);
      }
    }

    pex = ex;
    pey = ey;
    pez = ez;
    pbx = nbx;
    pby = nby;
    pbz = nbz;
    fence_async_smem();
    if (leader) bulk_wait_read_all();
    if (__syncthreads_or(timed_out)) {
      if (leader) drain_tile<NS>(bar, ring, it, issued, wc);
      return false;
    }
    if (kEdge && w == RY && lane < ny && (x0 == 0 || x0 + nx == L.Ni)) {
      // ghost columns the bulk copies do not write: x = Ni from column 0,
      // x = -1 from column nx-1, row y0+lane, copied as stored words
#pragma unroll 1
      for (int side = 0; side < 2; ++side) {
        const bool on = side == 0 ? (x0 == 0 && !ghost_r()) : (x0 + nx == L.Ni && !ghost_l());
        if (!on) continue;
        const int col = side == 0 ? 0 : nx - 1;
        const int64_t g = L.at(side == 0 ? L.Ni : -1, y0 + lane, 0);
        const HiT* bh = reinterpret_cast<const HiT*>(xb + P::kXHi) + lane * 32 + col;
        const LoT* bq = reinterpret_cast<const LoT*>(xb + P::kXLo) + lane * 32 + col;
        const HiT* eh = reinterpret_cast<const HiT*>(eb) + lane * 32 + col;
        const LoT* eq = reinterpret_cast<const LoT*>(eb + P::kBLo) + lane * 32 + col;
        if (t >= k0)
          for (int c = 0; c < 3; ++c)
            out.store_words(3 + c, g + (int64_t)t * L.pplane, bh[c * P::kXComp], P::kLo ? bq[c * P::kXComp] : LoT(0));
        if (e_step)
          for (int c = 0; c < 3; ++c)
            out.store_words(c, g + (int64_t)(t + 1) * L.pplane, eh[c * P::kBComp],
                            P::kLo ? eq[c * P::kBComp] : LoT(0));
      }
    }
    if (leader) {
      // the tile's boxes at its own columns, then the margins it fills
#pragma unroll 1
      for (int g = 0; g < (kEdge ? 3 : 1) && tma_out; ++g) {
        if ((g == 1 && !ghost_r()) || (g == 2 && !ghost_l())) continue;
        const int xs = g == 0 ? x0 + kPadX : g == 1 ? L.Ni + kPadX : 0;
        if (t >= k0)
          for (int c = 0; c < 3; ++c) {
            tma_store_3d(&maps.st.hi[3 + c], xb + P::kXHi + c * P::kXComp * P::HS, xs, y0, t);
            if (P::kLo) tma_store_3d(&maps.st.lo[3 + c], xb + P::kXLo + c * P::kXComp * P::LS, xs, y0, t);
          }
        if (e_step)
          for (int c = 0; c < 3; ++c) {
            tma_store_3d(&maps.st.hi[c], eb + c * P::kBComp * P::HS, xs, y0, t + 1);
            if (P::kLo) tma_store_3d(&maps.st.lo[c], eb + P::kBLo + c * P::kBComp * P::LS, xs, y0, t + 1);
          }
      }
      bulk_commit();
      if (it + NS < n_it) issue(it + NS);
    }
    if (++slot == NS) {
      slot = 0;
      phase ^= 1u;
    }
  }
  ring += (uint32_t)n_it;
  if (leader) bulk_wait_read_all();
  return true;
}

//
// kSplit: compile the plane loop twice and run the source-free copy on tiles
// that no source reaches (fewer live registers there).  The batched kernel
// takes either: where its tiles alternate between the two cases, two hot
// copies of the loop ran slower than one (its autotuner picks).  Returns false
// when a bounded wait gave up (uniform over the CTA).
template <class S, class A, int RY, int kApps, bool kDenseJ, bool kSplit>
__device__ __forceinline__ bool fused1_tile(const PLayout& L, const S& st, const S& out, const StepMaps& maps,
                                            const CoefSet& cs, int bx, int by, int bz, int kchunk, int2 zr,
                                            const float* __restrict__ Jx, const float* __restrict__ Jy,
                                            const float* __restrict__ Jz, const SourceSet& ss, int64_t step,
                                            const WaitCtl& wc, unsigned char* smem, uint32_t& ring) {
  using P = Plan1<S, RY>;
  int* list = reinterpret_cast<int*>(smem + P::kList);
  // Sources that can touch this tile's cells (with one cell of halo on each
  // side), in registration order; the exact per-cell test comes in the plane loop.
  if (threadIdx.y == 0) {
    const int lane = threadIdx.x;
    const int x0 = bx * 32, y0 = by * RY;
    const int nx = min(32, L.Ni - x0), ny = min(RY, L.Nj - y0);
    int n = 0;
    for (int b = 0; b < ss.count; b += 32) {
      const int q = b + lane;
      bool hit = false;
      if (q < ss.count) {
        const DevSource& d = ss.src[q];
        hit = step < d.n_amp && window_meets(d.i0, d.ni, L.Ni, x0, nx + 1) &&
              window_meets(d.j0, d.nj, L.Nj, y0, ny + 1);
      }
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if (hit) list[n + __popc(m & ((1u << lane) - 1u))] = q;
      n += __popc(m);
    }
    if (lane == 0) list[kMaxSources] = n;
  }
  __syncthreads();
  const int nsrc = list[kMaxSources];
  // Tiles on a face of the grid (ghost copies, partial columns) and the
  // rest, in separate copies of the plane loop for the plain forms (FP16
  // 12 % and FP32 2 % faster at 512^3); the compensated form keeps one copy
  // (two made it 7 % slower and the batched sweep spill).
  const int x0 = bx * 32, y0 = by * RY;
  const bool edge = S::kComp || x0 == 0 || x0 + 32 >= L.Ni || y0 == 0 || y0 + RY >= L.Nj;
#define FDTD_PLANES(SRC, NSRC, EDGE)                                                                               \
  return fused1b_planes<S, A, RY, kApps, kDenseJ, SRC, true, EDGE>(L, st, out, maps, cs, bx, by, bz, kchunk, zr, Jx, \
                                                                  Jy, Jz, ss, step, wc, smem, ring, NSRC)
  if (!kSplit || nsrc > 0) {
    if (edge) FDTD_PLANES(true, nsrc, true);
    FDTD_PLANES(true, nsrc, false);
  }
  if (edge) FDTD_PLANES(false, 0, true);
  FDTD_PLANES(false, 0, false);
#undef FDTD_PLANES
}

template <int NS>
__device__ __forceinline__ void init_ring(uint64_t* bar) {
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    for (int s = 0; s < NS; ++s) mbar_init(&bar[s], 1);
    mbar_init_fence();
  }
  __syncthreads();
}

template <class S, class A, int RY, int kApps, bool kDenseJ>
__global__ void __launch_bounds__(32 * (RY + 2), kMinCtas1<RY, S>)
    fused1(PLayout L, S st, S out, const __grid_constant__ StepMaps maps, CoefSet cs, int kchunk, int2 zr,
           const float* __restrict__ Jx, const float* __restrict__ Jy, const float* __restrict__ Jz,
           SourceSet ss, int64_t step, WaitCtl wc) {
  extern __shared__ __align__(128) unsigned char smem[];
  init_ring<Plan1<S, RY>::kNS>(reinterpret_cast<uint64_t*>(smem + Plan1<S, RY>::kBar));
  uint32_t ring = 0;
  fused1_tile<S, A, RY, kApps, kDenseJ, true>(L, st, out, maps, cs, blockIdx.x, blockIdx.y, blockIdx.z, kchunk, zr,
                                                   Jx, Jy, Jz, ss, step, wc, smem, ring);
  if (threadIdx.x == 0 && threadIdx.y == RY + 1) bulk_wait_all();  // the copy-engine leader's stores
}

// The B half steps alone (`apps` of them) over planes [zr.x, zr.y), from
// `st` into `out` (which may be `st`): the tile machinery of the fused sweep
// without its E step.
template <class S, class A, int RY, int kApps>
__global__ void __launch_bounds__(32 * (RY + 2), kMinCtas1<RY>)
    fused1_bhalf(PLayout L, S st, S out, const __grid_constant__ StepMaps maps, CoefSet cs, int kchunk, int2 zr,
                 WaitCtl wc) {
  extern __shared__ __align__(128) unsigned char smem[];
  init_ring<Plan1<S, RY>::kNS>(reinterpret_cast<uint64_t*>(smem + Plan1<S, RY>::kBar));
  uint32_t ring = 0;
  SourceSet none{};
  fused1b_planes<S, A, RY, kApps, false, false, false>(L, st, out, maps, cs, blockIdx.x, blockIdx.y, blockIdx.z,
                                                       kchunk, zr, nullptr, nullptr, nullptr, none, 0, wc, smem, ring,
                                                       0);
  if (threadIdx.x == 0 && threadIdx.y == RY + 1) bulk_wait_all();  // the copy-engine leader's stores
}

// Batched form: a persistent kernel of B-first sweeps; every CTA takes tiles
// (domain, bx, by, bz) from the tile table in order, through an atomic
// counter, until none are left.  `parity` selects which of each domain's two
// copies is read.  The last CTA to finish resets the counters for the next
// launch.
template <class S, class A, int RY, int kApps, bool kSplit>
__global__ void __launch_bounds__(32 * (RY + 2), kMinCtas1<RY>)
    fused1_batch(const BatchDomain<S>* __restrict__ doms, const StepMaps* __restrict__ maps,
                 const int4* __restrict__ tiles, int n_tiles, int parity, int kchunk,
                 const int64_t* __restrict__ step_base, int step_off, int* counters, WaitCtl wc) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ BatchDomain<S> dom;
  __shared__ int4 tile;
  init_ring<Plan1<S, RY>::kNS>(reinterpret_cast<uint64_t*>(smem + Plan1<S, RY>::kBar));
  const bool leader = threadIdx.x == 0 && threadIdx.y == 0;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const int64_t step = *step_base + step_off;
  uint32_t ring = 0;
  for (;;) {
    if (leader) {
      const int it = atomicAdd(&counters[0], 1);
      tile = it < n_tiles ? tiles[it] : make_int4(-1, 0, 0, 0);
    }
    __syncthreads();
    const int4 w = tile;
    if (w.x < 0) break;
    // the tile's domain record, copied word by word into shared memory
    constexpr int kWords = (int)(sizeof(BatchDomain<S>) / 4);
    const int* src = reinterpret_cast<const int*>(doms + w.x);
    int* dst = reinterpret_cast<int*>(&dom);
    for (int q = tid; q < kWords; q += blockDim.x * blockDim.y) dst[q] = src[q];
    if (threadIdx.y == 1 && threadIdx.x < 24) {
      // warm the descriptor cache for this tile's loads and stores
      const StepMaps& m = maps[2 * w.x + parity];
      const int q = threadIdx.x;
      const CUtensorMap* tm = q < 6 ? &m.ld.hi[q] : q < 12 ? &m.ld.lo[q - 6] : q < 18 ? &m.st.hi[q - 12] : &m.st.lo[q - 18];
      if (Plan1<S, RY>::kLo || (q < 6 || (q >= 12 && q < 18))) prefetch_tensormap(tm);
    }
    __syncthreads();
    const bool ok = fused1_tile<S, A, RY, kApps, false, kSplit>(
        dom.L, dom.s[parity], dom.s[parity ^ 1], maps[2 * w.x + parity], dom.cs, w.y, w.z, w.w, kchunk,
        make_int2(0, dom.L.Nk), nullptr,
        nullptr, nullptr, dom.ss, step, wc, smem, ring);
    if (!ok) break;  // a wait gave up: this CTA takes no more tiles
    __syncthreads();
  }
  if (threadIdx.x == 0 && threadIdx.y == RY + 1) bulk_wait_all();  // the copy-engine leader's stores
  if (leader) {
    __threadfence();
    if (atomicAdd(&counters[1], 1) == (int)(gridDim.x * gridDim.y * gridDim.z) - 1) {
      counters[0] = 0;
      counters[1] = 0;
    }
  }
}

// ---------------------------------------------------------------------------

template <class S, int RY, int APPS, bool DJ>
static cudaError_t launch1_one(dim3 grid, const PLayout& L, const S& st, const S& out, const StepMaps& maps,
                               const CoefSet& cs, int kchunk, int2 zr, const float* const J[3], const SourceSet& ss,
                               int64_t step, const WaitCtl& wc, cudaStream_t stream) {
  using A = typename ArithOf1<S>::type;
  auto kern = fused1<S, A, RY, APPS, DJ>;
  const int bytes = Plan1<S, RY>::kTotal;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  kern<<<grid, dim3(32, RY + 2), bytes, stream>>>(L, st, out, maps, cs, kchunk, zr, J[0], J[1], J[2], ss, step, wc);
  return cudaGetLastError();
}

template <class S, int RY>
static cudaError_t launch1_ry(const PLayout& L, const S& st, const S& out, const StepMaps& maps,
                              const float* const J[3], bool dense_j, const CoefSet& cs, const SourceSet& ss,
                              int64_t step, int applications, int kchunk, int2 zr, const WaitCtl& wc,
                              cudaStream_t stream) {
  if (ss.count > kMaxSources) return cudaErrorInvalidValue;
  if (zr.x < 0 || zr.y > L.Nk || zr.y <= zr.x) return cudaErrorInvalidValue;
  dim3 grid((L.Ni + 31) / 32, (L.Nj + RY - 1) / RY, (zr.y - zr.x + kchunk - 1) / kchunk);
#define FDTD_F(APPS, DJ) \
  return launch1_one<S, RY, APPS, DJ>(grid, L, st, out, maps, cs, kchunk, zr, J, ss, step, wc, stream)
  if (applications == 2) {
    if (dense_j) FDTD_F(2, true);
    FDTD_F(2, false);
  }
  if (dense_j) FDTD_F(1, true);
  FDTD_F(1, false);
#undef FDTD_F
}

template <class S>
cudaError_t launch_fused1_f32(const PLayout& L, const S& st, const S& out, const void* maps,
                              const float* const J[3], bool dense_j, const CoefSet& cs, const SourceSet& ss,
                              int64_t step, int applications, const FusedConfig& cfg, const WaitCtl& wc,
                              cudaStream_t stream, int kbeg, int kend) {
  const int kchunk = cfg.kchunk > 0 ? cfg.kchunk : 48;
  const StepMaps& m = *static_cast<const StepMaps*>(maps);
  const int2 zr = make_int2(kbeg, kend < 0 ? L.Nk : kend);
#define FDTD_RY(RY) \
  return launch1_ry<S, RY>(L, st, out, m, J, dense_j, cs, ss, step, applications, kchunk, zr, wc, stream)
  if (cfg.tile_y == 6) FDTD_RY(6);
  if (cfg.tile_y == 30) FDTD_RY(30);
  FDTD_RY(14);
#undef FDTD_RY
}

template <class S, int RY>
static cudaError_t launch_bhalf_ry(const PLayout& L, const S& st, const S& out, const StepMaps& m, const CoefSet& cs,
                                   int applications, int kchunk, int2 zr, const WaitCtl& wc, cudaStream_t stream) {
  using A = typename ArithOf1<S>::type;
  const dim3 grid((L.Ni + 31) / 32, (L.Nj + RY - 1) / RY, (zr.y - zr.x + kchunk - 1) / kchunk);
  auto kern = applications == 2 ? fused1_bhalf<S, A, RY, 2> : fused1_bhalf<S, A, RY, 1>;
  const int bytes = Plan1<S, RY>::kTotal;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  kern<<<grid, dim3(32, RY + 2), bytes, stream>>>(L, st, out, m, cs, kchunk, zr, wc);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_bhalf_f32(const PLayout& L, const S& st, const S& out, const void* maps, const CoefSet& cs,
                             int applications, const FusedConfig& cfg, const WaitCtl& wc, cudaStream_t stream,
                             int kbeg, int kend) {
  if (kend < 0) kend = L.Nk;
  if (kbeg < 0 || kend > L.Nk) return cudaErrorInvalidValue;
  if (kend <= kbeg) return cudaSuccess;
  const StepMaps& m = *static_cast<const StepMaps*>(maps);
  const int2 zr = make_int2(kbeg, kend);
  const int kchunk = cfg.kchunk > 0 ? cfg.kchunk : 48;
  if (cfg.tile_y == 6) return launch_bhalf_ry<S, 6>(L, st, out, m, cs, applications, kchunk, zr, wc, stream);
  if (cfg.tile_y == 30) return launch_bhalf_ry<S, 30>(L, st, out, m, cs, applications, kchunk, zr, wc, stream);
  return launch_bhalf_ry<S, 14>(L, st, out, m, cs, applications, kchunk, zr, wc, stream);
}

template <class S, int RY, int APPS, bool SPLIT>
static cudaError_t launch1_batch_one(const BatchDomain<S>* doms, const StepMaps* maps, const int4* tiles,
                                     int n_tiles, int parity, int kchunk, const int64_t* step_base, int step_off,
                                     int* counters, const WaitCtl& wc, cudaStream_t stream) {
  using A = typename ArithOf1<S>::type;
  auto kern = fused1_batch<S, A, RY, APPS, SPLIT>;
  const int bytes = Plan1<S, RY>::kTotal;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * (RY + 2), bytes)) != cudaSuccess)
    return e;
  const int grid = sms * (per_sm > 0 ? per_sm : 1);
  kern<<<grid, dim3(32, RY + 2), bytes, stream>>>(doms, maps, tiles, n_tiles, parity, kchunk, step_base, step_off,
                                                  counters, wc);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_fused1_batch(const void* doms, const StepMaps* maps, const int4* tiles, int n_tiles, int parity,
                                int applications, const FusedConfig& cfg, const int64_t* step_base, int step_off,
                                int* counters, const WaitCtl& wc, cudaStream_t stream) {
  const BatchDomain<S>* d = static_cast<const BatchDomain<S>*>(doms);
  const int kc = cfg.kchunk;
#define FDTD_B1(RY, SPLIT)                                                                                          \
  return applications == 2                                                                                       \
             ? launch1_batch_one<S, RY, 2, SPLIT>(d, maps, tiles, n_tiles, parity, kc, step_base, step_off, counters, \
                                                  wc, stream)                                                    \
             : launch1_batch_one<S, RY, 1, SPLIT>(d, maps, tiles, n_tiles, parity, kc, step_base, step_off, counters, \
                                                  wc, stream)
#define FDTD_B(RY)                  \
  {                                 \
    if (cfg.split_sources)          \
      FDTD_B1(RY, true);            \
    FDTD_B1(RY, false);             \
  }
  if (cfg.tile_y == 6) FDTD_B(6);
  if (cfg.tile_y == 30) FDTD_B(30);
  FDTD_B(14);
#undef FDTD_B
#undef FDTD_B1
}

template <class S>
void fused1_box_widths(int hi[6], int lo[6]) {
  const BoxTable b = Plan1<S, 14>::box();
  for (int c = 0; c < 6; ++c) {
    hi[c] = b.w[c];
    lo[c] = b.lw[c];
  }
}

#define FDTD_INSTANTIATE(S)                                                                              \
  template cudaError_t launch_fused1_f32<S>(const PLayout&, const S&, const S&, const void*,            \
                                            const float* const[3], bool, const CoefSet&, const SourceSet&, \
                                            int64_t, int, const FusedConfig&, const WaitCtl&, cudaStream_t,   \
                                            int, int);                                                     \
  template cudaError_t launch_fused1_batch<S>(const void*, const StepMaps*, const int4*, int, int, int,          \
                                              const FusedConfig&, const int64_t*, int, int*, const WaitCtl&,     \
                                              cudaStream_t);                                                     \
  template void fused1_box_widths<S>(int[6], int[6]);                                                 \
  template cudaError_t launch_bhalf_f32<S>(const PLayout&, const S&, const S&, const void*, const CoefSet&, int, \
                                           const FusedConfig&, const WaitCtl&, cudaStream_t, int, int);
FDTD_INSTANTIATE(StoreF32)
FDTD_INSTANTIATE(StoreF32C)
FDTD_INSTANTIATE(StoreF16)
#undef FDTD_INSTANTIATE

}  // namespace fdtd
