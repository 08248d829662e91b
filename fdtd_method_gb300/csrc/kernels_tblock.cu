// Temporal blocking: two update_fields steps per pass over the state (the
// depth-2 sweep), for the FP32-arithmetic forms.  The sweep is two B-first
// sweeps (kernels_fused1.cu) run together in one z march: the second step
// lags the first by two planes, so every value it needs from the first step
// is in registers or in a shared-memory exchange written one iteration
// earlier, and each iteration still has one CTA barrier.  Each stage uses the
// split sweeps' arithmetic (kernels_f32.cu, the reference's functors
// kokkos_functors.h:64-90 E and :128-151 B) on the stored (quantised) values
// of the stage before, so the result is the bits of two one-step sweeps.
//
// A CTA owns a tile of 32 x RY cells at (x0, y0).  The four stages cover
// shrinking regions around it (tile coordinates, nx x ny the tile's cells):
//   B1  first step's B half steps   x in [-2, nx], y in [-2, ny]
//   E1  first step's E              x in [-1, nx], y in [-1, ny]
//   B2  second step's B half steps  x in [-1, nx-1], y in [-1, ny-1]
//   E2  second step's E             the tile
// Warps 0..RY-1 are the tile rows; six more take the halo cells: rows y = -1,
// -2 and RY (lanes = x), columns x = -1, -2 and 32 (lane l = y + 2).
// Iteration s (planes k1 down to k0-3) computes B1(s), E1(s+1), B2(s+2) and
// E2(s+3); a stage reads its own cell's earlier values from registers and its
// neighbours' from the exchange planes of the iteration before:
//   B1(s)    E(s) at the cell, i+1, j+1 (the tile box), E(s+1) (registers)
//   E1(s+1)  B1(s+1) at i-1, j-1 (exchange X1), B1(s+1), B1(s) (registers)
//   B2(s+2)  E1(s+2) at i+1, j+1 (exchange X2), E1(s+2), E1(s+3) (registers)
//   E2(s+3)  B2(s+3) at i-1, j-1 (exchange X3), B2(s+3), B2(s+2) (registers)
// The boxes reach two cells past the tile, so the sweep reads the second
// ring of ghost cells (x = -2, Ni+1; y = -2, Nj+1), which launch_refresh_ghosts
// rewrites from the grid before every depth-2 sweep (the one-step kernels
// keep only the first ring current).
#include "arith.cuh"
#include "engine_internal.h"
#include "sources.cuh"
#include "tma.cuh"

#include <type_traits>

namespace fdtd {

namespace {

// ---------------------------------------------------------------------------
// Ghost refresh: both rings of periodic copies of one padded array, plane by
// plane (block (z, array)): the four ghost columns of every grid row, then
// the four ghost rows over their whole width (corners included).

__device__ __forceinline__ int wrap_any(int v, int n) {
  v %= n;
  return v < 0 ? v + n : v;
}

// Whether the periodic window [o, o+n) of an axis of length N meets the m
// consecutive cells a, a+1, .. (taken mod N).
__device__ __forceinline__ bool window_meets_t(int o, int n, int N, int a, int m) {
  int s = wrap_any(a - o, N);
  return s < n || s + m > N;
}

template <class T>
__global__ void __launch_bounds__(256) refresh_ghosts_kernel(PLayout L, GhostArrays arrays) {
  T* a = static_cast<T*>(arrays.p[blockIdx.y]);
  const int z = blockIdx.x;
  // ghost columns x = -2, -1, Ni, Ni+1 of the grid rows
  for (int q = threadIdx.x; q < 4 * L.Nj; q += blockDim.x) {
    const int y = q >> 2, g = q & 3;
    const int x = g < 2 ? g - 2 : L.Ni + g - 2;
    a[L.at(x, y, z)] = a[L.at(wrap_any(x, L.Ni), y, z)];
  }
  __syncthreads();
  // ghost rows y = -2, -1, Nj, Nj+1 over x = -2 .. Ni+1
  const int w = L.Ni + 4;
  for (int q = threadIdx.x; q < 4 * w; q += blockDim.x) {
    const int g = q / w, x = q - g * w - 2;
    const int y = g < 2 ? g - 2 : L.Nj + g - 2;
    a[L.at(x, y, z)] = a[L.at(x, wrap_any(y, L.Nj), z)];
  }
}

// ---------------------------------------------------------------------------

template <class S> struct ArithOf2 { using type = ArithPlain; };
template <> struct ArithOf2<StoreF32C> { using type = ArithComp; };

constexpr int kStagesT = 3;

// Box columns: all six boxes start kOff (kLoOff) columns left of the tile,
// on a 16-byte boundary, and reach x0+33 (E at i+1 of the column x0+32).
template <class S> struct BoxT;
template <> struct BoxT<StoreF32> { static constexpr int kW = 40, kOff = 4, kLoW = 0, kLoOff = 0; };
template <> struct BoxT<StoreF32C> { static constexpr int kW = 40, kOff = 4, kLoW = 48, kLoOff = 8; };
template <> struct BoxT<StoreF16> { static constexpr int kW = 48, kOff = 8, kLoW = 0, kLoOff = 0; };

constexpr int r128(int b) { return (b + 127) / 128 * 128; }

// Shared-memory plan (byte offsets).  Box rows: Ex and Ez y0-2 .. y0+RY+1
// (B1 reads them at j+1), the others y0-2 .. y0+RY.  Exchange planes, per
// component, hi words then lo words:
//   X1  B1 at x in [-2, 33), y in [-2, RY]: (RY+3) rows of 36, index (y+2)*36 + x+2
//   X2  E1 at x in [-1, 33), y in [-1, RY]: (RY+2) rows of 36, index (y+1)*36 + x+1
//   X3  B2: the tile (y*32 + x), then row y = -1 (RY*32 + x), then column
//       x = -1 ((RY+1)*32 + y+1); its first RY rows are B2's store box
//   E2s E2 store box: RY rows of 32
template <class S, int RY>
struct PlanT {
  using HiT = typename S::HiT;
  static constexpr bool kLo = S::kComp;
  static constexpr int HS = (int)sizeof(HiT), LS = (int)sizeof(LoT);
  static constexpr int W = BoxT<S>::kW, LW = BoxT<S>::kLoW, OFF = BoxT<S>::kOff, LOFF = BoxT<S>::kLoOff;
  template <int c> static constexpr int kRows = (c == 0 || c == 2) ? RY + 4 : RY + 3;
  static constexpr int kHiBox(int c) { return r128(((c == 0 || c == 2) ? RY + 4 : RY + 3) * W * HS); }
  static constexpr int kLoBox(int c) { return kLo ? r128(((c == 0 || c == 2) ? RY + 4 : RY + 3) * LW * LS) : 0; }
  static constexpr int hi_at(int c) { return c == 0 ? 0 : hi_at(c - 1) + kHiBox(c - 1); }
  static constexpr int lo_at(int c) { return c == 0 ? hi_at(6) : lo_at(c - 1) + kLoBox(c - 1); }
  template <int c> static constexpr int kHiAt = hi_at(c);
  template <int c> static constexpr int kLoAt = lo_at(c);
  static constexpr int kStage = lo_at(6);
  static constexpr uint32_t tx_bytes() {
    uint32_t t = 0;
    for (int c = 0; c < 6; ++c)
      t += (uint32_t)(((c == 0 || c == 2) ? RY + 4 : RY + 3) * (W * HS + (kLo ? LW * LS : 0)));
    return t;
  }
  static constexpr uint32_t kTx = tx_bytes();
  // exchange planes (elements per component) and their byte sizes
  static constexpr int kX1 = (RY + 3) * 36, kX2 = (RY + 2) * 36, kX3 = (RY + 2) * 32, kE2 = RY * 32;
  static constexpr int bytes(int n) { return r128(3 * n * HS) + (kLo ? r128(3 * n * LS) : 0); }
  static constexpr int kRing = 0;
  static constexpr int kX1At = kStagesT * kStage;
  static constexpr int kX2At = kX1At + 2 * bytes(kX1);
  static constexpr int kX3At = kX2At + 2 * bytes(kX2);
  static constexpr int kE2At = kX3At + 2 * bytes(kX3);
  static constexpr int kBar = kE2At + 2 * bytes(kE2);
  static constexpr int kList = kBar + kStagesT * 8;
  static constexpr int kTotal = kList + 4 * (kMaxSources + 1);
  static_assert(RY + 3 <= 32, "the halo columns' lanes cover y = -2 .. RY");
  static_assert((W * HS) % 16 == 0 && (LW * LS) % 16 == 0, "box rows must be whole 16-byte units");
  static_assert(W - OFF >= 34 && (!kLo || LW - LOFF >= 34), "boxes must reach x0+33");
  static_assert((kE2 * HS) % 128 == 0 && (kE2 * LS) % 128 == 0 && (kX3 * HS) % 128 == 0 && (kX3 * LS) % 128 == 0,
                "store boxes must start on 128-byte boundaries");
};

// One depth-2 tile: columns bx*32 .., rows by*RY .., planes bz*kchunk ..
// Returns false when a bounded wait gave up (uniform over the CTA).
template <class S, class A, int RY, int kApps1, bool kDenseJ>
__device__ __forceinline__ bool tblock_tile(const PLayout& L, const S& st, const S& out, const StepMaps& maps,
                                            const CoefSet& cs, int bx, int by, int bz, int kchunk,
                                            const float* __restrict__ Jx, const float* __restrict__ Jy,
                                            const float* __restrict__ Jz, const SourceSet& ss, int64_t step,
                                            const WaitCtl& wc, unsigned char* smem) {
  using P = PlanT<S, RY>;
  using HiT = typename S::HiT;
  using T = typename A::Cur;
  constexpr int NS = kStagesT;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + P::kBar);
  int* list = reinterpret_cast<int*>(smem + P::kList);

  const int lane = threadIdx.x, w = threadIdx.y;
  const int x0 = bx * 32, y0 = by * RY;
  const int nx = min(32, L.Ni - x0), ny = min(RY, L.Nj - y0);
  // the thread's cell in tile coordinates
  int cx, cy;
  if (w < RY) {
    cx = lane;
    cy = w;
  } else if (w < RY + 3) {
    cx = lane;
    cy = w == RY ? -1 : w == RY + 1 ? -2 : RY;
  } else {
    cx = w == RY + 3 ? -1 : w == RY + 4 ? -2 : 32;
    cy = lane - 2;
  }
  const bool b1 = cx >= -2 && cx <= nx && cy >= -2 && cy <= ny;
  const bool e1 = cx >= -1 && cx <= nx && cy >= -1 && cy <= ny;
  const bool b2 = cx >= -1 && cx < nx && cy >= -1 && cy < ny;
  const bool e2 = cx >= 0 && cx < nx && cy >= 0 && cy < ny;
  // unwrapped grid coordinates of the cell (E2 cells are grid cells), and
  // the grid cell it is a copy of (E1 is also computed on halo cells, which
  // take the current of the cells they copy)
  const int xu = x0 + cx, yu = y0 + cy;
  const int xl = wrap_any(xu, L.Ni), yl = wrap_any(yu, L.Nj);
  const int k0 = bz * kchunk;
  const int k1 = min(k0 + kchunk, L.Nk);
  const int n_it = k1 - k0 + 4;  // planes k1 .. k0-3
  const bool leader = (w == RY + 4 && lane == 0);  // column x = -2: the least arithmetic
  const bool tma_out = (nx == 32);
  const bool edge_cell = e2 && (xu == 0 || xu == L.Ni - 1 || yu == 0 || yu == L.Nj - 1);
  // clamped cell (every thread reads its box and exchange slots in range)
  const int qx = max(-2, min(cx, 32)), qy = max(-2, min(cy, RY));

  auto wrapk = [&](int k) { return k < 0 ? (k % L.Nk + L.Nk) % L.Nk : (k >= L.Nk ? k % L.Nk : k); };

  int issued = 0;
  auto issue = [&](int it) {  // ring fill `it`: plane k1 - it
    if (wc.withhold) return;
    ++issued;
    const int kk = wrapk(k1 - it);
    const int slot = it % NS;
    unsigned char* base = smem + P::kRing + slot * P::kStage;
    mbar_arrive_expect_tx(&bar[slot], P::kTx);
    // box row 0 is logical row y0-2: padded row y0 - 2 + kPadY
    const int yb = y0 - 2 + kPadY;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      tma_load_3d(base + P::hi_at(c), &maps.ld.hi[c], x0 + kPadX - P::OFF, yb, kk, &bar[slot]);
      if (P::kLo) tma_load_3d(base + P::lo_at(c), &maps.ld.lo[c], x0 + kPadX - P::LOFF, yb, kk, &bar[slot]);
    }
  };
  if (leader)
    for (int it = 0; it < n_it && it < NS; ++it) issue(it);

  // per-column factors (amp gx) gy of the first listed sources for both
  // steps' time indices
  T sxy[2][kFastSources];
  unsigned smask = 0;
#pragma unroll
  for (int q = 0; q < kFastSources; ++q) {
    sxy[0][q] = sxy[1][q] = A::cur_zero();
    if (q < list[kMaxSources]) {
      const DevSource& d = ss.src[list[q]];
      const int di = box_offset(xl, d.i0, d.ni, L.Ni);
      const int dj = box_offset(yl, d.j0, d.nj, L.Nj);
      if (e1 && di >= 0 && dj >= 0) {
#pragma unroll
        for (int h = 0; h < 2; ++h)
          if (step + h < d.n_amp)
            sxy[h][q] = A::cur_mul(A::cur_mul(A::cur_table(ss, d.amp_off + step + h), A::cur_table(ss, d.gx_off + di)),
                                   A::cur_table(ss, d.gy_off + dj));
        smask |= 1u << q;
      }
    }
  }
  const int nsrc = list[kMaxSources];

  // J term of the E updates of the cell (grid cell xl, yl) at plane ke
  // (0 <= ke < Nk), time index step + h
  auto add_current_terms = [&](Pair& qx_, Pair& qy_, Pair& qz_, int ke, int h) {
    if (!(kDenseJ || nsrc > 0)) return;
    T jv[3] = {A::cur_zero(), A::cur_zero(), A::cur_zero()};
    unsigned has = 0;
    if (kDenseJ) {
      const int64_t d = xl + (int64_t)yl * L.Ni + (int64_t)ke * L.Ni * L.Nj;
      jv[0] = A::cur_dense(Jx[d]);
      jv[1] = A::cur_dense(Jy[d]);
      jv[2] = A::cur_dense(Jz[d]);
      has = 7u;
    }
    const int64_t sh = step + h;
#pragma unroll
    for (int q = 0; q < kFastSources; ++q) {
      if (q < nsrc) {
        const DevSource& d = ss.src[list[q]];
        const int dk = box_offset(ke, d.k0, d.nk, L.Nk);
        if (dk >= 0 && (smask >> q & 1u) && sh < d.n_amp) {
          add_current<A>(jv, d.comp_mask, A::cur_mul(sxy[h][q], A::cur_table(ss, d.gz_off + dk)), has);
          has |= (unsigned)d.comp_mask;
        }
      }
    }
    for (int i = kFastSources; i < nsrc; ++i) {
      const DevSource& d = ss.src[list[i]];
      if (sh >= d.n_amp) continue;
      const int dk = box_offset(ke, d.k0, d.nk, L.Nk);
      if (dk < 0) continue;
      const int di = box_offset(xl, d.i0, d.ni, L.Ni);
      const int dj = box_offset(yl, d.j0, d.nj, L.Nj);
      if (di >= 0 && dj >= 0) {
        add_current<A>(jv, d.comp_mask,
                       A::cur_mul(A::cur_mul(A::cur_mul(A::cur_table(ss, d.amp_off + sh), A::cur_table(ss, d.gx_off + di)),
                                             A::cur_table(ss, d.gy_off + dj)),
                                  A::cur_table(ss, d.gz_off + dk)),
                       has);
        has |= (unsigned)d.comp_mask;
      }
    }
    if (has & 1u) qx_ = A::add(qx_, A::cur_term(jcoef<S>(cs, st, 0), jv[0]));
    if (has & 2u) qy_ = A::add(qy_, A::cur_term(jcoef<S>(cs, st, 1), jv[1]));
    if (has & 4u) qz_ = A::add(qz_, A::cur_term(jcoef<S>(cs, st, 2), jv[2]));
  };

  // registers: E(s+1) of the cell; B1(s+1), B1(s+2); E1(s+2), E1(s+3); B2(s+3)
  const Pair zero{0.f, 0.f};
  Pair eu[3] = {zero, zero, zero};
  Pair b1p1[3] = {zero, zero, zero}, b1p2[3] = {zero, zero, zero};
  Pair e1p1[3] = {zero, zero, zero}, e1p2[3] = {zero, zero, zero};
  Pair b2p1[3] = {zero, zero, zero};
  if (b1) {
    const int64_t e0 = L.at(xu, yu, wrapk(k1 + 1));
    eu[0] = st.load(0, e0);
    eu[1] = st.load(1, e0);
  }

  // exchange accessors (component c of buffer `at`, element index i)
  auto xput = [&](int at, int n, int c, int i, Pair v, int comp) {
    HiT* h = reinterpret_cast<HiT*>(smem + at);
    h[c * n + i] = st.enc_hi(comp, v);
    if (P::kLo) reinterpret_cast<LoT*>(smem + at + r128(3 * n * P::HS))[c * n + i] = st.enc_lo(v);
  };
  auto xget = [&](int at, int n, int c, int i, int comp) -> Pair {
    const HiT* h = reinterpret_cast<const HiT*>(smem + at);
    const LoT q = P::kLo ? reinterpret_cast<const LoT*>(smem + at + r128(3 * n * P::HS))[c * n + i] : LoT(0);
    return st.decode(comp, h[c * n + i], q);
  };
  auto q3 = [&](Pair v, int comp) { return st.decode(comp, st.enc_hi(comp, v), st.enc_lo(v)); };

  for (int it = 0; it < n_it; ++it) {
    const int s = k1 - it;
    const int slot = it % NS;
    const uint32_t phase = (uint32_t)(it / NS) & 1u;
    const int cur = it & 1, prv = cur ^ 1;
    const bool timed_out = !mbar_wait_bounded(&bar[slot], phase, wc);
    const unsigned char* stage = smem + P::kRing + slot * P::kStage;
    auto V = [&](int c, int dr, int dc) -> Pair {
      const int row = qy + 2 + dr, col = qx + P::OFF + dc;
      const HiT h = reinterpret_cast<const HiT*>(stage + P::hi_at(c))[row * P::W + col];
      const LoT q = P::kLo ? reinterpret_cast<const LoT*>(stage + P::lo_at(c))[row * P::LW + (qx + P::LOFF + dc)]
                           : LoT(0);
      return st.decode(c, h, q);
    };
    const int x1at = P::kX1At + cur * P::bytes(P::kX1), x1pv = P::kX1At + prv * P::bytes(P::kX1);
    const int x2at = P::kX2At + cur * P::bytes(P::kX2), x2pv = P::kX2At + prv * P::bytes(P::kX2);
    const int x3at = P::kX3At + cur * P::bytes(P::kX3), x3pv = P::kX3At + prv * P::bytes(P::kX3);
    const int e2at = P::kE2At + cur * P::bytes(P::kE2);

    // ---- B1(s) ----
    const Pair ex = V(0, 0, 0), ey = V(1, 0, 0), ez = V(2, 0, 0);
    Pair nb1[3];
    {
      Pair u[3];
      u[0] = A::curl(bcoef<S>(cs, st, 0, 0), eu[1], ey, bcoef<S>(cs, st, 0, 1), V(2, 1, 0), ez);
      u[1] = A::curl(bcoef<S>(cs, st, 1, 0), V(2, 0, 1), ez, bcoef<S>(cs, st, 1, 1), eu[0], ex);
      u[2] = A::curl(bcoef<S>(cs, st, 2, 0), V(0, 1, 0), ex, bcoef<S>(cs, st, 2, 1), V(1, 0, 1), ey);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (kApps1 == 2) u[c] = A::twice(u[c]);
        nb1[c] = q3(A::acc_curl(V(3 + c, 0, 0), u[c]), 3 + c);
      }
    }
    if (b1 && s >= k0 - 2)
#pragma unroll
      for (int c = 0; c < 3; ++c) xput(x1at, P::kX1, c, (cy + 2) * 36 + cx + 2, nb1[c], 3 + c);

    // ---- E1(s+1) ----
    Pair ne1[3] = {zero, zero, zero};
    if (e1 && it >= 1 && s >= k0 - 2) {
      const int ixl = (qy + 2) * 36 + qx + 1, ixd = (qy + 1) * 36 + qx + 2;  // (x-1, y), (x, y-1) in X1
      Pair q[3];
      q[0] = A::curl(ecoef<S>(cs, st, 0, 0), b1p1[2], xget(x1pv, P::kX1, 2, ixd, 5), ecoef<S>(cs, st, 0, 1), b1p1[1],
                     nb1[1]);
      q[1] = A::curl(ecoef<S>(cs, st, 1, 0), b1p1[0], nb1[0], ecoef<S>(cs, st, 1, 1), b1p1[2],
                     xget(x1pv, P::kX1, 2, ixl, 5));
      q[2] = A::curl(ecoef<S>(cs, st, 2, 0), b1p1[1], xget(x1pv, P::kX1, 1, ixl, 4), ecoef<S>(cs, st, 2, 1), b1p1[0],
                     xget(x1pv, P::kX1, 0, ixd, 3));
      add_current_terms(q[0], q[1], q[2], wrapk(s + 1), 0);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        ne1[c] = q3(A::acc(eu[c], q[c]), c);
        xput(x2at, P::kX2, c, (cy + 1) * 36 + cx + 1, ne1[c], c);
      }
    }

    // ---- B2(s+2) ----
    Pair nb2[3] = {zero, zero, zero};
    if (b2 && it >= 3 && s <= k1 - 3) {
      const int ixr = (qy + 1) * 36 + qx + 2, ixu = (qy + 2) * 36 + qx + 1;  // (x+1, y), (x, y+1) in X2
      Pair u[3];
      u[0] = A::curl(bcoef<S>(cs, st, 0, 0), e1p2[1], e1p1[1], bcoef<S>(cs, st, 0, 1), xget(x2pv, P::kX2, 2, ixu, 2),
                     e1p1[2]);
      u[1] = A::curl(bcoef<S>(cs, st, 1, 0), xget(x2pv, P::kX2, 2, ixr, 2), e1p1[2], bcoef<S>(cs, st, 1, 1), e1p2[0],
                     e1p1[0]);
      u[2] = A::curl(bcoef<S>(cs, st, 2, 0), xget(x2pv, P::kX2, 0, ixu, 0), e1p1[0], bcoef<S>(cs, st, 2, 1),
                     xget(x2pv, P::kX2, 1, ixr, 1), e1p1[1]);
      const int i3 = cy < 0 ? (cx < 0 ? (RY + 1) * 32 : RY * 32 + cx) : (cx < 0 ? (RY + 1) * 32 + cy + 1 : cy * 32 + cx);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        nb2[c] = q3(A::acc_curl(b1p2[c], A::twice(u[c])), 3 + c);
        xput(x3at, P::kX3, c, i3, nb2[c], 3 + c);
      }
    }

    // ---- E2(s+3) ----
    Pair ne2[3] = {zero, zero, zero};
    if (e2 && it >= 4) {
      const int il = cx == 0 ? (RY + 1) * 32 + cy + 1 : cy * 32 + cx - 1;
      const int id = cy == 0 ? RY * 32 + cx : (cy - 1) * 32 + cx;
      Pair q[3];
      q[0] = A::curl(ecoef<S>(cs, st, 0, 0), b2p1[2], xget(x3pv, P::kX3, 2, id, 5), ecoef<S>(cs, st, 0, 1), b2p1[1],
                     nb2[1]);
      q[1] = A::curl(ecoef<S>(cs, st, 1, 0), b2p1[0], nb2[0], ecoef<S>(cs, st, 1, 1), b2p1[2],
                     xget(x3pv, P::kX3, 2, il, 5));
      q[2] = A::curl(ecoef<S>(cs, st, 2, 0), b2p1[1], xget(x3pv, P::kX3, 1, il, 4), ecoef<S>(cs, st, 2, 1), b2p1[0],
                     xget(x3pv, P::kX3, 0, id, 3));
      add_current_terms(q[0], q[1], q[2], wrapk(s + 3), 1);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        ne2[c] = A::acc(e1p2[c], q[c]);
        xput(e2at, P::kE2, c, cy * 32 + cx, ne2[c], c);
      }
    }
    const bool st_b2 = it >= 3 && s + 2 >= k0 && s + 2 < k1;  // B2(s+2) is an owned plane
    const bool st_e2 = it >= 4 && s + 3 >= k0;                 // E2(s+3) is
    if (e2 && (!tma_out || edge_cell)) {
      const int64_t o = L.at(xu, yu, 0);
      for (int c = 0; c < 3; ++c) {
        if (st_b2) {
          if (!tma_out) out.store(3 + c, o + (int64_t)(s + 2) * L.pplane, nb2[c]);
          if (edge_cell) store_ghost_copies(out, L, 3 + c, xu, yu, s + 2, nb2[c]);
        }
        if (st_e2) {
          if (!tma_out) out.store(c, o + (int64_t)(s + 3) * L.pplane, ne2[c]);
          if (edge_cell) store_ghost_copies(out, L, c, xu, yu, s + 3, ne2[c]);
        }
      }
    }

    // rotate the registers
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      b2p1[c] = nb2[c];
      e1p2[c] = e1p1[c];
      e1p1[c] = ne1[c];
      b1p2[c] = b1p1[c];
      b1p1[c] = nb1[c];
    }
    eu[0] = ex;
    eu[1] = ey;
    eu[2] = ez;
    fence_async_smem();
    if (leader) bulk_wait_read_all();
    if (__syncthreads_or(timed_out)) {
      if (leader) {
        for (int f = it; f < issued; ++f) mbar_wait_bounded(&bar[f % NS], (uint32_t)(f / NS) & 1u, wc, 2);
        bulk_wait_all();
      }
      return false;
    }
    if (leader) {
      if (tma_out) {
        if (st_b2)
          for (int c = 0; c < 3; ++c) {
            tma_store_3d(&maps.st.hi[3 + c], smem + x3at + c * P::kX3 * P::HS, x0 + kPadX, y0, s + 2);
            if (P::kLo)
              tma_store_3d(&maps.st.lo[3 + c], smem + x3at + r128(3 * P::kX3 * P::HS) + c * P::kX3 * P::LS,
                           x0 + kPadX, y0, s + 2);
          }
        if (st_e2)
          for (int c = 0; c < 3; ++c) {
            tma_store_3d(&maps.st.hi[c], smem + e2at + c * P::kE2 * P::HS, x0 + kPadX, y0, s + 3);
            if (P::kLo)
              tma_store_3d(&maps.st.lo[c], smem + e2at + r128(3 * P::kE2 * P::HS) + c * P::kE2 * P::LS,
                           x0 + kPadX, y0, s + 3);
          }
      }
      bulk_commit();
      if (it + NS < n_it) issue(it + NS);
    }
  }
  if (leader) bulk_wait_all();
  return true;
}

template <class S, class A, int RY, int kApps1, bool kDenseJ>
__global__ void __launch_bounds__(32 * (RY + 6), 1)
    tblock2(PLayout L, S st, S out, const __grid_constant__ StepMaps maps, CoefSet cs, int kchunk,
            const float* __restrict__ Jx, const float* __restrict__ Jy, const float* __restrict__ Jz, SourceSet ss,
            int64_t step, WaitCtl wc) {
  using P = PlanT<S, RY>;
  extern __shared__ __align__(128) unsigned char smem[];
  int* list = reinterpret_cast<int*>(smem + P::kList);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    for (int q = 0; q < kStagesT; ++q) mbar_init(reinterpret_cast<uint64_t*>(smem + P::kBar) + q, 1);
    mbar_init_fence();
  }
  // sources that can reach the cells where E is updated (the E1 region:
  // one cell around the tile), for either time index
  if (threadIdx.y == 0) {
    const int lane = threadIdx.x;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * RY;
    const int nx = min(32, L.Ni - x0), ny = min(RY, L.Nj - y0);
    int n = 0;
    for (int b = 0; b < ss.count; b += 32) {
      const int q = b + lane;
      bool hit = false;
      if (q < ss.count) {
        const DevSource& d = ss.src[q];
        hit = step < d.n_amp && window_meets_t(d.i0, d.ni, L.Ni, x0 - 1, nx + 2) &&
              window_meets_t(d.j0, d.nj, L.Nj, y0 - 1, ny + 2);
      }
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if (hit) list[n + __popc(m & ((1u << lane) - 1u))] = q;
      n += __popc(m);
    }
    if (lane == 0) list[kMaxSources] = n;
  }
  __syncthreads();
  tblock_tile<S, A, RY, kApps1, kDenseJ>(L, st, out, maps, cs, blockIdx.x, blockIdx.y, blockIdx.z, kchunk, Jx, Jy, Jz,
                                         ss, step, wc, smem);
}

template <class S, int RY, int APPS, bool DJ>
cudaError_t launch_t_one(dim3 grid, const PLayout& L, const S& st, const S& out, const StepMaps& maps,
                         const CoefSet& cs, int kchunk, const float* const J[3], const SourceSet& ss, int64_t step,
                         const WaitCtl& wc, cudaStream_t stream) {
  using A = typename ArithOf2<S>::type;
  auto kern = tblock2<S, A, RY, APPS, DJ>;
  const int bytes = PlanT<S, RY>::kTotal;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  kern<<<grid, dim3(32, RY + 6), bytes, stream>>>(L, st, out, maps, cs, kchunk, J[0], J[1], J[2], ss, step, wc);
  return cudaGetLastError();
}

template <class S, int RY>
cudaError_t launch_t_ry(const PLayout& L, const S& st, const S& out, const StepMaps& maps, const float* const J[3],
                        bool dense_j, const CoefSet& cs, const SourceSet& ss, int64_t step, int apps1, int kchunk,
                        const WaitCtl& wc, cudaStream_t stream) {
  if (ss.count > kMaxSources) return cudaErrorInvalidValue;
  dim3 grid((L.Ni + 31) / 32, (L.Nj + RY - 1) / RY, (L.Nk + kchunk - 1) / kchunk);
#define FDTD_T(APPS, DJ) return launch_t_one<S, RY, APPS, DJ>(grid, L, st, out, maps, cs, kchunk, J, ss, step, wc, stream)
  if (apps1 == 2) {
    if (dense_j) FDTD_T(2, true);
    FDTD_T(2, false);
  }
  if (dense_j) FDTD_T(1, true);
  FDTD_T(1, false);
#undef FDTD_T
}

}  // namespace

cudaError_t launch_refresh_ghosts(const PLayout& L, const GhostArrays& arrays, int elem_bytes, cudaStream_t stream) {
  dim3 grid(L.Nk, 6);
  if (elem_bytes == 4)
    refresh_ghosts_kernel<uint32_t><<<grid, 256, 0, stream>>>(L, arrays);
  else
    refresh_ghosts_kernel<uint16_t><<<grid, 256, 0, stream>>>(L, arrays);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_tblock2_f32(const PLayout& L, const S& st, const S& out, const void* maps, const float* const J[3],
                               bool dense_j, const CoefSet& cs, const SourceSet& ss, int64_t step, int apps1,
                               const FusedConfig& cfg, const WaitCtl& wc, cudaStream_t stream) {
  const int kchunk = cfg.kchunk > 0 ? cfg.kchunk : 48;
  const StepMaps& m = *static_cast<const StepMaps*>(maps);
  if (cfg.tile_y == 6)
    return launch_t_ry<S, 6>(L, st, out, m, J, dense_j, cs, ss, step, apps1, kchunk, wc, stream);
  return launch_t_ry<S, 14>(L, st, out, m, J, dense_j, cs, ss, step, apps1, kchunk, wc, stream);
}

template <class S>
void tblock2_box_widths(int hi[6], int lo[6]) {
  for (int c = 0; c < 6; ++c) {
    hi[c] = BoxT<S>::kW;
    lo[c] = BoxT<S>::kLoW;
  }
}

#define FDTD_INSTANTIATE(S)                                                                                   \
  template cudaError_t launch_tblock2_f32<S>(const PLayout&, const S&, const S&, const void*, const float* const[3], \
                                             bool, const CoefSet&, const SourceSet&, int64_t, int, const FusedConfig&, \
                                             const WaitCtl&, cudaStream_t);                                     \
  template void tblock2_box_widths<S>(int[6], int[6]);
FDTD_INSTANTIATE(StoreF32)
FDTD_INSTANTIATE(StoreF32C)
FDTD_INSTANTIATE(StoreF16)
#undef FDTD_INSTANTIATE

}  // namespace fdtd
