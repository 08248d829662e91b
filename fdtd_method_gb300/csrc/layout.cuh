// Padded field layout of the FP32-arithmetic forms.
//
// Each component is stored as a 3-D array with kPadY ghost rows below and
// above the grid in y and a 32-element margin left and right of it in x, so
// that
//   * every x/y neighbour of a grid cell exists in memory (the first ghost
//     row and column on each side hold periodic copies: ghost x = -1 is cell
//     Ni-1, ghost x = Ni is cell 0, likewise in y and at the four corners),
//     and the second ones (x = -2, Ni+1; y = -2, Nj+1) have room for the
//     copies a two-step sweep reads, which it refreshes before it runs;
//   * cell x = 0 of every row starts a 32-byte memory sector for every
//     element size (pitch is a multiple of 32 elements), so the stores of a
//     warp's row segment cover whole sectors (no read-modify-write in L2)
//     and the tile copies start on the 16-byte boundaries TMA requires.
// The writer of a boundary cell also writes its first-ring ghost copies, so
// those are current whenever the cell is.  z is not padded: planes wrap by
// index.
//
// The FP64 drop-in keeps the reference's dense layout i + j*Ni + k*Ni*Nj.
#pragma once

#include <cstdint>

namespace fdtd {

constexpr int kPadX = 32;
constexpr int kPadY = 2;  // ghost rows on each side (padded row = logical row + kPadY)

struct PLayout {
  int Ni, Nj, Nk;
  int64_t pitch;   // elements per padded row
  int64_t pplane;  // elements per padded plane = pitch * (Nj + 2 kPadY)

  __host__ __device__ __forceinline__ int64_t at(int x, int y, int z) const {
    return (int64_t)(x + kPadX) + (int64_t)(y + kPadY) * pitch + (int64_t)z * pplane;
  }
  __host__ __device__ __forceinline__ int64_t elems() const { return pplane * Nk; }

  static PLayout make(int Ni, int Nj, int Nk) {
    PLayout L;
    L.Ni = Ni;
    L.Nj = Nj;
    L.Nk = Nk;
    L.pitch = ((int64_t)Ni + 2 * kPadX + 31) / 32 * 32;
    L.pplane = L.pitch * (Nj + 2 * kPadY);
    return L;
  }
};

// Stores v at every ghost position that mirrors cell (x, y, z).
template <class S, class V>
__device__ __forceinline__ void store_ghost_copies(const S& st, const PLayout& L, int c, int x, int y,
                                                   int z, V v) {
  const bool xl = (x == 0), xh = (x == L.Ni - 1), yl = (y == 0), yh = (y == L.Nj - 1);
  if (!(xl || xh || yl || yh)) return;
  // ghost columns of this row, then the ghost rows (with their corners)
  if (xl) st.store(c, L.at(L.Ni, y, z), v);
  if (xh) st.store(c, L.at(-1, y, z), v);
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    const bool on = b == 0 ? yl : yh;
    if (!on) continue;
    const int yg = b == 0 ? L.Nj : -1;
    st.store(c, L.at(x, yg, z), v);
    if (xl) st.store(c, L.at(L.Ni, yg, z), v);
    if (xh) st.store(c, L.at(-1, yg, z), v);
  }
}

// store_ghost_copies without the ghost column of the cell's own row where a
// bulk copy writes it: x = Ni (cell 0) when `right`, x = -1 (cell Ni-1)
// when `left`.  The ghost rows and their corners are still written.
template <class S, class V>
__device__ __forceinline__ void store_ghost_rows(const S& st, const PLayout& L, bool right, bool left, int c,
                                                 int x, int y, int z, V v) {
  const bool xl = (x == 0), xh = (x == L.Ni - 1), yl = (y == 0), yh = (y == L.Nj - 1);
  if (xl && !right) st.store(c, L.at(L.Ni, y, z), v);
  if (xh && !left) st.store(c, L.at(-1, y, z), v);
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    const bool on = b == 0 ? yl : yh;
    if (!on) continue;
    const int yg = b == 0 ? L.Nj : -1;
    st.store(c, L.at(x, yg, z), v);
    if (xl) st.store(c, L.at(L.Ni, yg, z), v);
    if (xh) st.store(c, L.at(-1, yg, z), v);
  }
}

// Stores v at (x, y, z) and at every ghost position that mirrors it.
template <class S, class V>
__device__ __forceinline__ void store_with_ghosts(const S& st, const PLayout& L, int c, int x, int y,
                                                  int z, V v) {
  st.store(c, L.at(x, y, z), v);
  store_ghost_copies(st, L, c, x, y, z, v);
}

}  // namespace fdtd
