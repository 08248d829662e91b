// Declarations shared between the C-ABI layer (engine.cu) and the kernel
// translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "common.cuh"
#include "layout.cuh"
#include "storage.cuh"
#include "tma.cuh"

namespace fdtd {

struct Fp64Fields {
  double* f[9];  // EX..JZ
};

struct CoefSet {
  Coef cb[3];   // C dt / (2 d) per axis, split hi + lo
  Coef ce[3];   // C dt / d per axis
  Coef cj;      // -4 pi dt
  double cj64;  // -4 pi dt in FP64 (current term of the compensated form)
};

// The axis and the source component of term t of component c's update
// (kokkos_functors.h:64-90 for E, :128-151 for B):
//   Ex: cy (Bz - Bz[j-1]) - cz (By - By[k-1])     Bx: cz (Ey[k+1] - Ey) - cy (Ez[j+1] - Ez)
//   Ey: cz (Bx - Bx[k-1]) - cx (Bz - Bz[i-1])     By: cx (Ez[i+1] - Ez) - cz (Ex[k+1] - Ex)
//   Ez: cx (By - By[i-1]) - cy (Bx - Bx[j-1])     Bz: cy (Ex[j+1] - Ex) - cx (Ey[i+1] - Ey)
__host__ __device__ constexpr int term_axis(int c, int t) {
  return c == 0 ? (t == 0 ? 1 : 2) : c == 1 ? (t == 0 ? 2 : 0) : (t == 0 ? 0 : 1);
}
__host__ __device__ constexpr int e_term_src(int c, int t) {  // a B component
  return c == 0 ? (t == 0 ? 5 : 4) : c == 1 ? (t == 0 ? 3 : 5) : (t == 0 ? 4 : 3);
}
__host__ __device__ constexpr int b_term_src(int c, int t) { return term_axis(c, t); }  // an E component

// The coefficient a kernel of storage form S multiplies term t of component
// c's update by: the per-axis set of CoefSet, except in the FP16 form, whose
// kernels compute on stored (scaled) values with the per-term coefficients
// its store carries (StoreF16::te, tb, tj).
template <class S>
__device__ __forceinline__ Coef ecoef(const CoefSet& cs, const S& st, int c, int t) {
  if constexpr (std::is_same<S, StoreF16>::value) return Coef{st.te[2 * c + t], 0.f};
  else return cs.ce[term_axis(c, t)];
}
template <class S>
__device__ __forceinline__ Coef bcoef(const CoefSet& cs, const S& st, int c, int t) {
  if constexpr (std::is_same<S, StoreF16>::value) return Coef{st.tb[2 * c + t], 0.f};
  else return cs.cb[term_axis(c, t)];
}
template <class S>
__device__ __forceinline__ Coef jcoef(const CoefSet& cs, const S& st, int c) {
  if constexpr (std::is_same<S, StoreF16>::value) return Coef{st.tj[c], 0.f};
  else return cs.cj;
}


// Launch shape of the fused step kernel: interior tile rows (14 or 6) and
// planes per tile.
struct FusedConfig {
  int depth = 1;     // steps per sweep: 1, or 2 (temporal blocking, kernels_tblock.cu)
  int tile_y = 14;
  int kchunk = 48;  // planes per tile (the autotuner picks from 16 to 96)
  int cells_per_thread = 1;  // 1: 32-wide tiles (kernels_fused1.cu); 2: 64-wide, packed float2
  // Batched sweep only: compile the plane loop with and without source
  // evaluation and run the source-free copy on tiles no source reaches.
  bool split_sources = false;
};

// A box of cells [i0,i1) x [j0,j1) x [k0,k1) (the ranges the reference's
// functors take, kokkos_functors.h:45-63 and :109-127).
struct Box {
  int i0, i1, j0, j1, k0, k1;
  __host__ __device__ bool empty() const { return i1 <= i0 || j1 <= j0 || k1 <= k0; }
  static Box whole(const Grid& g) { return Box{0, g.Ni, 0, g.Nj, 0, g.Nk}; }
};

// kernels_fp64.cu: the FP64 sweeps over a box; fma selects the contracted
// arithmetic (otherwise the reference's, bit for bit).
cudaError_t launch_b_fp64(const Grid& g, const Box& box, const Fp64Fields& F, const double cb[3],
                          int applications, bool fma, cudaStream_t st);
cudaError_t launch_e_fp64(const Grid& g, const Box& box, const Fp64Fields& F, const double ce[3], double cJ,
                          bool dense_j, const SourceSet& ss, int64_t step, bool fma, cudaStream_t st);

// kernels_pml.cu: the split-field layer updates (FP64) over a box.  split =
// Exy, Exz, Eyx, Eyz, Ezx, Ezy, Bxy, Bxz, Byx, Byz, Bzx, Bzy; decay[a][n] =
// exp(-sigma_a(n) c dt) and coef2[a][n] the curl coefficient along axis a,
// tables on the device.
struct PmlFields {
  double* split[12];
  const double* decay[3];
  const double* coef2[3];
};
cudaError_t launch_e_pml_fp64(const Grid& g, const Box& box, const Fp64Fields& F, const PmlFields& P,
                              cudaStream_t st);
cudaError_t launch_b_pml_fp64(const Grid& g, const Box& box, const Fp64Fields& F, const PmlFields& P,
                              cudaStream_t st);

// kernels_f32.cu (padded layout): the sweeps over planes [kbeg, kend).
template <class S>
cudaError_t launch_b_f32(const PLayout& L, const S& st, const CoefSet& cs, int applications, int kbeg, int kend,
                         cudaStream_t stream);
// One B half step of planes [kbeg, kend) from the state `st` (E and B) into
// the B arrays of `out`, which must not alias st's.
template <class S>
cudaError_t launch_b_f32_into(const PLayout& L, const S& st, const S& out, const CoefSet& cs, int kbeg, int kend,
                              cudaStream_t stream);
template <class S>
cudaError_t launch_e_f32(const PLayout& L, const S& st, const float* const J[3], bool dense_j,
                         const CoefSet& cs, const SourceSet& ss, int64_t step, int kbeg, int kend,
                         cudaStream_t stream);
// Reads the state from `st` (through the TMA maps in `maps`, a TmaMaps
// built by build_tma_maps for `st`'s arrays), writes the stepped state to `out`.
template <class S>
cudaError_t launch_fused_f32(const PLayout& L, const S& st, const S& out, const void* maps,
                             const float* const J[3], bool dense_j, const CoefSet& cs,
                             const SourceSet& ss, int64_t step, int applications,
                             const FusedConfig& cfg, const WaitCtl& wc, cudaStream_t stream);
template <class S>
int fused_box_width();
int fused_lo_box_width();
// kernels_fused1.cu: the B-first sweep (B half steps, then E) with one cell
// per thread (32-wide tiles); `maps` is a StepMaps: load maps of `st`'s
// arrays (BoxTrim::BFirst), store maps of `out`'s.  [kbeg, kend) are the
// planes it updates (kend < 0: Nk); a z slab's storage sweeps [1, nk+1) and
// reads its halo planes 0 and nk+1 unwrapped.
template <class S>
cudaError_t launch_fused1_f32(const PLayout& L, const S& st, const S& out, const void* maps,
                              const float* const J[3], bool dense_j, const CoefSet& cs,
                              const SourceSet& ss, int64_t step, int applications,
                              const FusedConfig& cfg, const WaitCtl& wc, cudaStream_t stream,
                              int kbeg = 0, int kend = -1);
// Per-component box widths (hi and lo words) of the one-cell kernel's load
// maps.
template <class S>
void fused1_box_widths(int hi[6], int lo[6]);
// kernels_fused1.cu: `applications` B half steps alone over planes
// [kbeg, kend) (kend < 0: Nk), from `st` into `out` (which may be `st`), with
// the fused sweep's tiles (32 x cfg.tile_y, cfg.kchunk planes) and its load
// and store maps (`maps`: a StepMaps built for that tile height).
template <class S>
cudaError_t launch_bhalf_f32(const PLayout& L, const S& st, const S& out, const void* maps, const CoefSet& cs,
                             int applications, const FusedConfig& cfg, const WaitCtl& wc, cudaStream_t stream,
                             int kbeg = 0, int kend = -1);

// kernels_tblock.cu: the depth-2 sweep (two B-first steps per pass; the
// first step applies `apps1` B half steps, the second two) of one cell per
// thread, 32 x tile_y tiles (6 or 14); `maps` is a StepMaps whose load maps
// (BoxTrim::BFirst, tile_y + 2, widths tblock2_box_widths) cover two rings of
// halo.  The input's second ghost ring must be current: launch_refresh_ghosts
// rewrites both rings of six padded arrays (elem_bytes 4 or 2) from the grid.
struct GhostArrays {
  void* p[6];
};
cudaError_t launch_refresh_ghosts(const PLayout& L, const GhostArrays& arrays, int elem_bytes, cudaStream_t stream);
template <class S>
cudaError_t launch_tblock2_f32(const PLayout& L, const S& st, const S& out, const void* maps, const float* const J[3],
                               bool dense_j, const CoefSet& cs, const SourceSet& ss, int64_t step, int apps1,
                               const FusedConfig& cfg, const WaitCtl& wc, cudaStream_t stream);
template <class S>
void tblock2_box_widths(int hi[6], int lo[6]);

// Batched form: one record per domain in device memory (its layout, its two
// state copies, coefficients and sources).
struct StepMaps;
template <class S>
struct BatchDomain {
  PLayout L;
  S s[2];
  CoefSet cs;
  SourceSet ss;
};

// kernels_fused1.cu: one fused sweep over every tile of every domain, as one
// persistent launch.  `doms` is a BatchDomain<S>[n], `maps` has two StepMaps
// per domain (index 2 d + parity: loads of copy parity, stores into the
// other), `tiles` the (domain, bx, by, bz) table; the step index is
// *step_base + step_off; counters (2 ints, zero before the first launch) are
// left at zero.
template <class S>
cudaError_t launch_fused1_batch(const void* doms, const StepMaps* maps, const int4* tiles, int n_tiles, int parity,
                                int applications, const FusedConfig& cfg, const int64_t* step_base, int step_off,
                                int* counters, const WaitCtl& wc, cudaStream_t stream);

// kernels_f32.cu: one B half step of every domain in place on copy `parity`
// (the batch's pending half), as one launch of 32 x 8 blocks marching
// kBatchBChunk planes;
// block_start[d] is the first block of domain d (n_dom + 1 entries).
constexpr int kBatchBChunk = 16;
template <class S>
cudaError_t launch_b_f32_batch(const void* doms, const int64_t* block_start, int n_dom, int64_t n_blocks,
                               int parity, cudaStream_t stream);

// tma_maps.cu: tensor maps of the six hi arrays (and six lo arrays of the
// compensated form) for a fused tile of `tile_y` interior rows.
enum class HiType { F32, F16 };
// Store maps of the fused1 kernel: the grid rows of each array with their x
// margins (x coordinate kPadX + x is cell x), box 32 x tile_y.
cudaError_t build_tma_store_maps(void* maps, const PLayout& L, HiType ht, void* const hi[6], LoT* const lo[6],
                                 int tile_y);
// Box heights of the load maps: None (the two-cell kernel) gives every
// component tile_y + 2 rows; BFirst (the one-cell and depth-2 sweeps) gives
// Ex and Ez tile_y + 2 and the others tile_y + 1 (the row below).
enum class BoxTrim { None, BFirst };
cudaError_t build_tma_maps(void* maps, const PLayout& L, HiType ht, void* const hi[6],
                           LoT* const lo[6], const int box_w[6], const int lo_box_w[6], int tile_y, BoxTrim trim);

// misc.cu — conversions, diagnostics, small helpers.
enum class Form { F64 = 0, F32 = 1, F32C = 2, F16 = 3 };

struct StateView {
  Form form;
  Grid g;      // logical grid
  PLayout L;   // padded layout of the FP32-arithmetic forms
  double* f64[6];
  StoreF32 s32;
  StoreF32C s32c;
  StoreF16 s16;
};

// Writes component c (0..5) of the state from n FP64 values at `src`, the
// logical cells off .. off+n-1 (flat index i + j*Ni + k*Ni*Nj), ghosts included.
cudaError_t launch_import(const StateView& v, int c, const double* src, int64_t off, int64_t n,
                          cudaStream_t st);
// Reads component c (0..5) of the state as FP64 into `dst` (logical cells).
cudaError_t launch_export(const StateView& v, int c, double* dst, int64_t off, int64_t n,
                          cudaStream_t st);
// Largest |stored value| of each FP16 component (grid cells), as FP32 bit
// patterns in out_dev[6] (device memory; zeroed here first).
cudaError_t launch_f16_absmax(const PLayout& L, const StoreF16& st, unsigned* out_dev, cudaStream_t stream);
// Multiplies n stored FP16 words (n even) by 2^shift, in place.
cudaError_t launch_f16_rescale(__half* v, int64_t n, int shift, cudaStream_t stream);
// FP64 -> FP32 conversion of n values.
cudaError_t launch_to_f32(const double* src, float* dst, int64_t n, cudaStream_t st);
// FP64 -> FP32 hi + FP32 lo (hi + lo carries the FP64 value to ~2^-48).
cudaError_t launch_split_f32(const double* src, float* hi, float* lo, int64_t n, cudaStream_t st);

// Field sums (fdtd_diag order, 10 values) in two passes through `partials`
// (room for `max_blocks` * 10 doubles); the result lands in out_dev[10].
constexpr int kDiagValues = 10;
constexpr int kDiagThreads = 256;
int diag_blocks_for(int64_t cells, int max_blocks);
cudaError_t launch_field_sums(const StateView& v, double* partials, int nblocks, double* out_dev,
                              cudaStream_t st);

}  // namespace fdtd
