// Internal: the state behind an fdtd_handle, shared by the C-ABI layer
// (engine.cu) and the batched form (batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "../../include/fdtd_gb300.h"
#include "engine_internal.h"
#include "tma.cuh"

namespace fdtd {

struct HostSource {
  fdtd_source s;  // table pointers are not kept
  std::vector<double> gx, gy, gz, amp;
};

// Reports through fdtd_last_error() (defined in engine.cu).
void set_last_error(const std::string& msg);

struct DeviceGuard {
  int prev = 0;
  bool ok = false;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) == cudaSuccess && cudaSetDevice(dev) == cudaSuccess) ok = true;
  }
  ~DeviceGuard() {
    if (ok) cudaSetDevice(prev);
  }
};

}  // namespace fdtd

using namespace fdtd;

struct fdtd_handle {
  fdtd_params p{};
  double dt = 0;
  int precision = 0;
  Form form = Form::F64;
  Grid g{};
  int device = 0;
  // {cEx, cEy, cEz, cBx, cBy, cBz, cJ}, src/FDTD_kokkos/FDTD_kokkos.cpp:45-55
  double coef[7] = {0, 0, 0, 0, 0, 0, 0};
  CoefSet cs{};
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;

  // Storage.  FP64: field[0..8] are double arrays (E, B, J).  Other forms:
  // field[0..5] hold the E/B words of the form, lo[0..5] the compensation
  // words (FP32_COMP), jf[0..2] FP32 current arrays (allocated on first use).
  void* field[9] = {nullptr};
  LoT* lo[6] = {nullptr};
  // Second copy of E/B (and lo) that the fused sweep writes into; swapped
  // with field/lo after every fused step.
  void* alt_field[6] = {nullptr};
  LoT* alt_lo[6] = {nullptr};
  float* jf[3] = {nullptr};
  bool dense_j = false;  // the E update reads the dense J arrays
  bool fp64_fma = false;  // FP64 form: contracted arithmetic (fdtd_set_fp64_arith)
  int fp16_exp[6] = {0, 0, 0, 0, 0, 0};
  // FP16 range checks (fdtd_set_fp16_autoscale): every n steps (0: off) the
  // stored peaks are scanned and components re-encoded around 2^target.
  int fp16_autoscale_every = 0;
  int fp16_autoscale_target = 10;
  int fp16_autoscale_headroom = 5;
  int fp16_autoscale_count = 0;  // steps since the last check

  // Sources.
  std::vector<HostSource> sources;
  DevSource* d_src = nullptr;
  double* d_tables = nullptr;
  float* d_tables_f = nullptr;  // FP32 hi tables, then FP32 lo tables
  int64_t tables_lo_off = 0;
  int source_calls = 0;   // fdtd_add_source calls since the last clear (the index it returns)
  int64_t host_step = 0;  // completed update_fields steps

  // Step pipeline of the FP32-arithmetic forms (FP64 always uses the split
  // sweeps, whose FP64 instruction count is the smallest).
  // PML (FDTD_PML, src/FDTD_kokkos/FDTD_PML_kokkos.cpp): layer thickness per
  // axis, the twelve split fields Exy, Exz, Eyx, Eyz, Ezx, Ezy, Bxy, Bxz, Byx,
  // Byz, Bzx, Bzy, and the per-axis decay / curl-coefficient tables.
  bool pml = false;
  int pml_size[3] = {0, 0, 0};
  double* split[12] = {nullptr};
  double* pml_decay[3] = {nullptr};
  double* pml_coef2[3] = {nullptr};
  // The box the ordinary updates cover: the whole grid, or inside the layer.
  Box main_box() const {
    return Box{pml_size[0], g.Ni - pml_size[0], pml_size[1], g.Nj - pml_size[1], pml_size[2], g.Nk - pml_size[2]};
  }

  // z slab (fdtd_slab_create): the handle owns planes [slab_k0, slab_k0 +
  // g.Nk) of a grid of slab_nk_global planes.  Its arrays hold zhalo (1)
  // more plane below and above the owned ones, which the halo exchange fills
  // with the neighbouring slabs' boundary planes; field / lo / jf point at
  // the first owned plane, so every host-facing call sees the owned grid.
  // zhalo is 0 for an ordinary handle.
  int zhalo = 0;
  int slab_k0 = 0;
  int slab_nk_global = 0;
  cudaEvent_t xev[2] = {nullptr, nullptr};  // halo exchange ordering (sent, received)
  // The planes a sweep updates, in the storage's plane numbering.
  Box sweep_box() const {
    Box b = main_box();
    b.k0 += zhalo;
    b.k1 += zhalo;
    return b;
  }
  // Elements between the first stored plane and the first owned plane.
  int64_t halo_elems() const { return form == Form::F64 ? zhalo * g.plane : zhalo * L.pplane; }

  int pipeline = FDTD_PIPELINE_AUTO;
  FusedConfig fused_cfg;
  PLayout L{};  // padded layout of the FP32-arithmetic forms
  // TMA maps of the current and the second copy (rebuilt when the tile
  // shape changes; swapped with the copies): load maps of the two-cell
  // kernel (uniform boxes; built only for it)...
  TmaMaps maps_cur;
  TmaMaps maps_alt;
  // ... store maps (grid cells and x margins) for the one-cell kernels ...
  TmaMaps smaps_cur;
  TmaMaps smaps_alt;
  // ... and load maps of the one-cell B-first sweep (per-component halos)
  // and of the depth-2 sweep (two rings of halo).
  TmaMaps bmaps_cur;
  TmaMaps bmaps_alt;
  TmaMaps tmaps_cur;
  TmaMaps tmaps_alt;
  int maps_tile_y = 0;
  int* d_err = nullptr;  // device status word (bounded waits that gave up)
  // Bounded waits of the fused sweeps: polls before a wait gives up, and the
  // test hook that issues no tile loads (fdtd_set_wait_limit).
  uint32_t wait_polls = kMaxBarrierPolls;
  int withhold_loads = 0;
  WaitCtl wait_ctl() const { return WaitCtl{d_err, wait_polls, withhold_loads}; }

  // Pending B half step (FP32-arithmetic forms, B-first fused sweeps): the
  // stored B lacks the trailing half step of the last update_fields; the next
  // step applies it together with its leading half (one sweep), and every
  // reader of B sees it applied (read_view).  b_side: the second copy's B
  // arrays hold the stored B with the pending half applied (valid until the
  // next sweep writes that copy).
  bool b_pending = false;
  bool b_side = false;
  // A z slab has no second copy: its side B arrays (allocated on first use,
  // halo planes included) take the pending half for readers.
  void* side_b[3] = {nullptr, nullptr, nullptr};
  LoT* side_lo[3] = {nullptr, nullptr, nullptr};

  // Scratch.
  double* d_staging = nullptr;
  double* d_partials = nullptr;
  double* d_diag_out = nullptr;

  std::vector<void*> allocations;

  // Kernel timing: event pairs recorded around launches while enabled.
  struct TimedLaunch {
    cudaEvent_t start, stop;
    int kind;
  };
  bool timing = false;
  std::vector<TimedLaunch> timed;
  std::vector<cudaEvent_t> event_pool;

  StateView make_view(void* const* f, LoT* const* l) const {
    StateView v{};
    v.form = form;
    v.g = g;
    v.L = L;
    for (int c = 0; c < 6; ++c) v.f64[c] = (form == Form::F64) ? (double*)f[c] : nullptr;
    for (int c = 0; c < 6; ++c) {
      v.s32.v[c] = (float*)f[c];
      v.s32c.hi[c] = (float*)f[c];
      v.s32c.lo[c] = l[c];
      v.s16.v[c] = (__half*)f[c];
      v.s16.scale[c] = std::ldexp(1.0f, fp16_exp[c]);
      v.s16.inv_scale[c] = std::ldexp(1.0f, -fp16_exp[c]);
    }
    // FP16 kernels compute on stored values: each coefficient carries the
    // power of two between its term's source and destination scales.
    const int* e = fp16_exp;
    for (int c = 0; c < 3; ++c) {
      for (int t = 0; t < 2; ++t) {
        v.s16.te[2 * c + t] = std::ldexp(cs.ce[term_axis(c, t)].hi, e[c] - e[e_term_src(c, t)]);
        v.s16.tb[2 * c + t] = std::ldexp(cs.cb[term_axis(c, t)].hi, e[3 + c] - e[b_term_src(c, t)]);
      }
      v.s16.tj[c] = std::ldexp(cs.cj.hi, e[c]);
    }
    return v;
  }
  StateView view() const { return make_view(field, lo); }
  StateView view_alt() const { return make_view(alt_field, alt_lo); }
  // E from the current copy, B from the second copy (a z slab: its side
  // arrays) with the pending half applied.
  StateView view_side() const {
    void* const* sb = zhalo ? side_b : alt_field + 3;
    LoT* const* sl = zhalo ? side_lo : alt_lo + 3;
    void* f[6] = {field[0], field[1], field[2], sb[0], sb[1], sb[2]};
    LoT* l[6] = {lo[0], lo[1], lo[2], sl[0], sl[1], sl[2]};
    return make_view(f, l);
  }
  // The storage the sweeps index: the owned planes and the halo planes.
  StateView sweep_view() const { return with_halo(view()); }
  StateView with_halo(StateView v) const {
    if (zhalo == 0) return v;
    v.g.Nk += 2 * zhalo;
    v.g.cells = v.g.plane * v.g.Nk;
    v.L = PLayout::make(g.Ni, g.Nj, g.Nk + 2 * zhalo);
    const int64_t d = halo_elems();
    for (int c = 0; c < 6; ++c) {
      switch (form) {
        case Form::F64: v.f64[c] -= d; break;
        case Form::F32: v.s32.v[c] -= d; break;
        case Form::F32C: v.s32c.hi[c] -= d; v.s32c.lo[c] -= d; break;
        case Form::F16: v.s16.v[c] -= d; break;
      }
    }
    return v;
  }
  SourceSet source_set() const {
    SourceSet ss{};
    ss.count = (int)sources.size();
    ss.src = d_src;
    ss.tables = d_tables;
    ss.tables_f = d_tables_f;
    ss.lo_off = tables_lo_off;
    return ss;
  }
};

namespace fdtd {
// Allocates the second copy of the E/B storage (first use) and builds the
// TMA maps of both copies for the handle's tile shape.
int ensure_alt(fdtd_handle* h);
// Swaps the current and the second copy (after a fused sweep).
void swap_copies(fdtd_handle* h);
// The state as readers see it: the stored state, or with a pending B half
// step applied (computed into the second copy's B arrays on first use).
int read_view(fdtd_handle* h, StateView* v);
// Applies a pending B half step to the stored state (before anything writes
// E or B, or runs a sweep that expects B at the step boundary).
int resolve_pending(fdtd_handle* h);
}  // namespace fdtd
