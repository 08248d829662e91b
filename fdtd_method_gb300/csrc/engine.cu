// C-ABI layer of the engine: handle lifetime, storage, step scheduling,
// host transfers, sources and diagnostics.  See include/fdtd_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fdtd_gb300.h"
#include "handle.h"

using namespace fdtd;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  return fail(e == cudaErrorMemoryAllocation ? FDTD_ERR_OUT_OF_MEMORY : FDTD_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define FDTD_CUDA(call, what)                   \
  do {                                          \
    cudaError_t e_ = (call);                    \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

// Speed of light and pi as the reference defines them (include/Constants.h:6,11).
constexpr double kC = 3e10;
constexpr double kPi = 3.14159265358;
// PML constants of the reference (include/Constants.h:7,10): reflection R and
// the order N of the conductivity profile.
constexpr double kPmlR = 1e-12;
constexpr double kPmlOrder = 4.0;

constexpr int64_t kStagingElems = int64_t(1) << 24;  // 16 Mi doubles = 128 MiB
constexpr int kMaxDiagBlocks = 152 * 8;

Coef split_coef(double c) {
  const float h = (float)c;
  return Coef{h, (float)(c - (double)h)};
}

}  // namespace

namespace fdtd {
// Lets other translation units of the library report through fdtd_last_error().
void set_last_error(const std::string& msg) { g_last_error = msg; }

}  // namespace fdtd

namespace {

cudaError_t dev_alloc(fdtd_handle* h, void** ptr, size_t bytes) {
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e == cudaSuccess) h->allocations.push_back(*ptr);
  return e;
}

void release(fdtd_handle* h) {
  if (!h) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (void* p : h->allocations) cudaFree(p);
  for (cudaEvent_t e : h->xev)
    if (e) cudaEventDestroy(e);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  cudaSetDevice(prev);
  delete h;
}

size_t elem_bytes(Form f) {
  switch (f) {
    case Form::F64: return 8;
    case Form::F32: return 4;
    case Form::F32C: return 4;
    case Form::F16: return 2;
  }
  return 8;
}

int ensure_staging(fdtd_handle* h) {
  // Transfers move at most kStagingElems values per chunk, and never more
  // than the grid holds (small grids, as in a batch, get small buffers).
  if (!h->d_staging)
    FDTD_CUDA(dev_alloc(h, (void**)&h->d_staging, sizeof(double) * std::min<int64_t>(kStagingElems, h->g.cells)),
              "staging buffer");
  return FDTD_OK;
}

int ensure_jf(fdtd_handle* h) {
  if (h->form == Form::F64 || h->jf[0]) return FDTD_OK;
  // a slab's currents carry its halo planes too (never read: J enters only
  // the owned planes' E update), so they index like its fields
  const int64_t halo = h->zhalo * h->g.plane, n = h->g.cells + 2 * halo;
  for (int c = 0; c < 3; ++c) {
    float* base = nullptr;
    FDTD_CUDA(dev_alloc(h, (void**)&base, sizeof(float) * n), "current arrays");
    FDTD_CUDA(cudaMemsetAsync(base, 0, sizeof(float) * n, h->stream), "zero current");
    h->jf[c] = base + halo;
  }
  return FDTD_OK;
}

// Uploads the source tables after any change to the source list.
int upload_sources(fdtd_handle* h) {
  std::vector<double> tables;
  std::vector<DevSource> ds;
  for (const HostSource& hs : h->sources) {
    DevSource d{};
    d.comp_mask = hs.s.comp_mask;
    d.i0 = hs.s.i0; d.j0 = hs.s.j0; d.k0 = hs.s.k0;
    d.ni = hs.s.ni; d.nj = hs.s.nj; d.nk = hs.s.nk;
    d.gx_off = (int64_t)tables.size(); tables.insert(tables.end(), hs.gx.begin(), hs.gx.end());
    d.gy_off = (int64_t)tables.size(); tables.insert(tables.end(), hs.gy.begin(), hs.gy.end());
    d.gz_off = (int64_t)tables.size(); tables.insert(tables.end(), hs.gz.begin(), hs.gz.end());
    d.amp_off = (int64_t)tables.size(); tables.insert(tables.end(), hs.amp.begin(), hs.amp.end());
    d.n_amp = (int64_t)hs.amp.size();
    ds.push_back(d);
  }
  // The previous tables may still be read by queued kernels.
  FDTD_CUDA(cudaStreamSynchronize(h->stream), "synchronize before source upload");
  if (h->d_src) { cudaFree(h->d_src); h->d_src = nullptr; }
  if (h->d_tables) { cudaFree(h->d_tables); h->d_tables = nullptr; }
  if (h->d_tables_f) { cudaFree(h->d_tables_f); h->d_tables_f = nullptr; }
  if (ds.empty()) return FDTD_OK;
  FDTD_CUDA(cudaMalloc(&h->d_src, sizeof(DevSource) * ds.size()), "source descriptors");
  FDTD_CUDA(cudaMalloc(&h->d_tables, sizeof(double) * tables.size()), "source tables");
  FDTD_CUDA(cudaMalloc(&h->d_tables_f, 2 * sizeof(float) * tables.size()), "source tables (fp32)");
  FDTD_CUDA(cudaMemcpy(h->d_src, ds.data(), sizeof(DevSource) * ds.size(), cudaMemcpyHostToDevice),
            "upload source descriptors");
  FDTD_CUDA(cudaMemcpy(h->d_tables, tables.data(), sizeof(double) * tables.size(),
                       cudaMemcpyHostToDevice),
            "upload source tables");
  h->tables_lo_off = (int64_t)tables.size();
  FDTD_CUDA(launch_split_f32(h->d_tables, h->d_tables_f, h->d_tables_f + h->tables_lo_off,
                             (int64_t)tables.size(), h->stream),
            "split source tables");
  FDTD_CUDA(cudaStreamSynchronize(h->stream), "source upload");
  return FDTD_OK;
}

cudaEvent_t take_event(fdtd_handle* h) {
  if (!h->event_pool.empty()) {
    cudaEvent_t e = h->event_pool.back();
    h->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

// Brackets one launch with events when kernel timing is on.
struct LaunchTimer {
  fdtd_handle* h;
  cudaEvent_t start = nullptr;
  int kind;
  LaunchTimer(fdtd_handle* hh, int k) : h(hh), kind(k) {
    if (h->timing && (start = take_event(h))) cudaEventRecord(start, h->stream);
  }
  void done() {
    if (!start) return;
    cudaEvent_t stop = take_event(h);
    if (!stop) {
      h->event_pool.push_back(start);
      return;
    }
    cudaEventRecord(stop, h->stream);
    h->timed.push_back({start, stop, kind});
  }
};

bool b_first(const fdtd_handle* h);

// B update with `apps` applications of the curl term (2: the last half
// step of one update_fields and the first of the next share one sweep).
int run_b(fdtd_handle* h, int apps) {
  // the fused sweep's tiles, in place, where the handle has its second copy
  // and one-cell maps (a z slab and the two-cell kernel use the column sweep)
  const bool tiles = h->form != Form::F64 && !h->zhalo && h->alt_field[0] && b_first(h);
  if (tiles)
    if (int rc = ensure_alt(h)) return rc;
  LaunchTimer lt(h, apps == 2 ? FDTD_KERNEL_B_DOUBLE : FDTD_KERNEL_B_HALF);
  cudaError_t e = cudaSuccess;
  const Box box = h->sweep_box();
  const StateView v = h->sweep_view();
  if (tiles) {
    StepMaps sm;
    sm.ld = h->bmaps_cur;
    sm.st = h->smaps_cur;
    const WaitCtl wc = h->wait_ctl();
    switch (h->form) {
      case Form::F32: e = launch_bhalf_f32(v.L, v.s32, v.s32, &sm, h->cs, apps, h->fused_cfg, wc, h->stream); break;
      case Form::F32C: e = launch_bhalf_f32(v.L, v.s32c, v.s32c, &sm, h->cs, apps, h->fused_cfg, wc, h->stream); break;
      case Form::F16: e = launch_bhalf_f32(v.L, v.s16, v.s16, &sm, h->cs, apps, h->fused_cfg, wc, h->stream); break;
      default: e = cudaErrorInvalidValue; break;
    }
  } else if (h->form == Form::F64) {
    Fp64Fields F;
    for (int c = 0; c < 9; ++c) F.f[c] = (double*)h->field[c] - h->halo_elems();
    e = launch_b_fp64(v.g, box, F, &h->coef[3], apps, h->fp64_fma, h->stream);
  } else {
    switch (h->form) {
      case Form::F32: e = launch_b_f32(v.L, v.s32, h->cs, apps, box.k0, box.k1, h->stream); break;
      case Form::F32C: e = launch_b_f32(v.L, v.s32c, h->cs, apps, box.k0, box.k1, h->stream); break;
      case Form::F16: e = launch_b_f32(v.L, v.s16, h->cs, apps, box.k0, box.k1, h->stream); break;
      default: break;
    }
  }
  lt.done();
  if (e != cudaSuccess) return cuda_fail(e, "B update launch");
  return FDTD_OK;
}

// E update of time step `step` (indexes the source amplitude tables).
int run_e(fdtd_handle* h, int64_t step) {
  LaunchTimer lt(h, FDTD_KERNEL_E);
  SourceSet ss = h->source_set();
  cudaError_t e = cudaSuccess;
  const Box box = h->sweep_box();
  const StateView v = h->sweep_view();
  if (h->form == Form::F64) {
    Fp64Fields F;
    for (int c = 0; c < 9; ++c) F.f[c] = (double*)h->field[c] - h->halo_elems();
    e = launch_e_fp64(v.g, box, F, &h->coef[0], h->coef[6], h->dense_j, ss, step, h->fp64_fma, h->stream);
  } else {
    // dense FP32 currents: the dense layout, with the same halo planes
    const int64_t dj0 = h->zhalo * h->g.plane;
    const bool dj = h->dense_j && h->jf[0];
    const float* J[3] = {dj ? h->jf[0] - dj0 : nullptr, dj ? h->jf[1] - dj0 : nullptr, dj ? h->jf[2] - dj0 : nullptr};
    switch (h->form) {
      case Form::F32: e = launch_e_f32(v.L, v.s32, J, dj, h->cs, ss, step, box.k0, box.k1, h->stream); break;
      case Form::F32C: e = launch_e_f32(v.L, v.s32c, J, dj, h->cs, ss, step, box.k0, box.k1, h->stream); break;
      case Form::F16: e = launch_e_f32(v.L, v.s16, J, dj, h->cs, ss, step, box.k0, box.k1, h->stream); break;
      default: break;
    }
  }
  lt.done();
  if (e != cudaSuccess) return cuda_fail(e, "E update launch");
  return FDTD_OK;
}

// Whether the handle's fused sweeps run B-first (one cell per thread) or
// E-first (the two-cell kernel).
bool b_first(const fdtd_handle* h) { return h->fused_cfg.cells_per_thread == 1; }

// One fused sweep of step `step` from the current copy into the second one,
// without the swap (the autotuner repeats it to time a tile shape: the state
// is only read).  B-first: `apps` B half steps, then E; E-first: E, then
// `apps` B half steps.
cudaError_t launch_fused_sweep(fdtd_handle* h, int64_t step, int apps, int depth = 1) {
  SourceSet ss = h->source_set();
  if (h->zhalo) {
    // z slab: the B-first sweep over the storage's owned planes, reading the
    // halo planes below and above (the copies carry them; the maps cover them)
    if (depth != 1 || !b_first(h)) return cudaErrorInvalidValue;
    const StateView v = h->sweep_view(), w = h->with_halo(h->view_alt());
    const int64_t dj0 = h->zhalo * h->g.plane;
    const bool dj = h->dense_j && h->jf[0];
    const float* J[3] = {dj ? h->jf[0] - dj0 : nullptr, dj ? h->jf[1] - dj0 : nullptr, dj ? h->jf[2] - dj0 : nullptr};
    StepMaps sm;
    sm.ld = h->bmaps_cur;
    sm.st = h->smaps_alt;
    const int kb = h->zhalo, ke = h->zhalo + h->g.Nk;
    const FusedConfig& cf = h->fused_cfg;
    const WaitCtl wc = h->wait_ctl();
    switch (h->form) {
      case Form::F32: return launch_fused1_f32(v.L, v.s32, w.s32, &sm, J, dj, h->cs, ss, step, apps, cf, wc, h->stream, kb, ke);
      case Form::F32C: return launch_fused1_f32(v.L, v.s32c, w.s32c, &sm, J, dj, h->cs, ss, step, apps, cf, wc, h->stream, kb, ke);
      case Form::F16: return launch_fused1_f32(v.L, v.s16, w.s16, &sm, J, dj, h->cs, ss, step, apps, cf, wc, h->stream, kb, ke);
      default: return cudaErrorInvalidValue;
    }
  }
  StateView v = h->view();
  StateView w = h->view_alt();
  const float* J[3] = {h->jf[0], h->jf[1], h->jf[2]};
  const bool dj = h->dense_j && h->jf[0];
  const FusedConfig& cf = h->fused_cfg;
  const WaitCtl wc = h->wait_ctl();
  StepMaps sm;
  sm.ld = h->bmaps_cur;
  sm.st = h->smaps_alt;
  cudaError_t e = cudaSuccess;
  if (depth == 2) {
    // both ghost rings of the input copy, then two steps in one pass
    GhostArrays ga{{h->field[0], h->field[1], h->field[2], h->field[3], h->field[4], h->field[5]}};
    e = launch_refresh_ghosts(h->L, ga, h->form == Form::F16 ? 2 : 4, h->stream);
    if (e == cudaSuccess && h->form == Form::F32C) {
      GhostArrays gl{{h->lo[0], h->lo[1], h->lo[2], h->lo[3], h->lo[4], h->lo[5]}};
      e = launch_refresh_ghosts(h->L, gl, 2, h->stream);
    }
    if (e != cudaSuccess) return e;
    StepMaps tm;
    tm.ld = h->tmaps_cur;
    tm.st = h->smaps_alt;
    switch (h->form) {
      case Form::F32: return launch_tblock2_f32(h->L, v.s32, w.s32, &tm, J, dj, h->cs, ss, step, apps, cf, wc, h->stream);
      case Form::F32C: return launch_tblock2_f32(h->L, v.s32c, w.s32c, &tm, J, dj, h->cs, ss, step, apps, cf, wc, h->stream);
      case Form::F16: return launch_tblock2_f32(h->L, v.s16, w.s16, &tm, J, dj, h->cs, ss, step, apps, cf, wc, h->stream);
      default: return cudaErrorInvalidValue;
    }
  }
  if (cf.cells_per_thread == 2) {
    const void* m = &h->maps_cur;
    switch (h->form) {
      case Form::F32: e = launch_fused_f32(h->L, v.s32, w.s32, m, J, dj, h->cs, ss, step, apps, cf, wc, h->stream); break;
      case Form::F32C: e = launch_fused_f32(h->L, v.s32c, w.s32c, m, J, dj, h->cs, ss, step, apps, cf, wc, h->stream); break;
      case Form::F16: e = launch_fused_f32(h->L, v.s16, w.s16, m, J, dj, h->cs, ss, step, apps, cf, wc, h->stream); break;
      default: e = cudaErrorInvalidValue; break;
    }
    return e;
  }
  switch (h->form) {
    case Form::F32: e = launch_fused1_f32(h->L, v.s32, w.s32, &sm, J, dj, h->cs, ss, step, apps, cf, wc, h->stream); break;
    case Form::F32C: e = launch_fused1_f32(h->L, v.s32c, w.s32c, &sm, J, dj, h->cs, ss, step, apps, cf, wc, h->stream); break;
    case Form::F16: e = launch_fused1_f32(h->L, v.s16, w.s16, &sm, J, dj, h->cs, ss, step, apps, cf, wc, h->stream); break;
    default: e = cudaErrorInvalidValue; break;
  }
  return e;
}

int run_fused(fdtd_handle* h, int64_t step, int apps, int depth = 1) {
  if (int rc = ensure_alt(h)) return rc;
  LaunchTimer lt(h, depth == 2 ? FDTD_KERNEL_FUSED2 : FDTD_KERNEL_FUSED);
  cudaError_t e = launch_fused_sweep(h, step, apps, depth);
  lt.done();
  if (e != cudaSuccess) return cuda_fail(e, "fused step launch");
  swap_copies(h);
  return FDTD_OK;
}

// Tile shapes the autotuner tries (one cell per thread: 6, 14 or 30 rows;
// two cells per thread: 6 or 14), each with every chunk length.
constexpr int kTuneRows1[] = {6, 14, 30};
constexpr int kTuneRows2[] = {6, 14};
constexpr int kTuneChunks[] = {16, 24, 32, 48, 64, 96};
// The depth-2 sweep: 6- or 14-row tiles; it reads four planes past its chunk,
// so only longer chunks.
constexpr int kTuneRowsDepth2[] = {6, 14};
constexpr int kTuneChunksDepth2[] = {24, 48, 96};

struct TuneKey {
  int form, Ni, Nj, Nk;
  bool operator<(const TuneKey& o) const {
    return std::tie(form, Ni, Nj, Nk) < std::tie(o.form, o.Ni, o.Nj, o.Nk);
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, fdtd_tune_result> g_tune_cache;

// Device address of a page-locked host buffer (nullptr for other memory).
// The conversion kernels read and write such buffers directly, over the
// host link, with no staging copy.
double* device_alias(const double* host) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free error of an unknown pointer
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  return static_cast<double*>(at.devicePointer);
}

// The six layer slabs of FDTD_PML::update_fields (FDTD_PML_kokkos.cpp:170-186),
// which tile everything outside the main box exactly once.
void pml_slabs(const fdtd_handle* h, Box out[6]) {
  const int Ni = h->g.Ni, Nj = h->g.Nj, Nk = h->g.Nk;
  const int pi = h->pml_size[0], pj = h->pml_size[1], pk = h->pml_size[2];
  out[0] = Box{0, Ni - pi, 0, Nj, 0, pk};
  out[1] = Box{pi, Ni - pi, 0, pj, pk, Nk - pk};
  out[2] = Box{0, pi, 0, Nj, pk, Nk};
  out[3] = Box{pi, Ni, 0, Nj, Nk - pk, Nk};
  out[4] = Box{pi, Ni - pi, Nj - pj, Nj, pk, Nk - pk};
  out[5] = Box{Ni - pi, Ni, 0, Nj, 0, Nk - pk};
}

// Split-field update of the layer: B (e = false) or E (e = true).
int run_pml(fdtd_handle* h, bool e) {
  Fp64Fields F;
  for (int c = 0; c < 9; ++c) F.f[c] = (double*)h->field[c];
  PmlFields P;
  for (int q = 0; q < 12; ++q) P.split[q] = h->split[q];
  for (int a = 0; a < 3; ++a) {
    P.decay[a] = h->pml_decay[a];
    P.coef2[a] = h->pml_coef2[a];
  }
  Box slab[6];
  pml_slabs(h, slab);
  for (int q = 0; q < 6; ++q) {
    const cudaError_t err = e ? launch_e_pml_fp64(h->g, slab[q], F, P, h->stream)
                              : launch_b_pml_fp64(h->g, slab[q], F, P, h->stream);
    if (err != cudaSuccess) return cuda_fail(err, "PML update launch");
  }
  return FDTD_OK;
}

int check_handle(fdtd_handle* h) {
  if (!h) return fail(FDTD_ERR_INVALID_ARGUMENT, "null handle");
  return FDTD_OK;
}

}  // namespace

namespace fdtd {

// Second copy of the E/B storage for the fused sweep (allocated on first
// use) and the TMA maps of both copies for the current tile shape.
int ensure_alt(fdtd_handle* h) {
  const size_t eb = elem_bytes(h->form);
  // a z slab's second copy has halo planes too (its fused step swaps copies)
  const int64_t halo = h->halo_elems();
  if (!h->alt_field[0]) {
    const int64_t n = h->L.elems() + 2 * halo;
    for (int c = 0; c < 6; ++c) {
      void* base = nullptr;
      FDTD_CUDA(dev_alloc(h, &base, eb * n), "second field copy");
      FDTD_CUDA(cudaMemsetAsync(base, 0, eb * n, h->stream), "zero second copy");
      h->alt_field[c] = static_cast<unsigned char*>(base) + eb * halo;
      if (h->form == Form::F32C) {
        LoT* lb = nullptr;
        FDTD_CUDA(dev_alloc(h, (void**)&lb, sizeof(LoT) * n), "second compensation copy");
        FDTD_CUDA(cudaMemsetAsync(lb, 0, sizeof(LoT) * n, h->stream), "zero second copy");
        h->alt_lo[c] = lb + halo;
      }
    }
    h->maps_tile_y = 0;
  }
  const int key = h->fused_cfg.tile_y * 10 + h->fused_cfg.cells_per_thread;
  if (h->maps_tile_y != key) {
    const HiType ht = h->form == Form::F16 ? HiType::F16 : HiType::F32;
    const bool two = h->fused_cfg.cells_per_thread == 2;
    // box widths per component: the two-cell kernel's are uniform, the
    // one-cell kernel's trimmed to what its stencil reads
    int bw[6], lbw[6];
    if (two) {
      for (int c = 0; c < 6; ++c) {
        bw[c] = h->form == Form::F16 ? fused_box_width<StoreF16>() : fused_box_width<StoreF32>();
        lbw[c] = fused_lo_box_width();
      }
    } else {
      switch (h->form) {
        case Form::F16: fused1_box_widths<StoreF16>(bw, lbw); break;
        case Form::F32C: fused1_box_widths<StoreF32C>(bw, lbw); break;
        default: fused1_box_widths<StoreF32>(bw, lbw); break;
      }
    }
    // The maps cover the storage: on a z slab its halo planes as well (plane
    // p of the map is storage plane p, the owned planes being 1..Nk).
    const PLayout Lm = h->zhalo ? PLayout::make(h->g.Ni, h->g.Nj, h->g.Nk + 2 * h->zhalo) : h->L;
    void* f_cur[6];
    void* f_alt[6];
    LoT* l_cur[6];
    LoT* l_alt[6];
    for (int c = 0; c < 6; ++c) {
      f_cur[c] = static_cast<unsigned char*>(h->field[c]) - eb * halo;
      f_alt[c] = static_cast<unsigned char*>(h->alt_field[c]) - eb * halo;
      l_cur[c] = h->form == Form::F32C ? h->lo[c] - halo : nullptr;
      l_alt[c] = h->form == Form::F32C ? h->alt_lo[c] - halo : nullptr;
    }
    LoT* const* lo_cur = h->form == Form::F32C ? l_cur : nullptr;
    LoT* const* lo_alt = h->form == Form::F32C ? l_alt : nullptr;
    const int ty = h->fused_cfg.tile_y;
    // the two-cell (E-first) kernel's load maps, or the one-cell kernel's
    if (two && (build_tma_maps(&h->maps_cur, Lm, ht, f_cur, lo_cur, bw, lbw, ty, BoxTrim::None) != cudaSuccess ||
                build_tma_maps(&h->maps_alt, Lm, ht, f_alt, lo_alt, bw, lbw, ty, BoxTrim::None) != cudaSuccess))
      return fail(FDTD_ERR_CUDA, "TMA tensor map encoding failed");
    if (!two && (build_tma_maps(&h->bmaps_cur, Lm, ht, f_cur, lo_cur, bw, lbw, ty, BoxTrim::BFirst) != cudaSuccess ||
                 build_tma_maps(&h->bmaps_alt, Lm, ht, f_alt, lo_alt, bw, lbw, ty, BoxTrim::BFirst) != cudaSuccess))
      return fail(FDTD_ERR_CUDA, "TMA tensor map encoding failed");
    if (!two && ty != 30) {
      int tw[6], tlw[6];
      switch (h->form) {
        case Form::F16: tblock2_box_widths<StoreF16>(tw, tlw); break;
        case Form::F32C: tblock2_box_widths<StoreF32C>(tw, tlw); break;
        default: tblock2_box_widths<StoreF32>(tw, tlw); break;
      }
      // depth-2 boxes: rows y0-2 .. y0+ty+1 for Ex, Ez, y0-2 .. y0+ty otherwise
      if (build_tma_maps(&h->tmaps_cur, Lm, ht, f_cur, lo_cur, tw, tlw, ty + 2, BoxTrim::BFirst) != cudaSuccess ||
          build_tma_maps(&h->tmaps_alt, Lm, ht, f_alt, lo_alt, tw, tlw, ty + 2, BoxTrim::BFirst) != cudaSuccess)
        return fail(FDTD_ERR_CUDA, "TMA tensor map encoding failed");
    }
    if (!two && (build_tma_store_maps(&h->smaps_cur, Lm, ht, f_cur, lo_cur, ty) != cudaSuccess ||
                 build_tma_store_maps(&h->smaps_alt, Lm, ht, f_alt, lo_alt, ty) != cudaSuccess))
      return fail(FDTD_ERR_CUDA, "TMA tensor map encoding failed");
    h->maps_tile_y = key;
  }
  return FDTD_OK;
}

void swap_copies(fdtd_handle* h) {
  for (int c = 0; c < 6; ++c) {
    std::swap(h->field[c], h->alt_field[c]);
    std::swap(h->lo[c], h->alt_lo[c]);
  }
  std::swap(h->maps_cur, h->maps_alt);
  std::swap(h->smaps_cur, h->smaps_alt);
  std::swap(h->bmaps_cur, h->bmaps_alt);
  std::swap(h->tmaps_cur, h->tmaps_alt);
}

int read_view(fdtd_handle* h, StateView* v) {
  if (!h->b_pending) {
    *v = h->view();
    return FDTD_OK;
  }
  if (!h->b_side) {
    // B with the pending half step, into the second copy's B arrays (the next
    // sweep overwrites that copy anyway; split sweeps may not have made it
    // yet); a z slab uses side arrays, and its halo plane above holds the
    // neighbour's E from the last exchange.
    if (!h->zhalo)
      if (int rc = ensure_alt(h)) return rc;
    if (h->zhalo && !h->side_b[0]) {
      const int64_t n = h->L.elems() + 2 * h->halo_elems();
      for (int c = 0; c < 3; ++c) {
        void* base = nullptr;
        FDTD_CUDA(dev_alloc(h, &base, elem_bytes(h->form) * n), "pending B half step arrays");
        h->side_b[c] = static_cast<unsigned char*>(base) + elem_bytes(h->form) * h->halo_elems();
        if (h->form == Form::F32C) {
          LoT* lb = nullptr;
          FDTD_CUDA(dev_alloc(h, (void**)&lb, sizeof(LoT) * n), "pending B half step arrays");
          h->side_lo[c] = lb + h->halo_elems();
        }
      }
    }
    const StateView cur = h->sweep_view(), side = h->with_halo(h->view_side());
    const Box box = h->sweep_box();
    cudaError_t e = cudaSuccess;
    if (!h->zhalo && b_first(h)) {
      // the fused sweep's tiles: loads from the current copy, stores into the
      // second copy's B arrays
      LaunchTimer lt(h, FDTD_KERNEL_B_HALF);
      StepMaps sm;
      sm.ld = h->bmaps_cur;
      sm.st = h->smaps_alt;
      const WaitCtl wc = h->wait_ctl();
      switch (h->form) {
        case Form::F32: e = launch_bhalf_f32(cur.L, cur.s32, side.s32, &sm, h->cs, 1, h->fused_cfg, wc, h->stream); break;
        case Form::F32C: e = launch_bhalf_f32(cur.L, cur.s32c, side.s32c, &sm, h->cs, 1, h->fused_cfg, wc, h->stream); break;
        case Form::F16: e = launch_bhalf_f32(cur.L, cur.s16, side.s16, &sm, h->cs, 1, h->fused_cfg, wc, h->stream); break;
        default: e = cudaErrorInvalidValue; break;
      }
      lt.done();
    } else {
      switch (h->form) {
        case Form::F32: e = launch_b_f32_into(cur.L, cur.s32, side.s32, h->cs, box.k0, box.k1, h->stream); break;
        case Form::F32C: e = launch_b_f32_into(cur.L, cur.s32c, side.s32c, h->cs, box.k0, box.k1, h->stream); break;
        case Form::F16: e = launch_b_f32_into(cur.L, cur.s16, side.s16, h->cs, box.k0, box.k1, h->stream); break;
        default: e = cudaErrorInvalidValue; break;
      }
    }
    if (e != cudaSuccess) return cuda_fail(e, "pending B half step");
    h->b_side = true;
  }
  *v = h->view_side();
  return FDTD_OK;
}

int resolve_pending(fdtd_handle* h) {
  if (!h->b_pending) return FDTD_OK;
  if (int rc = run_b(h, 1)) return rc;
  h->b_pending = false;
  h->b_side = false;
  return FDTD_OK;
}

}  // namespace fdtd

extern "C" {

const char* fdtd_last_error(void) { return g_last_error.c_str(); }
int fdtd_abi_version(void) { return FDTD_ABI_VERSION; }

// A handle of the grid `params` whose arrays carry `zhalo` extra planes
// below and above it (0: an ordinary handle; 1: a z slab).
static int create_handle(const fdtd_params* params, double dt, int precision, int zhalo, fdtd_handle** out) {
  if (!params || !out) return fail(FDTD_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  // src/FDTD_kokkos/FDTD_kokkos.cpp:7-12
  if (params->Ni <= 0 || params->Nj <= 0 || params->Nk <= 0 || !(dt > 0))
    return fail(FDTD_ERR_INVALID_ARGUMENT, "ERROR: invalid parameters");
  if (precision < FDTD_PRECISION_FP64 || precision > FDTD_PRECISION_FP16_SCALED)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "invalid precision");

  fdtd_handle* h = new fdtd_handle();
  h->zhalo = zhalo;
  h->p = *params;
  h->dt = dt;
  h->precision = precision;
  h->form = (Form)precision;
  h->g.Ni = params->Ni;
  h->g.Nj = params->Nj;
  h->g.Nk = params->Nk;
  h->g.plane = (int64_t)params->Ni * params->Nj;
  h->g.cells = h->g.plane * params->Nk;
  cudaGetDevice(&h->device);

  // src/FDTD_kokkos/FDTD_kokkos.cpp:45-55
  const double cdt = kC * dt;
  h->coef[0] = cdt / params->dx;
  h->coef[1] = cdt / params->dy;
  h->coef[2] = cdt / params->dz;
  h->coef[3] = cdt / (2.0 * params->dx);
  h->coef[4] = cdt / (2.0 * params->dy);
  h->coef[5] = cdt / (2.0 * params->dz);
  h->coef[6] = -4.0 * kPi * dt;
  for (int a = 0; a < 3; ++a) {
    h->cs.ce[a] = split_coef(h->coef[a]);
    h->cs.cb[a] = split_coef(h->coef[3 + a]);
  }
  h->cs.cj = split_coef(h->coef[6]);
  h->cs.cj64 = h->coef[6];
  if (h->form != Form::F32C) {  // only the compensated form carries coefficient lo parts
    for (int a = 0; a < 3; ++a) h->cs.ce[a].lo = h->cs.cb[a].lo = 0.f;
    h->cs.cj.lo = 0.f;
  }

  cudaError_t e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    int rc = cuda_fail(e, "stream creation");
    delete h;
    return rc;
  }
  h->stream = h->own_stream;

  // FP64: the reference's nine dense arrays.  Other forms: six padded E/B
  // arrays (ghosts included) and, for FP32_COMP, six padded lo arrays.
  h->L = PLayout::make(params->Ni, params->Nj, params->Nk);
  const size_t eb = elem_bytes(h->form);
  const int nfields = (h->form == Form::F64) ? 9 : 6;
  const int64_t halo = h->halo_elems();
  const int64_t per_field = ((h->form == Form::F64) ? h->g.cells : h->L.elems()) + 2 * halo;
  for (int c = 0; c < nfields; ++c) {
    void* base = nullptr;
    e = dev_alloc(h, &base, eb * per_field);
    if (e == cudaSuccess) e = cudaMemsetAsync(base, 0, eb * per_field, h->stream);
    if (e != cudaSuccess) {
      int rc = cuda_fail(e, "field allocation");
      release(h);
      return rc;
    }
    h->field[c] = static_cast<unsigned char*>(base) + eb * halo;
  }
  if (h->form == Form::F32C) {
    for (int c = 0; c < 6; ++c) {
      LoT* base = nullptr;
      e = dev_alloc(h, (void**)&base, sizeof(LoT) * per_field);
      if (e == cudaSuccess) e = cudaMemsetAsync(base, 0, sizeof(LoT) * per_field, h->stream);
      if (e != cudaSuccess) {
        int rc = cuda_fail(e, "compensation allocation");
        release(h);
        return rc;
      }
      h->lo[c] = base + halo;
    }
  }
  if (zhalo > 0) {
    for (cudaEvent_t& x : h->xev)
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      int rc = cuda_fail(e, "slab event creation");
      release(h);
      return rc;
    }
  }
  e = dev_alloc(h, (void**)&h->d_partials, sizeof(double) * kDiagValues * kMaxDiagBlocks);
  if (e == cudaSuccess) e = dev_alloc(h, (void**)&h->d_diag_out, sizeof(double) * kDiagValues);
  if (e == cudaSuccess) e = dev_alloc(h, (void**)&h->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    int rc = cuda_fail(e, "handle set-up");
    release(h);
    return rc;
  }
  *out = h;
  return FDTD_OK;
}

int fdtd_create(const fdtd_params* params, double dt, int precision, fdtd_handle** out) {
  return create_handle(params, dt, precision, 0, out);
}

int fdtd_create_pml(const fdtd_params* params, double dt, double pml_percent, int precision, fdtd_handle** out) {
  if (!params || !out) return fail(FDTD_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (!(pml_percent >= 0.0 && pml_percent < 0.5))
    return fail(FDTD_ERR_INVALID_ARGUMENT, "pml_percent must be in [0, 0.5)");
  if (precision != FDTD_PRECISION_FP64)
    return fail(FDTD_ERR_UNSUPPORTED, "the PML layer runs in the FP64 form");
  fdtd_handle* h = nullptr;
  if (int rc = fdtd_create(params, dt, precision, &h)) return rc;
  h->pml = true;
  // src/FDTD_kokkos/FDTD_PML_kokkos.cpp:71-73
  const int n[3] = {params->Ni, params->Nj, params->Nk};
  const double d[3] = {params->dx, params->dy, params->dz};
  for (int a = 0; a < 3; ++a) h->pml_size[a] = static_cast<int>(static_cast<double>(n[a]) * pml_percent);
  int rc = FDTD_OK;
  for (int q = 0; q < 12 && rc == FDTD_OK; ++q) {
    cudaError_t e = dev_alloc(h, (void**)&h->split[q], sizeof(double) * h->g.cells);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->split[q], 0, sizeof(double) * h->g.cells, h->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "PML split fields");
  }
  for (int a = 0; a < 3 && rc == FDTD_OK; ++a) {
    // Conductivity along axis a (FDTD_PML_kokkos.cpp:108-136 with
    // kokkos_functors.h:182-189), zero inside; then the per-step decay and the
    // curl coefficient of the split-field updates (kokkos_functors.h:211-213,
    // :279-292), all in FP64 on the host as the reference evaluates them.
    const int pml = h->pml_size[a];
    std::vector<double> sigma(n[a], 0.0), decay(n[a]), coef2(n[a]);
    if (pml > 0) {
      const double sgm = -(kPmlOrder + 1.0) / 2.0 * std::log(kPmlR) / (static_cast<double>(pml) * d[a]);
      for (int i = 0; i < pml; ++i)
        sigma[i] = sgm * std::pow(static_cast<double>(pml - i) / static_cast<double>(pml), kPmlOrder);
      for (int i = n[a] - pml; i < n[a]; ++i)
        sigma[i] = sgm * std::pow(static_cast<double>(i + 1 + pml - n[a]) / static_cast<double>(pml), kPmlOrder);
    }
    for (int i = 0; i < n[a]; ++i) {
      decay[i] = std::exp(-sigma[i] * dt * kC);
      coef2[i] = sigma[i] != 0.0 ? (1.0 - std::exp(-sigma[i] * dt * kC)) / (sigma[i] * d[a]) : kC * dt / d[a];
    }
    cudaError_t e = dev_alloc(h, (void**)&h->pml_decay[a], sizeof(double) * n[a]);
    if (e == cudaSuccess) e = dev_alloc(h, (void**)&h->pml_coef2[a], sizeof(double) * n[a]);
    if (e == cudaSuccess)
      e = cudaMemcpy(h->pml_decay[a], decay.data(), sizeof(double) * n[a], cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(h->pml_coef2[a], coef2.data(), sizeof(double) * n[a], cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = cuda_fail(e, "PML tables");
  }
  if (rc == FDTD_OK) {
    const cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "PML set-up");
  }
  if (rc != FDTD_OK) {
    const std::string msg = g_last_error;
    fdtd_destroy(h);
    return fail(rc, msg);
  }
  *out = h;
  return FDTD_OK;
}

int fdtd_get_pml(fdtd_handle* h, int sizes[3]) {
  if (int rc = check_handle(h)) return rc;
  if (!sizes) return fail(FDTD_ERR_INVALID_ARGUMENT, "null output pointer");
  for (int a = 0; a < 3; ++a) sizes[a] = h->pml_size[a];
  return FDTD_OK;
}

int fdtd_destroy(fdtd_handle* h) {
  if (!h) return FDTD_OK;
  // Source buffers are not in `allocations` (they are replaced on update).
  DeviceGuard dg(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->d_src) cudaFree(h->d_src);
  if (h->d_tables) cudaFree(h->d_tables);
  if (h->d_tables_f) cudaFree(h->d_tables_f);
  h->d_src = nullptr;
  h->d_tables = nullptr;
  h->d_tables_f = nullptr;
  for (auto& t : h->timed) {
    cudaEventDestroy(t.start);
    cudaEventDestroy(t.stop);
  }
  for (cudaEvent_t e : h->event_pool) cudaEventDestroy(e);
  release(h);
  return FDTD_OK;
}

int fdtd_set_kernel_timing(fdtd_handle* h, int enabled) {
  if (int rc = check_handle(h)) return rc;
  h->timing = enabled != 0;
  return FDTD_OK;
}

int fdtd_kernel_times(fdtd_handle* h, double ms[FDTD_KERNEL_KINDS], int64_t launches[FDTD_KERNEL_KINDS]) {
  if (int rc = check_handle(h)) return rc;
  if (!ms || !launches) return fail(FDTD_ERR_INVALID_ARGUMENT, "null output pointer");
  DeviceGuard dg(h->device);
  FDTD_CUDA(cudaStreamSynchronize(h->stream), "synchronize for kernel times");
  for (int k = 0; k < FDTD_KERNEL_KINDS; ++k) {
    ms[k] = 0.0;
    launches[k] = 0;
  }
  for (auto& t : h->timed) {
    float m = 0.f;
    if (cudaEventElapsedTime(&m, t.start, t.stop) == cudaSuccess) {
      ms[t.kind] += m;
      launches[t.kind] += 1;
    }
    h->event_pool.push_back(t.start);
    h->event_pool.push_back(t.stop);
  }
  h->timed.clear();
  return FDTD_OK;
}

}  // extern "C"

namespace {

// n steps without FP16 rescans.  src/FDTD_kokkos/FDTD_kokkos.cpp:91-104
// repeated n times; the trailing B half step of one step and the leading one
// of the next share one sweep.
int step_sweeps(fdtd_handle* h, int64_t n) {
  if (h->form == Form::F64) {
    // FP64: every call ends at the step boundary (get_field hands out the
    // storage itself, so no half step may be left pending); B + t + t keeps
    // the two additions, so the merged sweeps are the reference's bits.
    if (int rc = run_b(h, 1)) return rc;
    for (int64_t s = 0; s < n; ++s) {
      const int apps = s + 1 < n ? 2 : 1;
      if (h->pml) {
        // FDTD_PML::update_fields (FDTD_PML_kokkos.cpp:162-189): B/2 inside,
        // B on the six layer slabs, E inside, E on the slabs, B/2 inside.
        if (int rc = run_pml(h, false)) return rc;
        if (int rc = run_e(h, h->host_step + s)) return rc;
        if (int rc = run_pml(h, true)) return rc;
        if (int rc = run_b(h, apps)) return rc;
      } else {
        if (int rc = run_e(h, h->host_step + s)) return rc;
        if (int rc = run_b(h, apps)) return rc;
      }
    }
    return FDTD_OK;
  }
  // FP32-arithmetic forms: the last step's trailing B half is left pending
  // and applied with the next step's leading half (or by the reader of B).
  const bool fused = h->pipeline != FDTD_PIPELINE_SPLIT;
  if (fused && b_first(h)) {
    // B-first sweeps: sweep s applies the B half steps that meet before step
    // s, then E; a depth-2 sweep does that for steps s and s+1.
    for (int64_t s = 0; s < n;) {
      const int depth = (h->fused_cfg.depth == 2 && s + 1 < n) ? 2 : 1;
      if (int rc = run_fused(h, h->host_step + s, h->b_pending ? 2 : 1, depth)) return rc;
      h->b_pending = true;
      h->b_side = false;
      s += depth;
    }
    return FDTD_OK;
  }
  // E-first sweeps (two cells per thread) or split sweeps: the leading half
  // (with a pending one: both halves), then per step E and the two halves
  // that follow it, except the last step's trailing one.
  if (int rc = run_b(h, h->b_pending ? 2 : 1)) return rc;
  h->b_pending = false;
  h->b_side = false;
  for (int64_t s = 0; s < n; ++s) {
    const bool last = s + 1 == n;
    if (fused && !last) {
      if (int rc = run_fused(h, h->host_step + s, 2)) return rc;
    } else {
      if (int rc = run_e(h, h->host_step + s)) return rc;
      if (!last)
        if (int rc = run_b(h, 2)) return rc;
    }
  }
  h->b_pending = true;
  return FDTD_OK;
}

// FP16 exponents (fdtd_fp16_autoscale, fdtd_set_fp16_autoscale).  From the
// stored peaks m_c, the field peak of component c is below 2^k_c with
// k_c = ceil(log2 m_c) - e_c, and k_all = max k_c.  The wanted exponent puts
// the component's peak at 2^target, but never more than 2^headroom above the
// strongest component's scale: e*_c = min(target - k_c, target + headroom -
// k_all) (a component with no field gets the bound).  `force` sets every
// exponent to e*; otherwise a component is re-encoded when its exponent is
// above the bound or 3 or more from e*.  Synchronous (reads six maxima).
// The rule itself (host only): from the stored peaks m_c (FP32 values of
// the stored halves' magnitudes) and the current exponents, the exponents
// to re-encode to (equal to `cur` where nothing changes).
void fp16_choose(const float peak[6], const int cur[6], int target, int headroom, bool force, int out[6]) {
  int k[6];
  bool has[6];
  int k_all = INT_MIN;
  for (int c = 0; c < 6; ++c) {
    const float m = peak[c];
    has[c] = m > 0.f && std::isfinite(m);
    k[c] = has[c] ? (int)std::ceil(std::log2((double)m)) - cur[c] : 0;
    if (has[c]) k_all = std::max(k_all, k[c]);
  }
  for (int c = 0; c < 6; ++c) {
    out[c] = cur[c];
    if (k_all == INT_MIN) continue;  // no field anywhere: nothing to go by
    const int bound = target + headroom - k_all;
    const int want = std::max(-60, std::min(60, has[c] ? std::min(target - k[c], bound) : bound));
    if (!force && cur[c] <= bound && std::abs(want - cur[c]) < 3) continue;
    out[c] = want;
  }
}

int fp16_rescan(fdtd_handle* h, int target, int headroom, bool force, int out[6]) {
  unsigned* d_max = reinterpret_cast<unsigned*>(h->d_diag_out);
  FDTD_CUDA(launch_f16_absmax(h->L, h->view().s16, d_max, h->stream), "FP16 peak scan");
  unsigned bits[6];
  FDTD_CUDA(cudaMemcpyAsync(bits, d_max, sizeof(bits), cudaMemcpyDeviceToHost, h->stream), "FP16 peak scan");
  FDTD_CUDA(cudaStreamSynchronize(h->stream), "FP16 peak scan");
  float peak[6];
  std::memcpy(peak, bits, sizeof(peak));
  int want[6];
  fp16_choose(peak, h->fp16_exp, target, headroom, force, want);
  for (int c = 0; c < 6; ++c) {
    const int cur = h->fp16_exp[c];
    if (want[c] != cur) {
      FDTD_CUDA(launch_f16_rescale(static_cast<__half*>(h->field[c]), h->L.elems(), want[c] - cur, h->stream),
                "FP16 rescale");
      h->fp16_exp[c] = want[c];
      h->b_side = false;
    }
    if (out) out[c] = h->fp16_exp[c];
  }
  return FDTD_OK;
}

}  // namespace

extern "C" {

int fdtd_step(fdtd_handle* h, int64_t n) {
  if (int rc = check_handle(h)) return rc;
  if (n < 0) return fail(FDTD_ERR_INVALID_ARGUMENT, "negative step count");
  if (h->zhalo)
    return fail(FDTD_ERR_UNSUPPORTED, "a z slab steps through fdtd_slab_sweep and fdtd_slab_exchange");
  if (n == 0) return FDTD_OK;
  DeviceGuard dg(h->device);
  const int every = h->form == Form::F16 ? h->fp16_autoscale_every : 0;
  while (n > 0) {
    const int64_t m = every > 0 ? std::min<int64_t>(n, every - h->fp16_autoscale_count) : n;
    if (int rc = step_sweeps(h, m)) return rc;
    h->host_step += m;
    n -= m;
    if (every > 0 && (h->fp16_autoscale_count += (int)m) >= every) {
      h->fp16_autoscale_count = 0;
      if (int rc = fp16_rescan(h, h->fp16_autoscale_target, h->fp16_autoscale_headroom, false, nullptr)) return rc;
    }
  }
  return FDTD_OK;
}

int fdtd_update_fields(fdtd_handle* h) { return fdtd_step(h, 1); }

int fdtd_zeroed_currents(fdtd_handle* h) {
  if (int rc = check_handle(h)) return rc;
  DeviceGuard dg(h->device);
  // src/FDTD_kokkos/FDTD_kokkos.cpp:69-73.  The E update keeps reading J if a
  // J address was handed out (the holder may write it again).
  if (h->form == Form::F64) {
    for (int c = 6; c < 9; ++c)
      FDTD_CUDA(cudaMemsetAsync(h->field[c], 0, sizeof(double) * h->g.cells, h->stream), "zero J");
  } else if (h->jf[0]) {
    for (int c = 0; c < 3; ++c)
      FDTD_CUDA(cudaMemsetAsync(h->jf[c], 0, sizeof(float) * h->g.cells, h->stream), "zero J");
    h->dense_j = false;
  }
  return FDTD_OK;
}

int fdtd_get_field(fdtd_handle* h, int comp, double** device_ptr) {
  if (int rc = check_handle(h)) return rc;
  if (!device_ptr) return fail(FDTD_ERR_INVALID_ARGUMENT, "null output pointer");
  if (comp < FDTD_EX || comp > FDTD_JZ)
    return fail(FDTD_ERR_LOGIC, "ERROR: Invalid field component");  // FDTD_kokkos.cpp:87
  if (h->form != Form::F64)
    return fail(FDTD_ERR_UNSUPPORTED, "device field addresses are FP64-only; use fdtd_copy_field_*");
  if (comp >= FDTD_JX) h->dense_j = true;
  *device_ptr = (double*)h->field[comp];
  return FDTD_OK;
}

int fdtd_copy_field_to_host(fdtd_handle* h, int comp, double* host, size_t n) {
  if (int rc = check_handle(h)) return rc;
  if (comp < FDTD_EX || comp > FDTD_JZ) return fail(FDTD_ERR_LOGIC, "ERROR: Invalid field component");
  if (!host || (int64_t)n != h->g.cells) return fail(FDTD_ERR_INVALID_ARGUMENT, "host buffer size mismatch");
  DeviceGuard dg(h->device);
  if (h->form == Form::F64) {
    FDTD_CUDA(cudaMemcpyAsync(host, h->field[comp], sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream),
              "copy field to host");
    FDTD_CUDA(cudaStreamSynchronize(h->stream), "copy field to host");
    return FDTD_OK;
  }
  if (comp >= FDTD_JX && !h->jf[0]) {  // never written: zero
    std::memset(host, 0, sizeof(double) * n);
    return FDTD_OK;
  }
  StateView v;
  if (int rc = read_view(h, &v)) return rc;
  if (comp < FDTD_JX) {
    if (double* dev = device_alias(host)) {
      // pinned host memory the device addresses: convert in one pass
      FDTD_CUDA(launch_export(v, comp, dev, 0, (int64_t)n, h->stream), "copy field to host");
      FDTD_CUDA(cudaStreamSynchronize(h->stream), "copy field to host");
      return FDTD_OK;
    }
  }
  if (int rc = ensure_staging(h)) return rc;
  for (int64_t off = 0; off < (int64_t)n; off += kStagingElems) {
    const int64_t m = std::min<int64_t>(kStagingElems, (int64_t)n - off);
    cudaError_t e;
    if (comp >= FDTD_JX) {
      // J is stored as FP32: widen on the host side of the copy.
      std::vector<float> tmp(m);
      e = cudaMemcpyAsync(tmp.data(), h->jf[comp - FDTD_JX] + off, sizeof(float) * m,
                          cudaMemcpyDeviceToHost, h->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
      if (e != cudaSuccess) return cuda_fail(e, "copy current to host");
      for (int64_t t = 0; t < m; ++t) host[off + t] = tmp[t];
      continue;
    }
    e = launch_export(v, comp, h->d_staging, off, m, h->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(host + off, h->d_staging, sizeof(double) * m, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "copy field to host");
  }
  return FDTD_OK;
}

int fdtd_export_field(fdtd_handle* h, int comp, int64_t offset, int64_t count, double* device_dst) {
  if (int rc = check_handle(h)) return rc;
  if (comp < FDTD_EX || comp > FDTD_BZ) return fail(FDTD_ERR_LOGIC, "ERROR: Invalid field component");
  if (!device_dst || offset < 0 || count < 0 || offset + count > h->g.cells)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "export range outside the grid");
  DeviceGuard dg(h->device);
  StateView v;
  if (int rc = read_view(h, &v)) return rc;
  FDTD_CUDA(launch_export(v, comp, device_dst, offset, count, h->stream), "export field");
  return FDTD_OK;
}

int fdtd_copy_field_from_host(fdtd_handle* h, int comp, const double* host, size_t n) {
  if (int rc = check_handle(h)) return rc;
  if (comp < FDTD_EX || comp > FDTD_JZ) return fail(FDTD_ERR_LOGIC, "ERROR: Invalid field component");
  if (!host || (int64_t)n != h->g.cells) return fail(FDTD_ERR_INVALID_ARGUMENT, "host buffer size mismatch");
  DeviceGuard dg(h->device);
  if (comp < FDTD_JX)
    if (int rc = resolve_pending(h)) return rc;  // the pending half reads the E and B being replaced
  if (h->form == Form::F64) {
    FDTD_CUDA(cudaMemcpyAsync(h->field[comp], host, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream),
              "copy field from host");
    FDTD_CUDA(cudaStreamSynchronize(h->stream), "copy field from host");
    if (comp >= FDTD_JX) h->dense_j = true;
    return FDTD_OK;
  }
  if (comp < FDTD_JX) {
    if (double* dev = device_alias(host)) {
      // pinned host memory the device addresses: convert in one pass
      FDTD_CUDA(launch_import(h->view(), comp, dev, 0, (int64_t)n, h->stream), "copy field from host");
      FDTD_CUDA(cudaStreamSynchronize(h->stream), "copy field from host");
      return FDTD_OK;
    }
  }
  if (int rc = ensure_staging(h)) return rc;
  if (comp >= FDTD_JX) {
    if (int rc = ensure_jf(h)) return rc;
    h->dense_j = true;
  }
  StateView v = h->view();
  for (int64_t off = 0; off < (int64_t)n; off += kStagingElems) {
    const int64_t m = std::min<int64_t>(kStagingElems, (int64_t)n - off);
    cudaError_t e = cudaMemcpyAsync(h->d_staging, host + off, sizeof(double) * m,
                                    cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
      if (comp >= FDTD_JX) e = launch_to_f32(h->d_staging, h->jf[comp - FDTD_JX] + off, m, h->stream);
      else e = launch_import(v, comp, h->d_staging, off, m, h->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "copy field from host");
  }
  return FDTD_OK;
}

int fdtd_add_source(fdtd_handle* h, const fdtd_source* src, int* index) {
  if (int rc = check_handle(h)) return rc;
  if (!src) return fail(FDTD_ERR_INVALID_ARGUMENT, "null source");
  if (src->comp_mask <= 0 || src->comp_mask > 7) return fail(FDTD_ERR_INVALID_ARGUMENT, "source comp_mask must be 1..7");
  // a z slab takes sources in the coordinates of the whole grid
  const int nk_grid = h->zhalo ? h->slab_nk_global : h->g.Nk;
  if (src->ni <= 0 || src->nj <= 0 || src->nk <= 0 || src->ni > h->g.Ni || src->nj > h->g.Nj ||
      src->nk > nk_grid)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "source box extents must be in 1..N per axis");
  if (src->i0 < 0 || src->i0 >= h->g.Ni || src->j0 < 0 || src->j0 >= h->g.Nj || src->k0 < 0 ||
      src->k0 >= nk_grid)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "source box origin outside the grid");
  if (!src->gx || !src->gy || !src->gz || src->n_amp < 0 || (src->n_amp > 0 && !src->amp))
    return fail(FDTD_ERR_INVALID_ARGUMENT, "source tables missing");
  DeviceGuard dg(h->device);
  HostSource hs;
  hs.s = *src;
  hs.s.gx = hs.s.gy = hs.s.gz = hs.s.amp = nullptr;
  hs.gx.assign(src->gx, src->gx + src->ni);
  hs.gy.assign(src->gy, src->gy + src->nj);
  if (src->n_amp > 0) hs.amp.assign(src->amp, src->amp + src->n_amp);
  // The pieces to register: the whole box, or, on a z slab, each run of the
  // box's planes (taken mod Nk) that lies in the slab's owned planes and is
  // contiguous there, in the slab's storage numbering (k0 >= 1, and the
  // piece ends at or before the halo above, so the kernels' index wrap never
  // maps another plane into it).  A cell lies in one piece at most, so its
  // sources still add up in registration order.
  std::vector<HostSource> pieces;
  if (!h->zhalo) {
    hs.gz.assign(src->gz, src->gz + src->nk);
    pieces.push_back(std::move(hs));
  } else {
    const int kb = h->slab_k0, ke = h->slab_k0 + h->g.Nk;
    int t = 0;
    while (t < src->nk) {
      const int kg = (src->k0 + t) % nk_grid;
      if (kg < kb || kg >= ke) {
        ++t;
        continue;
      }
      int len = 1;
      while (t + len < src->nk && (src->k0 + t + len) % nk_grid == kg + len && kg + len < ke) ++len;
      HostSource piece = hs;
      piece.s.k0 = kg - kb + h->zhalo;
      piece.s.nk = len;
      piece.gz.assign(src->gz + t, src->gz + t + len);
      pieces.push_back(std::move(piece));
      t += len;
    }
  }
  if ((int)(h->sources.size() + pieces.size()) > kMaxSources)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "too many sources");
  const size_t before = h->sources.size();
  for (HostSource& q : pieces) h->sources.push_back(std::move(q));
  if (int rc = upload_sources(h)) {
    h->sources.resize(before);
    return rc;
  }
  if (index) *index = h->source_calls;
  ++h->source_calls;
  return FDTD_OK;
}

int fdtd_clear_sources(fdtd_handle* h) {
  if (int rc = check_handle(h)) return rc;
  DeviceGuard dg(h->device);
  h->sources.clear();
  h->source_calls = 0;
  return upload_sources(h);
}

int fdtd_get_step(fdtd_handle* h, int64_t* step) {
  if (int rc = check_handle(h)) return rc;
  if (!step) return fail(FDTD_ERR_INVALID_ARGUMENT, "null output pointer");
  *step = h->host_step;
  return FDTD_OK;
}

int fdtd_set_step(fdtd_handle* h, int64_t step) {
  if (int rc = check_handle(h)) return rc;
  if (step < 0) return fail(FDTD_ERR_INVALID_ARGUMENT, "negative step");
  h->host_step = step;
  return FDTD_OK;
}

int fdtd_set_pipeline(fdtd_handle* h, int pipeline, int tile_y, int kchunk, int cells_per_thread) {
  if (int rc = check_handle(h)) return rc;
  if (pipeline < FDTD_PIPELINE_AUTO || pipeline > FDTD_PIPELINE_FUSED)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "invalid pipeline");
  if (tile_y != 0 && tile_y != 6 && tile_y != 14 && tile_y != 30)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "tile_y must be 0 (default), 6, 14 or 30");
  if (tile_y == 30 && cells_per_thread == 2)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "tile_y 30 needs cells_per_thread 1");
  if (kchunk < 0) return fail(FDTD_ERR_INVALID_ARGUMENT, "kchunk must be >= 0");
  if (cells_per_thread < 0 || cells_per_thread > 2)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "cells_per_thread must be 0 (default), 1 or 2");
  if (h->zhalo && cells_per_thread == 2)
    return fail(FDTD_ERR_UNSUPPORTED, "a z slab's fused sweep has one cell per thread");
  if (h->fused_cfg.depth == 2 && (cells_per_thread == 2 || tile_y == 30))
    return fail(FDTD_ERR_INVALID_ARGUMENT, "the depth-2 sweep needs cells_per_thread 1 and tile_y 6 or 14");
  h->pipeline = pipeline;
  h->fused_cfg.tile_y = tile_y ? tile_y : 14;
  h->fused_cfg.kchunk = kchunk ? kchunk : 48;
  h->fused_cfg.cells_per_thread = cells_per_thread ? cells_per_thread : 1;
  return FDTD_OK;
}

int fdtd_autotune(fdtd_handle* h, int sweeps, int reuse, fdtd_tune_result* out) {
  if (int rc = check_handle(h)) return rc;
  if (h->form == Form::F64) return fail(FDTD_ERR_UNSUPPORTED, "the FP64 form has one pipeline; nothing to tune");
  if (h->zhalo) return fail(FDTD_ERR_UNSUPPORTED, "a z slab has no autotuner (fdtd_set_pipeline sets its fused sweep's shape)");
  if (sweeps <= 0) sweeps = 10;
  DeviceGuard dg(h->device);
  const TuneKey key{(int)h->form, h->g.Ni, h->g.Nj, h->g.Nk};
  fdtd_tune_result best{};
  bool cached = false;
  if (reuse) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      best = it->second;
      cached = true;
    }
  }
  if (!cached) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    FDTD_CUDA(cudaEventCreate(&e0), "autotune events");
    if (cudaEventCreate(&e1) != cudaSuccess) {
      cudaEventDestroy(e0);
      return fail(FDTD_ERR_CUDA, "autotune events");
    }
    best.ms_per_sweep = 1e30;
    // candidates: (depth, cells per thread, tile rows, chunk)
    std::vector<std::tuple<int, int, int, int>> cands;
    for (int cpt = 1; cpt <= 2; ++cpt)
      for (int ry : (cpt == 1 ? std::vector<int>(std::begin(kTuneRows1), std::end(kTuneRows1))
                              : std::vector<int>(std::begin(kTuneRows2), std::end(kTuneRows2))))
        for (int kc : kTuneChunks) cands.emplace_back(1, cpt, ry, kc);
    for (int ry : kTuneRowsDepth2)
      for (int kc : kTuneChunksDepth2) cands.emplace_back(2, 1, ry, kc);
    const int depth_before = h->fused_cfg.depth;
    int rc = FDTD_OK;
    // An E-first (two-cell) sweep needs a B half sweep at the start of every
    // call: with update_fields called once per step, as the reference's
    // callers do, that is one more sweep per step, which its candidates pay.
    double ms_lead_half = -1.0;
    for (const auto& cand : cands) {
      const int depth = std::get<0>(cand);
      h->fused_cfg.depth = 1;
      h->fused_cfg.cells_per_thread = std::get<1>(cand);
      h->fused_cfg.tile_y = std::get<2>(cand);
      h->fused_cfg.kchunk = std::get<3>(cand);
      if ((rc = ensure_alt(h)) != FDTD_OK) break;
      // the timed sweeps read the current copy (a depth-2 sweep also rewrites
      // its ghost copies with the values they hold) and write the second one
      cudaError_t e = launch_fused_sweep(h, h->host_step, 2, depth);  // warm-up
      if (e == cudaSuccess) e = cudaEventRecord(e0, h->stream);
      for (int q = 0; q < sweeps && e == cudaSuccess; ++q) e = launch_fused_sweep(h, h->host_step, 2, depth);
      if (e == cudaSuccess) e = cudaEventRecord(e1, h->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess) {
        rc = cuda_fail(e, "autotune sweep");
        break;
      }
      best.candidates += 1;
      if (std::get<1>(cand) == 2 && ms_lead_half < 0.0) {
        // the column B half sweep the E-first pipeline starts a call with,
        // timed into the second copy's B arrays (the state is only read)
        const StateView cur = h->view(), side = h->view_side();
        e = cudaEventRecord(e0, h->stream);
        for (int q = 0; q < sweeps && e == cudaSuccess; ++q) {
          switch (h->form) {
            case Form::F32: e = launch_b_f32_into(h->L, cur.s32, side.s32, h->cs, 0, h->g.Nk, h->stream); break;
            case Form::F32C: e = launch_b_f32_into(h->L, cur.s32c, side.s32c, h->cs, 0, h->g.Nk, h->stream); break;
            case Form::F16: e = launch_b_f32_into(h->L, cur.s16, side.s16, h->cs, 0, h->g.Nk, h->stream); break;
            default: e = cudaErrorInvalidValue; break;
          }
        }
        if (e == cudaSuccess) e = cudaEventRecord(e1, h->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float mh = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&mh, e0, e1);
        if (e != cudaSuccess) {
          rc = cuda_fail(e, "autotune B half sweep");
          break;
        }
        ms_lead_half = mh / sweeps;
      }
      const double per_step = ms / sweeps / depth + (std::get<1>(cand) == 2 ? ms_lead_half : 0.0);
      if (per_step < best.ms_per_sweep) {
        best.ms_per_sweep = per_step;
        best.tile_y = std::get<2>(cand);
        best.kchunk = std::get<3>(cand);
        best.cells_per_thread = std::get<1>(cand);
        best.depth = depth;
      }
    }
    h->fused_cfg.depth = depth_before;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    h->b_side = false;  // the timed sweeps wrote the second copy
    if (rc != FDTD_OK) return rc;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = best;
  }
  h->fused_cfg.tile_y = best.tile_y;
  h->fused_cfg.kchunk = best.kchunk;
  h->fused_cfg.cells_per_thread = best.cells_per_thread;
  h->fused_cfg.depth = best.depth;
  if (int rc = ensure_alt(h)) return rc;
  if (out) {
    *out = best;
    out->cached = cached ? 1 : 0;
  }
  return FDTD_OK;
}

int fdtd_field_sums(fdtd_handle* h, double out[FDTD_DIAG_COUNT]) {
  if (int rc = check_handle(h)) return rc;
  if (!out) return fail(FDTD_ERR_INVALID_ARGUMENT, "null output pointer");
  DeviceGuard dg(h->device);
  const int nb = diag_blocks_for(h->g.cells, kMaxDiagBlocks);
  StateView v;
  if (int rc = read_view(h, &v)) return rc;
  FDTD_CUDA(launch_field_sums(v, h->d_partials, nb, h->d_diag_out, h->stream), "field sums");
  FDTD_CUDA(cudaMemcpyAsync(out, h->d_diag_out, sizeof(double) * kDiagValues, cudaMemcpyDeviceToHost,
                            h->stream),
            "field sums readback");
  FDTD_CUDA(cudaStreamSynchronize(h->stream), "field sums");
  return FDTD_OK;
}

int fdtd_get_params(fdtd_handle* h, fdtd_params* params, double* dt, int* precision) {
  if (int rc = check_handle(h)) return rc;
  if (params) *params = h->p;
  if (dt) *dt = h->dt;
  if (precision) *precision = h->precision;
  return FDTD_OK;
}

int fdtd_set_stream(fdtd_handle* h, void* stream) {
  if (int rc = check_handle(h)) return rc;
  DeviceGuard dg(h->device);
  FDTD_CUDA(cudaStreamSynchronize(h->stream), "synchronize previous stream");
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return FDTD_OK;
}

int fdtd_synchronize(fdtd_handle* h) {
  if (int rc = check_handle(h)) return rc;
  DeviceGuard dg(h->device);
  FDTD_CUDA(cudaStreamSynchronize(h->stream), "synchronize");
  int status = 0;
  FDTD_CUDA(cudaMemcpy(&status, h->d_err, sizeof(int), cudaMemcpyDeviceToHost), "read device status");
  if (status != 0) {
    cudaMemset(h->d_err, 0, sizeof(int));
    return fail(FDTD_ERR_TIMEOUT, (status & 2) ? "a bounded wait in a step kernel gave up, and so did the wait for its "
                                                 "copies in flight; results of that step are invalid"
                                               : "a bounded wait in a step kernel gave up; results of that step are "
                                                 "invalid");
  }
  return FDTD_OK;
}

int fdtd_fp16_autoscale(fdtd_handle* h, int target_log2, int headroom_log2, int exponents[6]) {
  if (int rc = check_handle(h)) return rc;
  if (h->form != Form::F16) return fail(FDTD_ERR_UNSUPPORTED, "scales apply to the FP16_SCALED form only");
  if (target_log2 < 0 || target_log2 > 15) return fail(FDTD_ERR_INVALID_ARGUMENT, "target_log2 must be in [0, 15]");
  if (headroom_log2 < 0 || headroom_log2 > 60) return fail(FDTD_ERR_INVALID_ARGUMENT, "headroom_log2 must be in [0, 60]");
  DeviceGuard dg(h->device);
  if (int rc = fp16_rescan(h, target_log2, headroom_log2, true, exponents)) return rc;
  FDTD_CUDA(cudaStreamSynchronize(h->stream), "FP16 rescale");
  return FDTD_OK;
}

int fdtd_fp16_choose_exponents(const float peaks[6], const int current[6], int target_log2, int headroom_log2,
                               int force, int exponents[6]) {
  if (!peaks || !current || !exponents) return fail(FDTD_ERR_INVALID_ARGUMENT, "null pointer");
  if (target_log2 < 0 || target_log2 > 15) return fail(FDTD_ERR_INVALID_ARGUMENT, "target_log2 must be in [0, 15]");
  if (headroom_log2 < 0 || headroom_log2 > 60) return fail(FDTD_ERR_INVALID_ARGUMENT, "headroom_log2 must be in [0, 60]");
  for (int c = 0; c < 6; ++c)
    if (current[c] < -60 || current[c] > 60) return fail(FDTD_ERR_INVALID_ARGUMENT, "exponents must be in [-60, 60]");
  fp16_choose(peaks, current, target_log2, headroom_log2, force != 0, exponents);
  return FDTD_OK;
}

int fdtd_set_fp16_autoscale(fdtd_handle* h, int every_steps, int target_log2, int headroom_log2) {
  if (int rc = check_handle(h)) return rc;
  if (h->form != Form::F16) return fail(FDTD_ERR_UNSUPPORTED, "scales apply to the FP16_SCALED form only");
  if (every_steps < 0) return fail(FDTD_ERR_INVALID_ARGUMENT, "every_steps must be >= 0");
  if (target_log2 < 0 || target_log2 > 15) return fail(FDTD_ERR_INVALID_ARGUMENT, "target_log2 must be in [0, 15]");
  if (headroom_log2 < 0 || headroom_log2 > 60) return fail(FDTD_ERR_INVALID_ARGUMENT, "headroom_log2 must be in [0, 60]");
  h->fp16_autoscale_every = every_steps;
  h->fp16_autoscale_target = target_log2;
  h->fp16_autoscale_headroom = headroom_log2;
  h->fp16_autoscale_count = 0;
  return FDTD_OK;
}

int fdtd_get_fp16_exponents(fdtd_handle* h, int exponents[6]) {
  if (int rc = check_handle(h)) return rc;
  if (!exponents) return fail(FDTD_ERR_INVALID_ARGUMENT, "null exponents");
  for (int c = 0; c < 6; ++c) exponents[c] = h->fp16_exp[c];
  return FDTD_OK;
}

int fdtd_set_temporal_depth(fdtd_handle* h, int depth) {
  if (int rc = check_handle(h)) return rc;
  if (depth != 1 && depth != 2) return fail(FDTD_ERR_INVALID_ARGUMENT, "depth must be 1 or 2");
  if (depth == 2) {
    if (h->form == Form::F64 || h->zhalo || h->pml)
      return fail(FDTD_ERR_UNSUPPORTED, "the depth-2 sweep runs the FP32-arithmetic forms of whole grids");
    if (h->fused_cfg.cells_per_thread != 1 || h->fused_cfg.tile_y == 30)
      return fail(FDTD_ERR_INVALID_ARGUMENT, "the depth-2 sweep needs cells_per_thread 1 and tile_y 6 or 14");
  }
  h->fused_cfg.depth = depth;
  return FDTD_OK;
}

int fdtd_set_wait_limit(fdtd_handle* h, int64_t polls, int withhold_loads) {
  if (int rc = check_handle(h)) return rc;
  if (polls < 0 || polls > (int64_t)kMaxBarrierPolls)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "polls must be in [0, 2^24] (0: the default)");
  h->wait_polls = polls ? (uint32_t)polls : kMaxBarrierPolls;
  h->withhold_loads = withhold_loads ? 1 : 0;
  return FDTD_OK;
}

int fdtd_set_fp64_arith(fdtd_handle* h, int arith) {
  if (int rc = check_handle(h)) return rc;
  if (arith != FDTD_FP64_BITWISE && arith != FDTD_FP64_CONTRACTED)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "invalid FP64 arithmetic mode");
  if (h->form != Form::F64) return fail(FDTD_ERR_UNSUPPORTED, "the arithmetic mode applies to the FP64 form only");
  h->fp64_fma = arith == FDTD_FP64_CONTRACTED;
  return FDTD_OK;
}

int fdtd_set_fp16_exponents(fdtd_handle* h, const int exponents[6]) {
  if (int rc = check_handle(h)) return rc;
  if (!exponents) return fail(FDTD_ERR_INVALID_ARGUMENT, "null exponents");
  if (h->form != Form::F16) return fail(FDTD_ERR_UNSUPPORTED, "exponents apply to the FP16_SCALED form only");
  for (int c = 0; c < 6; ++c)
    // |e| <= 60 keeps every coefficient times 2^(e_dst - e_src) a finite float
    if (exponents[c] < -60 || exponents[c] > 60) return fail(FDTD_ERR_INVALID_ARGUMENT, "exponent out of range [-60, 60]");
  // Rescale stored values so the fields they represent are unchanged.
  DeviceGuard dg(h->device);
  if (int rc = resolve_pending(h)) return rc;
  if (int rc = ensure_staging(h)) return rc;
  for (int c = 0; c < 6; ++c) {
    if (exponents[c] == h->fp16_exp[c]) continue;
    for (int64_t off = 0; off < h->g.cells; off += kStagingElems) {
      const int64_t m = std::min<int64_t>(kStagingElems, h->g.cells - off);
      FDTD_CUDA(launch_export(h->view(), c, h->d_staging, off, m, h->stream), "rescale export");
      const int old = h->fp16_exp[c];
      h->fp16_exp[c] = exponents[c];
      cudaError_t e = launch_import(h->view(), c, h->d_staging, off, m, h->stream);
      h->fp16_exp[c] = old;
      if (e != cudaSuccess) return cuda_fail(e, "rescale import");
    }
    h->fp16_exp[c] = exponents[c];
  }
  FDTD_CUDA(cudaStreamSynchronize(h->stream), "rescale");
  return FDTD_OK;
}


// ---------------------------------------------------------------------------
// Compact forms of the entry points above.

int fdtd_energy(fdtd_handle* h, double out[3]) {
  if (!out) return fail(FDTD_ERR_INVALID_ARGUMENT, "null output pointer");
  double sums[FDTD_DIAG_COUNT];
  if (int rc = fdtd_field_sums(h, sums)) return rc;
  const double dv8pi = h->p.dx * h->p.dy * h->p.dz / (8.0 * kPi);
  out[0] = (sums[FDTD_DIAG_EX2] + sums[FDTD_DIAG_EY2] + sums[FDTD_DIAG_EZ2]) * dv8pi;
  out[1] = (sums[FDTD_DIAG_BX2] + sums[FDTD_DIAG_BY2] + sums[FDTD_DIAG_BZ2]) * dv8pi;
  out[2] = out[0] + out[1];
  return FDTD_OK;
}

int fdtd_set_sources(fdtd_handle* h, const fdtd_source* src, int n) {
  if (int rc = check_handle(h)) return rc;
  if (n < 0 || (n > 0 && !src)) return fail(FDTD_ERR_INVALID_ARGUMENT, "invalid source list");
  const std::vector<HostSource> keep = h->sources;
  const int calls = h->source_calls;
  if (int rc = fdtd_clear_sources(h)) return rc;
  for (int q = 0; q < n; ++q) {
    if (int rc = fdtd_add_source(h, &src[q], nullptr)) {
      // leave the previous list in place
      const std::string msg = fdtd_last_error();
      DeviceGuard dg(h->device);
      h->sources = keep;
      h->source_calls = calls;
      upload_sources(h);
      return fail(rc, msg);
    }
  }
  return FDTD_OK;
}

int fdtd_field_device_ptr(fdtd_handle* h, int comp, void** device_ptr) {
  if (!device_ptr) return fail(FDTD_ERR_INVALID_ARGUMENT, "null output pointer");
  double* p = nullptr;
  if (int rc = fdtd_get_field(h, comp, &p)) return rc;
  *device_ptr = p;
  return FDTD_OK;
}

int fdtd_copy_field(fdtd_handle* h, int comp, double* host, int dir) {
  if (int rc = check_handle(h)) return rc;
  if (dir != FDTD_TO_HOST && dir != FDTD_FROM_HOST) return fail(FDTD_ERR_INVALID_ARGUMENT, "invalid direction");
  const size_t n = (size_t)h->g.cells;
  return dir == FDTD_TO_HOST ? fdtd_copy_field_to_host(h, comp, host, n) : fdtd_copy_field_from_host(h, comp, host, n);
}

int fdtd_sync(fdtd_handle* h) { return fdtd_synchronize(h); }

// ---------------------------------------------------------------------------
// z slabs: the decomposition of the reference's coarray program
// (coarray/fdtd.F90:90-98), where image s owns a range of z planes and reads
// the neighbours' boundary planes of E (for B at k+1, kokkos_functors.h:141)
// and of B (for E at k-1, :78) between the sweeps.

int fdtd_slab_create(const fdtd_params* params, double dt, int precision, int k_begin, int k_end,
                     fdtd_handle** out) {
  if (!params || !out) return fail(FDTD_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (params->Ni <= 0 || params->Nj <= 0 || params->Nk <= 0 || !(dt > 0))
    return fail(FDTD_ERR_INVALID_ARGUMENT, "ERROR: invalid parameters");
  if (k_begin < 0 || k_end <= k_begin || k_end > params->Nk)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "slab planes must satisfy 0 <= k_begin < k_end <= Nk");
  fdtd_params owned = *params;
  owned.Nk = k_end - k_begin;
  owned.az = params->az + k_begin * params->dz;
  owned.bz = owned.az + owned.Nk * params->dz;
  fdtd_handle* h = nullptr;
  if (int rc = create_handle(&owned, dt, precision, 1, &h)) return rc;
  h->slab_k0 = k_begin;
  h->slab_nk_global = params->Nk;
  h->pipeline = FDTD_PIPELINE_SPLIT;
  *out = h;
  return FDTD_OK;
}

int fdtd_slab_info(fdtd_handle* h, int* k_begin, int* k_end, int* nk_global) {
  if (int rc = check_handle(h)) return rc;
  const bool slab = h->zhalo != 0;
  if (k_begin) *k_begin = slab ? h->slab_k0 : 0;
  if (k_end) *k_end = slab ? h->slab_k0 + h->g.Nk : h->g.Nk;
  if (nk_global) *nk_global = slab ? h->slab_nk_global : h->g.Nk;
  return FDTD_OK;
}

int fdtd_slab_sweep(fdtd_handle* h, int sweep) {
  if (int rc = check_handle(h)) return rc;
  if (h->pml) return fail(FDTD_ERR_UNSUPPORTED, "the PML form steps through fdtd_step");
  if (sweep < FDTD_SWEEP_B_HALF || sweep > FDTD_SWEEP_STEP) return fail(FDTD_ERR_INVALID_ARGUMENT, "invalid sweep");
  DeviceGuard dg(h->device);
  switch (sweep) {
    case FDTD_SWEEP_STEP:
      // One B-first fused sweep (the single-grid step's kernel, over the
      // owned planes of the storage): the pending half with the leading one,
      // then E; the trailing half stays pending.
      if (h->form == Form::F64) return fail(FDTD_ERR_UNSUPPORTED, "the FP64 form runs the split sweeps");
      if (h->fused_cfg.cells_per_thread != 1)
        return fail(FDTD_ERR_UNSUPPORTED, "a z slab's fused sweep has one cell per thread");
      if (int rc = run_fused(h, h->host_step, h->b_pending ? 2 : 1)) return rc;
      ++h->host_step;
      h->b_pending = true;
      h->b_side = false;
      return FDTD_OK;
    case FDTD_SWEEP_E:
      if (int rc = resolve_pending(h)) return rc;
      if (int rc = run_e(h, h->host_step)) return rc;
      ++h->host_step;
      return FDTD_OK;
    case FDTD_SWEEP_B_DEFER:
      // the FP64 form hands out its storage (fdtd_get_field): nothing may be
      // left pending there
      if (h->form == Form::F64) return fail(FDTD_ERR_UNSUPPORTED, "the FP64 form applies every half step");
      if (h->b_pending) return fail(FDTD_ERR_LOGIC, "a B half step is already pending");
      h->b_pending = true;
      h->b_side = false;
      return FDTD_OK;
    default:
      // with a half step pending, it is the first of the half steps applied
      if (int rc = run_b(h, sweep == FDTD_SWEEP_B_DOUBLE ? 2 : 1)) return rc;
      h->b_pending = false;
      h->b_side = false;
      return FDTD_OK;
  }
}

}  // extern "C"

namespace {

// Device address and byte size of one stored plane of component c (0..5):
// its E/B words (part 0) or its compensation words (part 1).
unsigned char* slab_plane(fdtd_handle* h, int c, int plane, int part, size_t* bytes) {
  const int64_t pe = h->form == Form::F64 ? h->g.plane : h->L.pplane;
  const int64_t k = plane == FDTD_PLANE_HALO_BELOW ? -1
                    : plane == FDTD_PLANE_FIRST    ? 0
                    : plane == FDTD_PLANE_LAST     ? h->g.Nk - 1
                                                   : h->g.Nk;
  const size_t eb = part == 0 ? elem_bytes(h->form) : sizeof(LoT);
  unsigned char* base = part == 0 ? static_cast<unsigned char*>(h->field[c]) : reinterpret_cast<unsigned char*>(h->lo[c]);
  *bytes = eb * (size_t)pe;
  return base + (int64_t)eb * pe * k;
}

}  // namespace

extern "C" {

int fdtd_slab_plane(fdtd_handle* h, int comp, int plane, int part, void** device_ptr, size_t* bytes) {
  if (int rc = check_handle(h)) return rc;
  if (!device_ptr || !bytes) return fail(FDTD_ERR_INVALID_ARGUMENT, "null output pointer");
  if (comp < FDTD_EX || comp > FDTD_BZ) return fail(FDTD_ERR_LOGIC, "ERROR: Invalid field component");
  if (plane < FDTD_PLANE_HALO_BELOW || plane > FDTD_PLANE_HALO_ABOVE)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "invalid plane");
  if (!h->zhalo && (plane == FDTD_PLANE_HALO_BELOW || plane == FDTD_PLANE_HALO_ABOVE))
    return fail(FDTD_ERR_INVALID_ARGUMENT, "only a z slab has halo planes");
  if (part != 0 && !(part == 1 && h->form == Form::F32C))
    return fail(FDTD_ERR_INVALID_ARGUMENT, "part 1 (compensation words) exists in the FP32_COMP form only");
  // Planes are handed out as stored: with a B half step pending, B lacks it
  // on every slab alike (the schedules exchange B that way, and the next
  // sweep applies the half on both sides of each face).
  *device_ptr = slab_plane(h, comp, plane, part, bytes);
  return FDTD_OK;
}

int fdtd_slab_exchange(fdtd_handle* const* slabs, int n, int halo) {
  if (!slabs || n <= 0) return fail(FDTD_ERR_INVALID_ARGUMENT, "no slabs");
  if (halo != FDTD_HALO_E && halo != FDTD_HALO_B && halo != FDTD_HALO_STEP)
    return fail(FDTD_ERR_INVALID_ARGUMENT, "invalid halo");
  for (int s = 0; s < n; ++s)
    if (!slabs[s] || !slabs[s]->zhalo) return fail(FDTD_ERR_INVALID_ARGUMENT, "every handle must be a z slab");
  for (int s = 0; s < n; ++s) {
    const fdtd_handle* h = slabs[s];
    const fdtd_handle* h0 = slabs[0];
    if (h->form != h0->form || h->g.Ni != h0->g.Ni || h->g.Nj != h0->g.Nj || h->device != h0->device ||
        h->slab_nk_global != h0->slab_nk_global)
      return fail(FDTD_ERR_INVALID_ARGUMENT, "slabs must share the form, the x-y grid and the device");
    for (int c = 0; c < 6; ++c)
      if (h->fp16_exp[c] != h0->fp16_exp[c]) return fail(FDTD_ERR_INVALID_ARGUMENT, "slabs must share FP16 exponents");
    const int next = s + 1 < n ? slabs[s + 1]->slab_k0 : h0->slab_nk_global;
    if ((s == 0 && h->slab_k0 != 0) || h->slab_k0 + h->g.Nk != next)
      return fail(FDTD_ERR_INVALID_ARGUMENT, "slabs must tile the grid's planes in order");
  }
  DeviceGuard dg(slabs[0]->device);
  // E: slab s's first owned plane of Ex, Ey becomes the halo above of slab
  // s-1.  B: slab s's last owned plane of Bx, By becomes the halo below of
  // slab s+1; STEP sends Ex, Ey, Ez of that plane along with them.  The ring
  // closes periodically, as the reference's z wrap does.
  struct Group {
    int comps[5];
    int n_comps, from, to;
    bool up;  // sent to the slab above (else below)
  };
  Group groups[2];
  int n_groups = 0;
  if (halo != FDTD_HALO_B) groups[n_groups++] = {{FDTD_EX, FDTD_EY}, 2, FDTD_PLANE_FIRST, FDTD_PLANE_HALO_ABOVE, false};
  if (halo == FDTD_HALO_B) groups[n_groups++] = {{FDTD_BX, FDTD_BY}, 2, FDTD_PLANE_LAST, FDTD_PLANE_HALO_BELOW, true};
  if (halo == FDTD_HALO_STEP)
    groups[n_groups++] = {{FDTD_BX, FDTD_BY, FDTD_EX, FDTD_EY, FDTD_EZ}, 5, FDTD_PLANE_LAST, FDTD_PLANE_HALO_BELOW, true};
  const int parts = slabs[0]->form == Form::F32C ? 2 : 1;
  for (int s = 0; s < n; ++s) FDTD_CUDA(cudaEventRecord(slabs[s]->xev[0], slabs[s]->stream), "halo exchange");
  // Each slab receives on its own stream, after its sources' queued work.
  for (int d = 0; d < n; ++d) {
    fdtd_handle* dst = slabs[d];
    for (int g = 0; g < n_groups; ++g) {
      const Group& q = groups[g];
      fdtd_handle* src = slabs[q.up ? (d + n - 1) % n : (d + 1) % n];
      FDTD_CUDA(cudaStreamWaitEvent(dst->stream, src->xev[0], 0), "halo exchange");
      for (int i = 0; i < q.n_comps; ++i)
        for (int part = 0; part < parts; ++part) {
          size_t nb = 0, nb2 = 0;
          unsigned char* a = slab_plane(src, q.comps[i], q.from, part, &nb);
          unsigned char* b = slab_plane(dst, q.comps[i], q.to, part, &nb2);
          FDTD_CUDA(cudaMemcpyAsync(b, a, nb, cudaMemcpyDeviceToDevice, dst->stream), "halo exchange");
        }
    }
  }
  // A slab rewrites the planes it sent only after the copies have read them.
  for (int s = 0; s < n; ++s) FDTD_CUDA(cudaEventRecord(slabs[s]->xev[1], slabs[s]->stream), "halo exchange");
  for (int s = 0; s < n; ++s)
    for (int g = 0; g < n_groups; ++g)
      FDTD_CUDA(cudaStreamWaitEvent(slabs[s]->stream, slabs[groups[g].up ? (s + 1) % n : (s + n - 1) % n]->xev[1], 0),
                "halo exchange");
  return FDTD_OK;
}

}  // extern "C"
