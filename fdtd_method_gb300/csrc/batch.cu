// Batched form of the engine: many independent periodic domains of uneven
// sizes advanced together.  Each domain is an ordinary handle (storage,
// sources, host copies and diagnostics are the single-domain code's); the
// batch adds device tables that describe every domain to one persistent
// fused-step kernel, and runs a step group as one CUDA graph:
//
//   n B-first sweeps of every domain         (n persistent launches over the
//                                             tile table, kernels_fused1.cu)
//   step counter += n                        (one thread)
//
// As for a single handle, the last step's trailing B half is left pending
// and the next group's first sweep applies it with its own leading half;
// readers of a domain see it applied (the domain handle's read path), and
// before anything writes a domain's E or B the batch applies it to every
// domain in one launch (kernels_f32.cu b_sweep_batch), so all domains stay
// at the same point of the step.
//
// The per-domain tile table lists (domain, bx, by, bz) for every tile of every
// domain, domain by domain; the persistent CTAs take tiles from it in order.
// A graph is captured once per (step count, parity) and replayed; the source
// step index is read from device memory, so a replay needs no new arguments.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "handle.h"

using namespace fdtd;

namespace {

int bfail(int code, const std::string& msg) {
  set_last_error(msg);
  return code;
}
int bcuda(cudaError_t e, const char* what) {
  return bfail(e == cudaErrorMemoryAllocation ? FDTD_ERR_OUT_OF_MEMORY : FDTD_ERR_CUDA,
               std::string(what) + ": " + cudaGetErrorString(e));
}

#define FDTD_BCUDA(call, what)                 \
  do {                                         \
    cudaError_t e_ = (call);                   \
    if (e_ != cudaSuccess) return bcuda(e_, what); \
  } while (0)

__global__ void advance_step(int64_t* step, int64_t n) { *step += n; }

}  // namespace

struct fdtd_batch {
  std::vector<fdtd_handle*> doms;
  int precision = 0;
  Form form = Form::F32C;
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  FusedConfig cfg;
  bool use_graphs = true;
  int parity = 0;     // which copy of the tables' two is current
  int64_t step = 0;   // completed steps
  bool dirty = true;  // device tables out of date
  bool pending = false;  // every domain's trailing B half step is pending
  // device tables
  void* d_doms = nullptr;        // BatchDomain<S>[n]
  StepMaps* d_maps = nullptr;    // [2 n]
  int4* d_tiles = nullptr;
  int n_tiles = 0;
  int64_t* d_bstart = nullptr;   // [n + 1]
  int64_t n_bblocks = 0;
  int* d_counters = nullptr;     // 2 ints, zero between launches
  int64_t* d_step = nullptr;
  int* d_err = nullptr;
  std::map<std::tuple<int64_t, int, int>, cudaGraphExec_t> graphs;  // (steps, parity, first sweep's apps)
};

namespace {

void drop_graphs(fdtd_batch* b) {
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.second);
  b->graphs.clear();
}

void free_tables(fdtd_batch* b) {
  drop_graphs(b);
  cudaFree(b->d_doms);
  cudaFree(b->d_maps);
  cudaFree(b->d_tiles);
  cudaFree(b->d_bstart);
  b->d_doms = nullptr;
  b->d_maps = nullptr;
  b->d_tiles = nullptr;
  b->d_bstart = nullptr;
}

template <class S>
S store_of(const StateView& v);
template <>
StoreF32 store_of<StoreF32>(const StateView& v) { return v.s32; }
template <>
StoreF32C store_of<StoreF32C>(const StateView& v) { return v.s32c; }
template <>
StoreF16 store_of<StoreF16>(const StateView& v) { return v.s16; }

template <class S>
int upload_domains(fdtd_batch* b) {
  std::vector<BatchDomain<S>> recs(b->doms.size());
  for (size_t d = 0; d < b->doms.size(); ++d) {
    fdtd_handle* h = b->doms[d];
    BatchDomain<S>& r = recs[d];
    r.L = h->L;
    r.s[0] = store_of<S>(h->view());
    r.s[1] = store_of<S>(h->view_alt());
    r.cs = h->cs;
    r.ss = h->source_set();
  }
  FDTD_BCUDA(cudaMalloc(&b->d_doms, sizeof(BatchDomain<S>) * recs.size()), "batch domain table");
  FDTD_BCUDA(cudaMemcpy(b->d_doms, recs.data(), sizeof(BatchDomain<S>) * recs.size(), cudaMemcpyHostToDevice),
             "upload batch domain table");
  return FDTD_OK;
}

// Rebuilds every device table from the domains' current state: copy 0 of
// each domain is its current copy.
int build_tables(fdtd_batch* b) {
  free_tables(b);
  const int n = (int)b->doms.size();
  std::vector<StepMaps> maps(2 * n);
  std::vector<int4> tiles;
  std::vector<int64_t> bstart(n + 1, 0);
  for (int d = 0; d < n; ++d) {
    fdtd_handle* h = b->doms[d];
    h->fused_cfg = b->cfg;
    if (int rc = ensure_alt(h)) return rc;
    maps[2 * d].ld = h->bmaps_cur;
    maps[2 * d].st = h->smaps_alt;
    maps[2 * d + 1].ld = h->bmaps_alt;
    maps[2 * d + 1].st = h->smaps_cur;
    const int tx = (h->g.Ni + 31) / 32, ty = (h->g.Nj + b->cfg.tile_y - 1) / b->cfg.tile_y;
    const int tz = (h->g.Nk + b->cfg.kchunk - 1) / b->cfg.kchunk;
    for (int z = 0; z < tz; ++z)
      for (int y = 0; y < ty; ++y)
        for (int x = 0; x < tx; ++x) tiles.push_back(make_int4(d, x, y, z));
    const int64_t nb = (int64_t)((h->g.Ni + 31) / 32) * ((h->g.Nj + 7) / 8) *
                       ((h->g.Nk + kBatchBChunk - 1) / kBatchBChunk);
    bstart[d + 1] = bstart[d] + nb;
  }
  if (tiles.size() > 0x7fffffff) return bfail(FDTD_ERR_INVALID_ARGUMENT, "batch has too many tiles");
  int rc = FDTD_OK;
  switch (b->form) {
    case Form::F32: rc = upload_domains<StoreF32>(b); break;
    case Form::F32C: rc = upload_domains<StoreF32C>(b); break;
    case Form::F16: rc = upload_domains<StoreF16>(b); break;
    default: rc = bfail(FDTD_ERR_UNSUPPORTED, "batched form needs an FP32-arithmetic precision");
  }
  if (rc) return rc;
  FDTD_BCUDA(cudaMalloc(&b->d_maps, sizeof(StepMaps) * maps.size()), "batch tensor maps");
  FDTD_BCUDA(cudaMemcpy(b->d_maps, maps.data(), sizeof(StepMaps) * maps.size(), cudaMemcpyHostToDevice),
             "upload batch tensor maps");
  FDTD_BCUDA(cudaMalloc(&b->d_tiles, sizeof(int4) * tiles.size()), "batch tile table");
  FDTD_BCUDA(cudaMemcpy(b->d_tiles, tiles.data(), sizeof(int4) * tiles.size(), cudaMemcpyHostToDevice),
             "upload batch tile table");
  FDTD_BCUDA(cudaMalloc(&b->d_bstart, sizeof(int64_t) * bstart.size()), "batch block table");
  FDTD_BCUDA(cudaMemcpy(b->d_bstart, bstart.data(), sizeof(int64_t) * bstart.size(), cudaMemcpyHostToDevice),
             "upload batch block table");
  FDTD_BCUDA(cudaMemcpy(b->d_step, &b->step, sizeof(int64_t), cudaMemcpyHostToDevice), "batch step counter");
  b->n_tiles = (int)tiles.size();
  b->n_bblocks = bstart[n];
  b->parity = 0;
  b->dirty = false;
  return FDTD_OK;
}

cudaError_t launch_fused_all(fdtd_batch* b, int parity, int apps, int step_off) {
  const WaitCtl wc{b->d_err, kMaxBarrierPolls, 0};
  switch (b->form) {
    case Form::F32:
      return launch_fused1_batch<StoreF32>(b->d_doms, b->d_maps, b->d_tiles, b->n_tiles, parity, apps, b->cfg,
                                           b->d_step, step_off, b->d_counters, wc, b->stream);
    case Form::F32C:
      return launch_fused1_batch<StoreF32C>(b->d_doms, b->d_maps, b->d_tiles, b->n_tiles, parity, apps, b->cfg,
                                            b->d_step, step_off, b->d_counters, wc, b->stream);
    case Form::F16:
      return launch_fused1_batch<StoreF16>(b->d_doms, b->d_maps, b->d_tiles, b->n_tiles, parity, apps, b->cfg,
                                           b->d_step, step_off, b->d_counters, wc, b->stream);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_b_all(fdtd_batch* b, int parity) {
  const int n = (int)b->doms.size();
  switch (b->form) {
    case Form::F32: return launch_b_f32_batch<StoreF32>(b->d_doms, b->d_bstart, n, b->n_bblocks, parity, b->stream);
    case Form::F32C: return launch_b_f32_batch<StoreF32C>(b->d_doms, b->d_bstart, n, b->n_bblocks, parity, b->stream);
    case Form::F16: return launch_b_f32_batch<StoreF16>(b->d_doms, b->d_bstart, n, b->n_bblocks, parity, b->stream);
    default: return cudaErrorInvalidValue;
  }
}

// The launches of `n` steps from copy `parity`; the first sweep applies
// `first_apps` B half steps (2: the pending one and its own leading one).
cudaError_t enqueue_steps(fdtd_batch* b, int64_t n, int parity, int first_apps) {
  cudaError_t e = cudaSuccess;
  for (int64_t s = 0; s < n && e == cudaSuccess; ++s)
    e = launch_fused_all(b, parity ^ (int)(s & 1), s == 0 ? first_apps : 2, (int)s);
  if (e == cudaSuccess) {
    advance_step<<<1, 1, 0, b->stream>>>(b->d_step, n);
    e = cudaGetLastError();
  }
  return e;
}

// Applies the pending B half step of every domain (one launch) before
// anything writes a domain's E or B.
int resolve_batch(fdtd_batch* b) {
  if (!b->pending) return FDTD_OK;
  if (b->dirty)
    if (int rc = build_tables(b)) return rc;
  FDTD_BCUDA(launch_b_all(b, b->parity), "pending B half step of the batch");
  b->pending = false;
  for (fdtd_handle* h : b->doms) {
    h->b_pending = false;
    h->b_side = false;
  }
  return FDTD_OK;
}

int check_batch(fdtd_batch* b) {
  if (!b) return bfail(FDTD_ERR_INVALID_ARGUMENT, "null batch");
  return FDTD_OK;
}

int check_domain(fdtd_batch* b, int d) {
  if (int rc = check_batch(b)) return rc;
  if (d < 0 || d >= (int)b->doms.size()) return bfail(FDTD_ERR_INVALID_ARGUMENT, "domain index out of range");
  return FDTD_OK;
}

}  // namespace

extern "C" {

int fdtd_batch_create(const fdtd_params* params, int n, double dt, int precision, fdtd_batch** out) {
  if (!params || !out) return bfail(FDTD_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (n <= 0) return bfail(FDTD_ERR_INVALID_ARGUMENT, "a batch needs at least one domain");
  if (precision != FDTD_PRECISION_FP32 && precision != FDTD_PRECISION_FP32_COMP &&
      precision != FDTD_PRECISION_FP16_SCALED)
    return bfail(FDTD_ERR_UNSUPPORTED, "the batched form runs FP32, FP32_COMP or FP16_SCALED");
  fdtd_batch* b = new fdtd_batch();
  b->precision = precision;
  b->form = (Form)precision;
  cudaGetDevice(&b->device);
  cudaError_t e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete b;
    return bcuda(e, "batch stream");
  }
  b->stream = b->own_stream;
  int rc = FDTD_OK;
  for (int d = 0; d < n && rc == FDTD_OK; ++d) {
    fdtd_handle* h = nullptr;
    rc = fdtd_create(&params[d], dt, precision, &h);
    if (rc == FDTD_OK) {
      b->doms.push_back(h);
      rc = fdtd_set_stream(h, b->stream);
    }
  }
  if (rc == FDTD_OK) {
    e = cudaMalloc(&b->d_counters, 2 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(b->d_counters, 0, 2 * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_step, sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(b->d_err, 0, sizeof(int));
    if (e != cudaSuccess) rc = bcuda(e, "batch set-up");
  }
  if (rc != FDTD_OK) {
    std::string msg = fdtd_last_error();
    fdtd_batch_destroy(b);
    return bfail(rc, msg);
  }
  *out = b;
  return FDTD_OK;
}

int fdtd_batch_destroy(fdtd_batch* b) {
  if (!b) return FDTD_OK;
  DeviceGuard dg(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  free_tables(b);
  for (fdtd_handle* h : b->doms) fdtd_destroy(h);
  cudaFree(b->d_counters);
  cudaFree(b->d_step);
  cudaFree(b->d_err);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
  return FDTD_OK;
}

int fdtd_batch_size(fdtd_batch* b, int* n) {
  if (int rc = check_batch(b)) return rc;
  if (!n) return bfail(FDTD_ERR_INVALID_ARGUMENT, "null output pointer");
  *n = (int)b->doms.size();
  return FDTD_OK;
}

int fdtd_batch_domain_params(fdtd_batch* b, int d, fdtd_params* params) {
  if (int rc = check_domain(b, d)) return rc;
  if (!params) return bfail(FDTD_ERR_INVALID_ARGUMENT, "null output pointer");
  *params = b->doms[d]->p;
  return FDTD_OK;
}

int fdtd_batch_copy_field_to_host(fdtd_batch* b, int d, int comp, double* host, size_t n) {
  if (int rc = check_domain(b, d)) return rc;
  if (comp < FDTD_EX || comp > FDTD_BZ)
    return bfail(FDTD_ERR_LOGIC, "ERROR: Invalid field component");
  DeviceGuard dg(b->device);
  return fdtd_copy_field_to_host(b->doms[d], comp, host, n);
}

int fdtd_batch_copy_field_from_host(fdtd_batch* b, int d, int comp, const double* host, size_t n) {
  if (int rc = check_domain(b, d)) return rc;
  if (comp < FDTD_EX || comp > FDTD_BZ)
    return bfail(FDTD_ERR_LOGIC, "ERROR: Invalid field component");
  DeviceGuard dg(b->device);
  if (int rc = resolve_batch(b)) return rc;
  return fdtd_copy_field_from_host(b->doms[d], comp, host, n);
}

int fdtd_batch_field_sums(fdtd_batch* b, int d, double out[FDTD_DIAG_COUNT]) {
  if (int rc = check_domain(b, d)) return rc;
  DeviceGuard dg(b->device);
  return fdtd_field_sums(b->doms[d], out);
}

int fdtd_batch_set_fp16_exponents(fdtd_batch* b, int d, const int exponents[6]) {
  if (int rc = check_domain(b, d)) return rc;
  {
    DeviceGuard dg(b->device);
    if (int rc = resolve_batch(b)) return rc;
  }
  const int rc = fdtd_set_fp16_exponents(b->doms[d], exponents);
  if (rc == FDTD_OK) b->dirty = true;
  return rc;
}

int fdtd_batch_add_source(fdtd_batch* b, int d, const fdtd_source* src, int* index) {
  if (int rc = check_domain(b, d)) return rc;
  DeviceGuard dg(b->device);
  const int rc = fdtd_add_source(b->doms[d], src, index);
  if (rc == FDTD_OK) b->dirty = true;
  return rc;
}

int fdtd_batch_set_config(fdtd_batch* b, int tile_y, int kchunk, int use_graphs) {
  if (int rc = check_batch(b)) return rc;
  if (tile_y != 0 && tile_y != 6 && tile_y != 14 && tile_y != 30)
    return bfail(FDTD_ERR_INVALID_ARGUMENT, "tile_y must be 0 (default), 6, 14 or 30");
  if (kchunk < 0) return bfail(FDTD_ERR_INVALID_ARGUMENT, "kchunk must be >= 0");
  b->cfg.tile_y = tile_y ? tile_y : 14;
  b->cfg.kchunk = kchunk ? kchunk : 48;
  b->cfg.cells_per_thread = 1;
  b->use_graphs = use_graphs != 0;
  b->dirty = true;
  return FDTD_OK;
}

int fdtd_batch_step(fdtd_batch* b, int64_t n) {
  if (int rc = check_batch(b)) return rc;
  if (n < 0) return bfail(FDTD_ERR_INVALID_ARGUMENT, "negative step count");
  if (n == 0) return FDTD_OK;
  if (n > 0x7fffffff) return bfail(FDTD_ERR_INVALID_ARGUMENT, "step count too large for one call");
  DeviceGuard dg(b->device);
  if (b->dirty)
    if (int rc = build_tables(b)) return rc;
  const int first_apps = b->pending ? 2 : 1;
  if (b->use_graphs) {
    const auto key = std::make_tuple(n, b->parity, first_apps);
    auto it = b->graphs.find(key);
    if (it == b->graphs.end()) {
      cudaGraph_t g = nullptr;
      cudaGraphExec_t ge = nullptr;
      FDTD_BCUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed), "graph capture");
      cudaError_t e = enqueue_steps(b, n, b->parity, first_apps);
      cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
      if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bcuda(e, "batch step capture");
      }
      if (e2 != cudaSuccess) return bcuda(e2, "graph capture");
      e = cudaGraphInstantiate(&ge, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return bcuda(e, "graph instantiation");
      it = b->graphs.emplace(key, ge).first;
    }
    FDTD_BCUDA(cudaGraphLaunch(it->second, b->stream), "batch step graph launch");
  } else {
    FDTD_BCUDA(enqueue_steps(b, n, b->parity, first_apps), "batch step launch");
  }
  if (n & 1) {
    b->parity ^= 1;
    for (fdtd_handle* h : b->doms) swap_copies(h);
  }
  b->step += n;
  b->pending = true;
  for (fdtd_handle* h : b->doms) {
    h->host_step = b->step;
    h->b_pending = true;
    h->b_side = false;
  }
  return FDTD_OK;
}

int fdtd_batch_autotune(fdtd_batch* b, int sweeps, fdtd_tune_result* out) {
  if (int rc = check_batch(b)) return rc;
  if (sweeps <= 0) sweeps = 5;
  DeviceGuard dg(b->device);
  // The timed sweeps read copy `parity` and write the other copy: the state
  // is left as it was.  Tables are rebuilt per candidate (copy 0 = current).
  static const int rows[] = {6, 14, 30};
  static const int chunks[] = {16, 24, 32, 48, 64};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  FDTD_BCUDA(cudaEventCreate(&e0), "autotune events");
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return bfail(FDTD_ERR_CUDA, "autotune events");
  }
  fdtd_tune_result best{};
  best.ms_per_sweep = 1e30;
  best.cells_per_thread = 1;
  const bool graphs = b->use_graphs;
  int rc = FDTD_OK;
  for (int ty : rows) {
    for (int kc : chunks) {
      b->cfg.tile_y = ty;
      b->cfg.kchunk = kc;
      b->cfg.cells_per_thread = 1;
      if ((rc = build_tables(b)) != FDTD_OK) break;
      for (int split = 0; split < 2 && rc == FDTD_OK; ++split) {
        b->cfg.split_sources = split != 0;
        cudaError_t e = launch_fused_all(b, 0, 2, 0);  // warm-up
        if (e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
        for (int q = 0; q < sweeps && e == cudaSuccess; ++q) e = launch_fused_all(b, 0, 2, 0);
        if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess) {
          rc = bcuda(e, "batch autotune sweep");
          break;
        }
        best.candidates += 1;
        if (ms / sweeps < best.ms_per_sweep) {
          best.ms_per_sweep = ms / sweeps;
          best.tile_y = ty;
          best.kchunk = kc;
          best.split_sources = split;
        }
      }
    }
    if (rc != FDTD_OK) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (fdtd_handle* h : b->doms) h->b_side = false;  // the timed sweeps wrote the second copies
  if (rc != FDTD_OK) return rc;
  b->cfg.tile_y = best.tile_y;
  b->cfg.kchunk = best.kchunk;
  b->cfg.split_sources = best.split_sources != 0;
  b->use_graphs = graphs;
  b->dirty = true;
  if (out) *out = best;
  return FDTD_OK;
}

int fdtd_batch_set_split_sources(fdtd_batch* b, int on) {
  if (int rc = check_batch(b)) return rc;
  b->cfg.split_sources = on != 0;
  b->dirty = true;
  return FDTD_OK;
}

int fdtd_batch_synchronize(fdtd_batch* b) {
  if (int rc = check_batch(b)) return rc;
  DeviceGuard dg(b->device);
  FDTD_BCUDA(cudaStreamSynchronize(b->stream), "batch synchronize");
  int err = 0;
  FDTD_BCUDA(cudaMemcpy(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost), "batch status");
  if (err) {
    cudaMemset(b->d_err, 0, sizeof(int));
    return bfail(FDTD_ERR_TIMEOUT, "a bounded device wait of the batched step gave up");
  }
  return FDTD_OK;
}

int fdtd_batch_set_stream(fdtd_batch* b, void* stream) {
  if (int rc = check_batch(b)) return rc;
  DeviceGuard dg(b->device);
  FDTD_BCUDA(cudaStreamSynchronize(b->stream), "batch stream switch");
  b->stream = stream ? static_cast<cudaStream_t>(stream) : b->own_stream;
  for (fdtd_handle* h : b->doms)
    if (int rc = fdtd_set_stream(h, b->stream)) return rc;
  drop_graphs(b);
  return FDTD_OK;
}

int fdtd_batch_get_step(fdtd_batch* b, int64_t* step) {
  if (int rc = check_batch(b)) return rc;
  if (!step) return bfail(FDTD_ERR_INVALID_ARGUMENT, "null output pointer");
  *step = b->step;
  return FDTD_OK;
}

int fdtd_batch_tiles(fdtd_batch* b, int64_t* tiles) {
  if (int rc = check_batch(b)) return rc;
  if (!tiles) return bfail(FDTD_ERR_INVALID_ARGUMENT, "null output pointer");
  DeviceGuard dg(b->device);
  if (b->dirty)
    if (int rc = build_tables(b)) return rc;
  *tiles = b->n_tiles;
  return FDTD_OK;
}

}  // extern "C"
