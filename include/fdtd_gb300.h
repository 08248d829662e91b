/*
 * fdtd_gb300.h — C ABI of the GB300 (sm_103a) Yee FDTD engine.
 *
 * One handle = one periodic 3-D grid on one GPU, driven on one CUDA stream.
 * The entry points replace the public surface of the reference's Kokkos
 * solver class FDTD_kokkos::FDTD (Amazingkivas/FDTD_Method,
 * include/FDTD_kokkos/FDTD_kokkos.h:7-36); each declaration names the
 * reference interface it stands in for.  Plain pointers and sizes only.
 *
 * Every function returns FDTD_OK (0) or a negative FDTD_ERR_* code; the text
 * of the last error on the calling thread is fdtd_last_error().  A handle is
 * not thread-safe; distinct handles are independent.
 *
 * Field storage: component c lives in device memory as Ni*Nj*Nk values, flat
 * index i + j*Ni + k*Ni*Nj (x fastest), the layout of the reference's
 * Kokkos::View<double*, LayoutLeft> fields (include/FDTD_kokkos/kokkos_shared.h:16).
 */
#ifndef FDTD_GB300_H
#define FDTD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FDTD_ABI_VERSION 1

/* Status codes. */
#define FDTD_OK 0
#define FDTD_ERR_INVALID_ARGUMENT (-1) /* reference: std::invalid_argument */
#define FDTD_ERR_LOGIC (-2)            /* reference: std::logic_error     */
#define FDTD_ERR_CUDA (-3)             /* a CUDA call failed              */
#define FDTD_ERR_OUT_OF_MEMORY (-4)    /* device allocation failed        */
#define FDTD_ERR_UNSUPPORTED (-5)      /* not available for this storage  */
#define FDTD_ERR_TIMEOUT (-6)          /* a bounded device wait gave up   */

/* Field components, numbered as the reference's enum class Component
 * (include/Enums.h:5). */
enum fdtd_component {
    FDTD_EX = 0, FDTD_EY, FDTD_EZ,
    FDTD_BX, FDTD_BY, FDTD_BZ,
    FDTD_JX, FDTD_JY, FDTD_JZ
};

/* Storage / arithmetic forms of the field state.
 *   FP64        — the drop-in: FP64 storage and arithmetic, evaluated in the
 *                 reference's operation order with no fused multiply-add, so
 *                 results are bit-identical to the reference's.
 *   FP32        — FP32 storage and arithmetic.
 *   FP32_COMP   — compensated: each E/B value stored as an FP32 "hi" word plus
 *                 a BF16 "lo" word holding what FP32 rounds away (at least a
 *                 32-bit significand in 6 bytes), updated with error-free
 *                 FP32 transformations (TwoSum, FMA products).
 *   FP16_SCALED — FP16 storage with a power-of-two scale per component and
 *                 FP32 arithmetic. */
enum fdtd_precision {
    FDTD_PRECISION_FP64 = 0,
    FDTD_PRECISION_FP32 = 1,
    FDTD_PRECISION_FP32_COMP = 2,
    FDTD_PRECISION_FP16_SCALED = 3
};

/* Grid description; same members, order and meaning as the reference's
 * struct Parameters (include/Structures.h:23-38). */
typedef struct fdtd_params {
    int Ni, Nj, Nk;
    double ax, bx, ay, by, az, bz;
    double dx, dy, dz;
} fdtd_params;

/* A separable current source.  During time step s (s = number of completed
 * update_fields calls) it adds, for every component c with bit c of
 * comp_mask set (bit 0 = Jx, 1 = Jy, 2 = Jz),
 *     amp[s] * gx[di] * gy[dj] * gz[dk]        (product formed left to right)
 * to J at cell ((i0+di) mod Ni, (j0+dj) mod Nj, (k0+dk) mod Nk) for
 * 0 <= di < ni, 0 <= dj < nj, 0 <= dk < nk.  Steps s >= n_amp add nothing.
 * This is the form of the reference sample's box current
 * sin(2 pi t/T) cos^2(2 pi x/Tx) cos^2(2 pi y/Ty) cos^2(2 pi z/Tz)
 * (perf-tests/kokkos_sample/kokkos_sample.cpp:91-108) and of a Gaussian pulse
 * with a Gaussian spatial envelope.  The tables are copied at registration. */
typedef struct fdtd_source {
    int comp_mask;
    int i0, j0, k0;
    int ni, nj, nk;
    const double* gx;
    const double* gy;
    const double* gz;
    const double* amp;
    int64_t n_amp;
} fdtd_source;

/* Diagnostics vector filled by fdtd_field_sums (FP64 sums over all cells). */
enum fdtd_diag {
    FDTD_DIAG_EX2 = 0, FDTD_DIAG_EY2, FDTD_DIAG_EZ2,  /* sum of E_c^2            */
    FDTD_DIAG_BX2, FDTD_DIAG_BY2, FDTD_DIAG_BZ2,      /* sum of B_c^2            */
    FDTD_DIAG_SX, FDTD_DIAG_SY, FDTD_DIAG_SZ,         /* sum of (E x B)_c        */
    FDTD_DIAG_NONFINITE,                              /* count of NaN/Inf values */
    FDTD_DIAG_COUNT
};

typedef struct fdtd_handle fdtd_handle;

/* Text of the last error on this thread ("" if none). */
const char* fdtd_last_error(void);
int fdtd_abi_version(void);

/* Replaces FDTD::FDTD(Parameters, FP dt) (src/FDTD_kokkos/FDTD_kokkos.cpp:5-67):
 * validates (any N <= 0 or dt <= 0 -> FDTD_ERR_INVALID_ARGUMENT with the
 * reference's message "ERROR: invalid parameters"), allocates the nine
 * zero-filled fields on the current CUDA device and derives the reference's
 * coefficients.  `precision` is an fdtd_precision. */
int fdtd_create(const fdtd_params* params, double dt, int precision, fdtd_handle** out);

/* Replaces FDTD_PML::FDTD_PML(Parameters, FP dt, FP pml_percent)
 * (include/FDTD_kokkos/FDTD_PML_kokkos.h:10-33, src/FDTD_kokkos/FDTD_PML_kokkos.cpp:22-160):
 * a grid whose outer (int)(N * pml_percent) cells on each face of every axis
 * form a split-field absorbing layer (conductivity (d/pml)^4 profile,
 * reflection 1e-12).  update_fields / fdtd_step then follow
 * FDTD_PML::update_fields (:162-189): B/2 inside, the split-field B update on
 * the layer, E inside (with current), the split-field E update on the layer,
 * B/2 inside.  FP64 form only (other precisions give FDTD_ERR_UNSUPPORTED);
 * pml_percent must be in [0, 0.5).  The split fields and conductivities start
 * at zero (the reference leaves them unset).  All other entry points work as
 * for fdtd_create's handles; fdtd_destroy releases it. */
int fdtd_create_pml(const fdtd_params* params, double dt, double pml_percent, int precision, fdtd_handle** out);
/* Layer thickness per axis in cells (all zero for a handle without PML). */
int fdtd_get_pml(fdtd_handle* h, int sizes[3]);

/* Releases the fields (the reference's Views are freed with the object). */
int fdtd_destroy(fdtd_handle* h);

/* Replaces FDTD::update_fields() (src/FDTD_kokkos/FDTD_kokkos.cpp:91-104):
 * one full step B/2, E, B/2.  Asynchronous on the handle's stream.
 * In the FP32-arithmetic forms with the default fused pipeline a step is one
 * sweep (B half steps, then E): the trailing B/2 of the step is applied by
 * the next step's sweep, together with that step's leading B/2.  Every entry
 * point that reads B (copies, exports, field sums) sees it applied, and every
 * one that writes E or B applies it first, so a sequence of update_fields
 * calls, with or without reads in between, gives the bits of fdtd_step(n). */
int fdtd_update_fields(fdtd_handle* h);

/* n consecutive update_fields() calls, scheduled as one sequence (the two B
 * half steps that meet between steps share one sweep). */
int fdtd_step(fdtd_handle* h, int64_t n);

/* Replaces FDTD::zeroed_currents() (src/FDTD_kokkos/FDTD_kokkos.cpp:69-73). */
int fdtd_zeroed_currents(fdtd_handle* h);

/* Replaces FDTD::get_field(Component) (src/FDTD_kokkos/FDTD_kokkos.cpp:75-89)
 * for the FP64 form: the device address of the component's Ni*Nj*Nk doubles,
 * which aliases the engine's storage as the reference's View handle does.
 * Writing J through it switches the E update to read J.  An out-of-range
 * component gives FDTD_ERR_LOGIC ("ERROR: Invalid field component"); other
 * storage forms give FDTD_ERR_UNSUPPORTED (use fdtd_copy_field). */
int fdtd_get_field(fdtd_handle* h, int comp, double** device_ptr);

/* Host mirror + deep_copy of one component (the reference's
 * create_mirror_view / deep_copy, perf-tests/kokkos_sample/kokkos_sample.cpp:135-139),
 * converting to/from FP64 for every storage form.  n must be Ni*Nj*Nk.
 * Synchronous with respect to the host buffer. */
int fdtd_copy_field_to_host(fdtd_handle* h, int comp, double* host, size_t n);
int fdtd_copy_field_from_host(fdtd_handle* h, int comp, const double* host, size_t n);

/* New: FP64 values of the E/B component `comp` at the flat cells
 * offset .. offset+count-1 (any storage form), written into device memory at
 * device_dst.  Asynchronous on the handle's stream (device-side diagnostics
 * and comparisons; no host copy). */
int fdtd_export_field(fdtd_handle* h, int comp, int64_t offset, int64_t count, double* device_dst);

/* Registers a separable current source (see fdtd_source); returns its index
 * through *index if non-null.  Sources replace the reference sample driver's
 * per-step SetCurrent kernel (perf-tests/kokkos_sample/kokkos_sample.cpp:88-129). */
int fdtd_add_source(fdtd_handle* h, const fdtd_source* src, int* index);
int fdtd_clear_sources(fdtd_handle* h);

/* Number of completed update_fields steps (indexes source amplitude tables). */
int fdtd_get_step(fdtd_handle* h, int64_t* step);
int fdtd_set_step(fdtd_handle* h, int64_t step);

/* FP64 field sums (fdtd_diag order) over the whole grid; synchronous.  New:
 * the reference has no energy or Poynting diagnostics.  Energy
 * = (sum E^2 + sum B^2) dV / (8 pi); Poynting integral = c dV/(4 pi) sum E x B. */
int fdtd_field_sums(fdtd_handle* h, double out[FDTD_DIAG_COUNT]);

/* Grid and storage information. */
int fdtd_get_params(fdtd_handle* h, fdtd_params* params, double* dt, int* precision);

/* Stream control: the handle's work runs on `stream` (a cudaStream_t; 0 = the
 * handle's own stream).  fdtd_synchronize waits for it (Kokkos::fence()). */
int fdtd_set_stream(fdtd_handle* h, void* stream);
int fdtd_synchronize(fdtd_handle* h);

/* Arithmetic of the FP64 form (new).  BITWISE (the default) evaluates the
 * reference's expressions (kokkos_functors.h:64-90, :128-151) in its
 * operation order with no fused multiply-add: bit-identical to the
 * reference.  CONTRACTED accumulates each curl and current term into the
 * field with DFMA (24 FP64 instructions per cell-step against 39; the FP64
 * pipe bounds these sweeps on GB300): within a few ulps of the reference per
 * step.  Other storage forms give FDTD_ERR_UNSUPPORTED. */
enum fdtd_fp64_arith { FDTD_FP64_BITWISE = 0, FDTD_FP64_CONTRACTED = 1 };
int fdtd_set_fp64_arith(fdtd_handle* h, int arith);

/* Test hook of the bounded device waits (new).  The fused sweeps' waits on
 * their tile loads give up after `polls` polls (0: the default, 2^24) and
 * then stop the sweep: every CTA leaves its tile loop, waits (bounded) for
 * its copies in flight and exits; fdtd_synchronize then reports
 * FDTD_ERR_TIMEOUT and the step's results are invalid.  withhold_loads != 0
 * makes the sweeps issue no tile loads at all, so that every wait gives up
 * with no copy in flight: the way to exercise that path without a fault. */
int fdtd_set_wait_limit(fdtd_handle* h, int64_t polls, int withhold_loads);

/* Measured issue rate of the FP64 pipe of the current device (new; the
 * roofline of the FP64 sweeps): independent DMUL/DADD chains on every SM,
 * timed with CUDA events.  Synchronous; about 50 ms. */
int fdtd_measure_fp64_rate(double* dp_instr_per_s, double* ms);

/* Per-component power-of-two scales of the FP16_SCALED form: stored value =
 * field * 2^exponent.  `exponents` has 6 entries (Ex..Bz), each in [-60, 60]. */
int fdtd_set_fp16_exponents(fdtd_handle* h, const int exponents[6]);
int fdtd_get_fp16_exponents(fdtd_handle* h, int exponents[6]);
/* Exponents chosen by the engine (new).  From the stored peaks, each
 * component's field peak is below 2^k_c; with k_all the largest, the wanted
 * exponent puts the component's peak at 2^target_log2 but never more than
 * 2^headroom_log2 above the strongest component's scale:
 *     e_c = min(target_log2 - k_c, target_log2 + headroom_log2 - k_all)
 * (a component with no field gets the second term).  The bound keeps a weak
 * component that grows to the strongest one's size inside FP16's range
 * (target 10, headroom 5: peaks up to 2^15 before anything overflows, and
 * 64x of growth for the strongest); where components cannot exchange
 * magnitude, a large headroom gives each its own scale.
 * fdtd_fp16_autoscale sets the exponents now (target_log2 in [0, 15],
 * headroom_log2 in [0, 60]) and returns them in `exponents` if non-null.
 * fdtd_set_fp16_autoscale makes fdtd_step scan every `every_steps` steps
 * (0: never) and re-encode a component whose exponent is above the bound or
 * 3 or more from the wanted one; the scan interval must be short against the
 * fields' growth.  Re-encoding multiplies stored values by a power of two,
 * which commutes with the FP32 arithmetic on them: results change only where
 * a value would otherwise have left FP16's normal range.  Each scan
 * synchronises the handle's stream. */
int fdtd_fp16_autoscale(fdtd_handle* h, int target_log2, int headroom_log2, int exponents[6]);
int fdtd_set_fp16_autoscale(fdtd_handle* h, int every_steps, int target_log2, int headroom_log2);
/* The rule alone, on the host (no handle, no GPU): from the six stored peaks
 * (the largest |stored value| per component; 0, Inf or NaN counts as no
 * field) and the current exponents, the exponents a scan re-encodes to; a
 * component keeps its exponent unless `force`, its exponent is above the
 * bound, or the wanted one is 3 or more away.  No field anywhere: unchanged. */
int fdtd_fp16_choose_exponents(const float peaks[6], const int current[6], int target_log2, int headroom_log2,
                               int force, int exponents[6]);

/* Kernel timing (new; for roofline accounting).  While enabled, every kernel
 * launch of the step pipeline is bracketed by CUDA events on the handle's
 * stream.  fdtd_kernel_times synchronizes, then returns per kernel kind the
 * summed duration in milliseconds and the launch count since the last call,
 * and clears them.  Kinds: FDTD_KERNEL_E, _B_HALF, _B_DOUBLE, _FUSED,
 * _FUSED2. */
enum fdtd_kernel_kind {
    FDTD_KERNEL_E = 0,        /* E update sweep                            */
    FDTD_KERNEL_B_HALF = 1,   /* one B half step                           */
    FDTD_KERNEL_B_DOUBLE = 2, /* two B half steps sharing one sweep        */
    FDTD_KERNEL_FUSED = 3,    /* a whole step (B/2, E, B/2) in one sweep   */
    FDTD_KERNEL_FUSED2 = 4,   /* two whole steps in one sweep (depth 2)    */
    FDTD_KERNEL_KINDS = 5
};
int fdtd_set_kernel_timing(fdtd_handle* h, int enabled);

/* Step pipeline of the FP32-arithmetic forms (new; tuning and testing).
 * AUTO and FUSED: one sweep per step (E step + double B half step); SPLIT:
 * one sweep per half step.  All give bit-identical results.  The fused
 * launch is shaped by tile_y (interior rows of a tile: 6, 14 or 30; 0 = 14;
 * 30 only with cells_per_thread 1),
 * kchunk (planes per tile; 0 = 48) and cells_per_thread (1: 32-wide tiles,
 * 2: 64-wide tiles with packed two-cell arithmetic; 0 = 1).  The FP64 form
 * always uses the split sweeps. */
enum fdtd_pipeline { FDTD_PIPELINE_AUTO = 0, FDTD_PIPELINE_SPLIT = 1, FDTD_PIPELINE_FUSED = 2 };
int fdtd_set_pipeline(fdtd_handle* h, int pipeline, int tile_y, int kchunk, int cells_per_thread);
int fdtd_kernel_times(fdtd_handle* h, double ms[FDTD_KERNEL_KINDS], int64_t launches[FDTD_KERNEL_KINDS]);

/* Autotuner (new).  Times `sweeps` fused sweeps (0 = 10) for every candidate
 * launch shape of the FP32-arithmetic forms (cells_per_thread 1 with tile_y
 * 6, 14 and 30; cells_per_thread 2 with tile_y 6 and 14; each with kchunk 16,
 * 24, 32, 48, 64 and 96; and the depth-2 sweep with tile_y 6 and 14 and
 * kchunk 24, 48 and 96, compared per step; a two-cell shape, whose E-first
 * pipeline starts every call with a B half sweep, is charged that sweep per
 * step, as update_fields once per step costs it) on the handle's own grid,
 * and keeps the fastest
 * (fdtd_set_pipeline's shape arguments).  The timed sweeps read the current
 * state and write the handle's second copy, so the simulation state does not
 * change.  Results are cached per (precision, Ni, Nj, Nk) in the process;
 * reuse != 0 takes a cached result without timing.  Synchronous.  The FP64
 * form gives FDTD_ERR_UNSUPPORTED. */
typedef struct fdtd_tune_result {
    int tile_y, kchunk, cells_per_thread;
    double ms_per_sweep;  /* of the chosen shape, per step (a depth-2 sweep's time halved) */
    int candidates;       /* shapes timed */
    int cached;           /* 1 if taken from the cache */
    int split_sources;    /* batched sweep: 1 if the chosen sweep runs the split plane loop */
    int depth;            /* steps per sweep of the chosen shape: 1 or 2 */
} fdtd_tune_result;
int fdtd_autotune(fdtd_handle* h, int sweeps, int reuse, fdtd_tune_result* out);

/* Temporal blocking (new).  depth 2: fdtd_step runs two steps per pass over
 * the state (a depth-2 sweep reads E and B once and writes them once for both
 * steps; an odd last step is a one-step sweep); depth 1: one step per sweep.
 * Both give the same bits.  Depth 2 needs the FP32-arithmetic forms, the
 * fused pipeline with one cell per thread, and tile_y 6 or 14; the
 * autotuner also tries it (its result's depth field).  Batches and z slabs
 * step one step per sweep. */
int fdtd_set_temporal_depth(fdtd_handle* h, int depth);

/* ------------------------------------------------------------------------
 * Batched form (new; the reference advances one grid per object).  A batch
 * holds n independent periodic domains of any sizes on one GPU, stored in an
 * FP32-arithmetic form (FP32, FP32_COMP or FP16_SCALED), all with the same
 * dt.  fdtd_batch_step(b, n) advances every domain by n update_fields steps:
 * each B-first fused sweep of all domains is one persistent kernel launch
 * that works through a per-domain tile table, and the whole step group runs
 * as one CUDA graph (captured on first use for each step count, then
 * replayed).  As on a single handle, the last step's trailing B half step is
 * applied by the next group's first sweep; domain reads see it applied and
 * domain writes apply it first (to every domain).  Each domain's results are
 * bit-identical to a single-domain handle of the same form run alone with
 * the same step calls.  Domains take analytic sources only (no dense J arrays).
 * Not thread-safe per batch. */
typedef struct fdtd_batch fdtd_batch;

/* params[0..n-1] describe the domains (as fdtd_create; same validation). */
int fdtd_batch_create(const fdtd_params* params, int n, double dt, int precision, fdtd_batch** out);
int fdtd_batch_destroy(fdtd_batch* b);
int fdtd_batch_size(fdtd_batch* b, int* n);
int fdtd_batch_domain_params(fdtd_batch* b, int domain, fdtd_params* params);
/* Domain-wise versions of fdtd_add_source, fdtd_copy_field_to_host/from_host
 * (E and B components only), fdtd_field_sums and fdtd_set_fp16_exponents. */
int fdtd_batch_add_source(fdtd_batch* b, int domain, const fdtd_source* src, int* index);
int fdtd_batch_copy_field_to_host(fdtd_batch* b, int domain, int comp, double* host, size_t n);
int fdtd_batch_copy_field_from_host(fdtd_batch* b, int domain, int comp, const double* host, size_t n);
int fdtd_batch_field_sums(fdtd_batch* b, int domain, double out[FDTD_DIAG_COUNT]);
int fdtd_batch_set_fp16_exponents(fdtd_batch* b, int domain, const int exponents[6]);
/* Tile shape of the fused sweep (tile_y 6, 14 or 30; kchunk planes per tile;
 * 0 = defaults 14 and 24) and whether step groups run as CUDA graphs. */
int fdtd_batch_set_config(fdtd_batch* b, int tile_y, int kchunk, int use_graphs);
/* n steps of every domain; asynchronous on the batch's stream. */
int fdtd_batch_step(fdtd_batch* b, int64_t n);
int fdtd_batch_get_step(fdtd_batch* b, int64_t* step);
/* Number of fused-sweep tiles of the batch at its current tile shape. */
int fdtd_batch_tiles(fdtd_batch* b, int64_t* tiles);
int fdtd_batch_set_stream(fdtd_batch* b, void* stream);
/* Autotuner of the batch: times `sweeps` (0 = 5) persistent fused sweeps of
 * every domain for tile_y 6, 14 and 30 with kchunk 16, 24, 32, 48 and 64,
 * each with the plane loop compiled once or split (below), and keeps the
 * fastest; the state does not change.  Synchronous. */
int fdtd_batch_autotune(fdtd_batch* b, int sweeps, fdtd_tune_result* out);
/* Split plane loop (on != 0): the sweep carries a source-free copy of its
 * plane loop for tiles no source reaches.  Faster where most tiles have no
 * source; slower where tiles of both kinds alternate.  Same results. */
int fdtd_batch_set_split_sources(fdtd_batch* b, int on);
int fdtd_batch_synchronize(fdtd_batch* b);

/* No counterpart in the reference.  The ten field sums of fdtd_field_sums,
 * for callers that cannot allocate device memory (an application whose pool
 * allocator owns every device allocation, a monitor that must not call
 * cudaMalloc beside a running simulation): no handle, no allocation.  Inputs:
 * six FP64 device arrays Ex..Bz of `cells` values (dense drop-in layout);
 * output: 10 doubles at out_device (fdtd_diag order), written on `stream`
 * (a cudaStream_t, 0 = default stream).  Scratch is a fixed device array of
 * 65536 block partials built into the library (5 MiB per device that loads
 * it, held until exit), which caps `cells` at 268,435,456; larger grids give
 * FDTD_ERR_INVALID_ARGUMENT.  The first call on a device resolves that array's
 * device address (make it before any stream capture); later calls resolve it
 * again unless their stream is capturing, so a reset device context is
 * followed.  Calls share the array: calls that overlap on the GPU race. */
int fdtd_field_sums_noalloc(const double* const fields[6], int64_t cells, double* out_device, void* stream);

/* ------------------------------------------------------------------------
 * Compact forms of the entry points above. */
/* Field energy in Gaussian units, from fdtd_field_sums: out[0] electric
 * (sum E^2) dV/(8 pi), out[1] magnetic (sum B^2) dV/(8 pi), out[2] their sum,
 * dV = dx dy dz.  Synchronous. */
int fdtd_energy(fdtd_handle* h, double out[3]);
/* Replaces the handle's source list by src[0..n-1] (fdtd_clear_sources, then
 * fdtd_add_source for each).  On an error the previous list stays. */
int fdtd_set_sources(fdtd_handle* h, const fdtd_source* src, int n);
/* fdtd_get_field as an untyped device pointer (FP64 form). */
int fdtd_field_device_ptr(fdtd_handle* h, int comp, void** device_ptr);
/* fdtd_copy_field_to_host (dir FDTD_TO_HOST) or _from_host (FDTD_FROM_HOST)
 * of all Ni*Nj*Nk values. */
enum fdtd_direction { FDTD_TO_HOST = 0, FDTD_FROM_HOST = 1 };
int fdtd_copy_field(fdtd_handle* h, int comp, double* host, int dir);
/* fdtd_synchronize. */
int fdtd_sync(fdtd_handle* h);

/* ------------------------------------------------------------------------
 * z slabs: the domain decomposition of the reference's coarray program
 * (coarray/fdtd.F90:90-98, 149-164).  A slab handle owns planes
 * [k_begin, k_end) of the grid `params` plus one halo plane below and one
 * above.  Every host-facing call (fdtd_copy_field_*, fdtd_get_field,
 * fdtd_export_field, fdtd_field_sums, fdtd_get_params) sees the owned planes
 * only: a grid of Ni x Nj x (k_end - k_begin), az/bz moved to the slab.
 * fdtd_add_source takes boxes in the coordinates of the whole grid and
 * keeps the part in the owned planes.
 *
 * A set of slabs that tile the planes in order (k_begin of the first 0, each
 * k_end the next k_begin, the last k_end Nk) steps like one handle of the
 * whole grid when every slab runs, per call of n update_fields steps,
 *     exchange E, B_HALF (B_DOUBLE if the previous call left a half step
 *     pending), then per step: exchange B, E, exchange E, B_DOUBLE between
 *     steps and after the last one B_DEFER (FP32-arithmetic forms; B_HALF in
 *     the FP64 form):
 * the results are the whole-grid handle's bit for bit, in every precision.
 * In the FP32-arithmetic forms a call may instead run the fused schedule,
 *     exchange STEP, then per step: STEP, exchange STEP
 * (one fused sweep and one exchange per step; the trailing B half stays
 * pending as above, and the exchange after each sweep keeps the halo planes
 * current for readers that apply it).  Both schedules give the whole-grid
 * handle's bits and may alternate between calls.
 * fdtd_step on a slab gives FDTD_ERR_UNSUPPORTED; slabs take no autotuner
 * (the fused sweep uses the handle's launch shape: fdtd_set_pipeline with one
 * cell per thread) and have no PML.
 *
 * One GPU: fdtd_slab_exchange copies the boundary planes between the slabs
 * of one device.  Several GPUs: each rank exchanges the planes that
 * fdtd_slab_plane addresses with its neighbours (NCCL send / receive), in
 * the same order. */
int fdtd_slab_create(const fdtd_params* params, double dt, int precision, int k_begin, int k_end,
                     fdtd_handle** out);
/* Owned planes and the whole grid's plane count (an ordinary handle: 0, Nk, Nk). */
int fdtd_slab_info(fdtd_handle* h, int* k_begin, int* k_end, int* nk_global);

enum fdtd_sweep {
    FDTD_SWEEP_B_HALF = 0,   /* B += curl term (kokkos_functors.h:128-151), once  */
    FDTD_SWEEP_B_DOUBLE = 1, /* the same term added twice (two half steps)        */
    FDTD_SWEEP_E = 2,        /* E update of the current step; the step count + 1  */
    FDTD_SWEEP_B_DEFER = 3,  /* no sweep: the step's trailing B half is left
                                pending (FP32-arithmetic forms), as fdtd_step
                                leaves it; the next B_DOUBLE sweep applies it
                                with the next step's leading half, readers of
                                B see it applied, writers apply it first      */
    FDTD_SWEEP_STEP = 4      /* a whole update_fields step as one fused
                                B-first sweep (FP32-arithmetic forms): the
                                pending B half, if any, and the step's leading
                                half, then E; the trailing half is left
                                pending (as B_DEFER); the step count + 1.
                                Reads Bx, By, Ex, Ey, Ez of the halo below and
                                Ex, Ey of the halo above: run FDTD_HALO_STEP
                                before it                                     */
};
/* One sweep over the owned planes (any non-PML handle: the whole grid).  With
 * a B half step pending, B_HALF applies it and B_DOUBLE applies it and one
 * more; E applies it first. */
int fdtd_slab_sweep(fdtd_handle* h, int sweep);

enum fdtd_plane {
    FDTD_PLANE_HALO_BELOW = 0, FDTD_PLANE_FIRST = 1, FDTD_PLANE_LAST = 2, FDTD_PLANE_HALO_ABOVE = 3
};
enum fdtd_halo {
    FDTD_HALO_E = 0,    /* Ex, Ey of each slab's first plane -> the halo above of the slab below */
    FDTD_HALO_B = 1,    /* Bx, By of each slab's last plane  -> the halo below of the slab above */
    FDTD_HALO_STEP = 2  /* what FDTD_SWEEP_STEP reads: HALO_E, and Bx, By, Ex, Ey, Ez of each
                           slab's last plane -> the halo below of the slab above */
};
/* Device address and size in bytes of one stored plane of component comp
 * (FDTD_EX..FDTD_BZ) in the handle's storage form: part 0 the E/B words,
 * part 1 the compensation words (FP32_COMP).  The FP32-arithmetic forms store
 * padded planes; a plane is copied whole. */
int fdtd_slab_plane(fdtd_handle* h, int comp, int plane, int part, void** device_ptr, size_t* bytes);
/* Halo exchange between the n slabs of one device, listed in plane order
 * (the last one's neighbour above is the first: the grid is periodic).
 * Asynchronous: ordered after each slab's queued work and before its next. */
int fdtd_slab_exchange(fdtd_handle* const* slabs, int n, int halo);

#ifdef __cplusplus
}
#endif

#endif /* FDTD_GB300_H */
