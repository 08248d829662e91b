// FP64 Yee kernels — the drop-in form.
//
// Each update is evaluated in the reference's operation order with explicit
// round-to-nearest intrinsics (__dadd_rn / __dsub_rn / __dmul_rn), which the
// compiler never fuses into FMA.  Results are therefore bit-identical to the
// reference's (kokkos_functors.h:64-90 and :128-151 built without FMA
// contraction, which is what its stock x86-64 build does).
//
// On GB300 the FP64 pipe issues ~5e11 instructions/s in total, 1/64 of the
// FP32 rate, so these kernels are bound by FP64 issue, not by HBM: a B half
// step costs 18 FP64 instructions per cell, a merged double half step 21 and
// the E step 18 (24 with current).  The kernels keep every other cost off the
// FP64 pipe: one thread per (i, j) column marching along z with the z
// neighbour carried in registers, all index arithmetic in 32-bit integers
// plus one 64-bit plane offset per z step.
//
// Contracted variant (kFma, fdtd_set_fp64_arith): the same sweeps with each
// curl term accumulated by DFMA into the field, B += (apps cB) d1 - (apps cB) d2
// as two DFMAs after the two differences (apps cB is exact: apps is 1 or 2),
// E likewise, with cJ J as one more DFMA.  A B double half step then costs 12
// FP64 instructions per cell and E 12 (15 with current), against 21 and 18:
// the results are no longer the reference's bit for bit but stay within a
// few ulps per step (the drop-in contract is 1e-12 of the field amplitude).
#include "engine_internal.h"

namespace fdtd {

#define DADD __dadd_rn
#define DSUB __dsub_rn
#define DMUL __dmul_rn

// B += t (once: a half step; twice: the second half step of one update_fields
// followed by the first half step of the next, which see the same E and
// therefore the same t — the two additions stay separate, so the result is
// the reference's bit for bit).  kernels: kokkos_functors.h:128-151.
template <int kApplications, bool kFma>
__global__ void __launch_bounds__(256) b_update_fp64(Grid g, Box b, const double* __restrict__ Ex,
                                                     const double* __restrict__ Ey,
                                                     const double* __restrict__ Ez,
                                                     double* __restrict__ Bx, double* __restrict__ By,
                                                     double* __restrict__ Bz, double cx, double cy,
                                                     double cz, int kchunk) {
  const int i = b.i0 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.j0 + blockIdx.y * blockDim.y + threadIdx.y;
  const int k0 = b.k0 + blockIdx.z * kchunk;
  if (i >= b.i1 || j >= b.j1 || k0 >= b.k1) return;
  const int k1 = min(k0 + kchunk, b.k1);
  const int64_t col = i + (int64_t)j * g.Ni;
  const int64_t col_in = wrap_next(i, g.Ni) + (int64_t)j * g.Ni;
  const int64_t col_jn = i + (int64_t)wrap_next(j, g.Nj) * g.Ni;

  int64_t base = (int64_t)k0 * g.plane;
  double ex = Ex[col + base];
  double ey = Ey[col + base];
  for (int k = k0; k < k1; ++k) {
    const int64_t nbase = (int64_t)wrap_next(k, g.Nk) * g.plane;
    const double ex_kn = Ex[col + nbase];
    const double ey_kn = Ey[col + nbase];
    const double ez = Ez[col + base];
    const double ez_jn = Ez[col_jn + base];
    const double ez_in = Ez[col_in + base];
    const double ey_in = Ey[col_in + base];
    const double ex_jn = Ex[col_jn + base];

    if (kFma) {
      // c' = apps * c (exact); B + c' d1 - c' d2 as two DFMAs
      const double ax = kApplications * cx, ay = kApplications * cy, az = kApplications * cz;
      Bx[col + base] = __fma_rn(az, DSUB(ey_kn, ey), __fma_rn(-ay, DSUB(ez_jn, ez), Bx[col + base]));
      By[col + base] = __fma_rn(ax, DSUB(ez_in, ez), __fma_rn(-az, DSUB(ex_kn, ex), By[col + base]));
      Bz[col + base] = __fma_rn(ay, DSUB(ex_jn, ex), __fma_rn(-ax, DSUB(ey_in, ey), Bz[col + base]));
      ex = ex_kn;
      ey = ey_kn;
      base = nbase;
      continue;
    }
    const double tx = DSUB(DMUL(cz, DSUB(ey_kn, ey)), DMUL(cy, DSUB(ez_jn, ez)));
    const double ty = DSUB(DMUL(cx, DSUB(ez_in, ez)), DMUL(cz, DSUB(ex_kn, ex)));
    const double tz = DSUB(DMUL(cy, DSUB(ex_jn, ex)), DMUL(cx, DSUB(ey_in, ey)));

    double bx = DADD(Bx[col + base], tx);
    double by = DADD(By[col + base], ty);
    double bz = DADD(Bz[col + base], tz);
    if (kApplications == 2) {
      bx = DADD(bx, tx);
      by = DADD(by, ty);
      bz = DADD(bz, tz);
    }
    Bx[col + base] = bx;
    By[col + base] = by;
    Bz[col + base] = bz;

    ex = ex_kn;
    ey = ey_kn;
    base = nbase;
  }
}

// E += cJ*J + c*curl(B), kokkos_functors.h:64-90.  Cells with no current skip
// the cJ*J term: cJ < 0, so cJ*0 = -0 and x + (-0) = x for every x, which
// leaves the result bit-identical.
template <bool kDenseJ, bool kSources, bool kFma>
__global__ void __launch_bounds__(256) e_update_fp64(Grid g, Box b, const double* __restrict__ Bx,
                                                     const double* __restrict__ By,
                                                     const double* __restrict__ Bz,
                                                     const double* __restrict__ Jx,
                                                     const double* __restrict__ Jy,
                                                     const double* __restrict__ Jz,
                                                     double* __restrict__ Ex, double* __restrict__ Ey,
                                                     double* __restrict__ Ez, double cJ, double cx,
                                                     double cy, double cz, int kchunk, SourceSet ss,
                                                     int64_t s) {
  const int i = b.i0 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.j0 + blockIdx.y * blockDim.y + threadIdx.y;
  const int k0 = b.k0 + blockIdx.z * kchunk;
  if (i >= b.i1 || j >= b.j1 || k0 >= b.k1) return;
  const int k1 = min(k0 + kchunk, b.k1);
  const int64_t col = i + (int64_t)j * g.Ni;
  const int64_t col_ip = wrap_prev(i, g.Ni) + (int64_t)j * g.Ni;
  const int64_t col_jp = i + (int64_t)wrap_prev(j, g.Nj) * g.Ni;

  int64_t base = (int64_t)k0 * g.plane;
  const int64_t pbase0 = (int64_t)wrap_prev(k0, g.Nk) * g.plane;
  double bx_kp = Bx[col + pbase0];
  double by_kp = By[col + pbase0];
  for (int k = k0; k < k1; ++k) {
    const double bx = Bx[col + base];
    const double by = By[col + base];
    const double bz = Bz[col + base];
    const double bz_jp = Bz[col_jp + base];
    const double bz_ip = Bz[col_ip + base];
    const double by_ip = By[col_ip + base];
    const double bx_jp = Bx[col_jp + base];

    if (kFma) {
      // E + cJ J + c1 d1 - c2 d2 as DFMAs into E
      bool has_j = false;
      double jx = 0.0, jy = 0.0, jz = 0.0;
      if (kDenseJ) {
        jx = Jx[col + base];
        jy = Jy[col + base];
        jz = Jz[col + base];
        has_j = true;
      }
      if (kSources) has_j |= source_current(ss, s, i, j, k, g, jx, jy, jz);
      double ex = Ex[col + base], ey = Ey[col + base], ez = Ez[col + base];
      if (has_j) {
        ex = __fma_rn(cJ, jx, ex);
        ey = __fma_rn(cJ, jy, ey);
        ez = __fma_rn(cJ, jz, ez);
      }
      Ex[col + base] = __fma_rn(cy, DSUB(bz, bz_jp), __fma_rn(-cz, DSUB(by, by_kp), ex));
      Ey[col + base] = __fma_rn(cz, DSUB(bx, bx_kp), __fma_rn(-cx, DSUB(bz, bz_ip), ey));
      Ez[col + base] = __fma_rn(cx, DSUB(by, by_ip), __fma_rn(-cy, DSUB(bx, bx_jp), ez));
      bx_kp = bx;
      by_kp = by;
      base += g.plane;
      continue;
    }
    double tx = DSUB(DMUL(cy, DSUB(bz, bz_jp)), DMUL(cz, DSUB(by, by_kp)));
    double ty = DSUB(DMUL(cz, DSUB(bx, bx_kp)), DMUL(cx, DSUB(bz, bz_ip)));
    double tz = DSUB(DMUL(cx, DSUB(by, by_ip)), DMUL(cy, DSUB(bx, bx_jp)));

    bool has_j = false;
    double jx = 0.0, jy = 0.0, jz = 0.0;
    if (kDenseJ) {
      jx = Jx[col + base];
      jy = Jy[col + base];
      jz = Jz[col + base];
      has_j = true;
    }
    if (kSources) has_j |= source_current(ss, s, i, j, k, g, jx, jy, jz);
    if (has_j) {
      // (cJ*J + c1*d1) - c2*d2, the reference's association.
      tx = DSUB(DADD(DMUL(cJ, jx), DMUL(cy, DSUB(bz, bz_jp))), DMUL(cz, DSUB(by, by_kp)));
      ty = DSUB(DADD(DMUL(cJ, jy), DMUL(cz, DSUB(bx, bx_kp))), DMUL(cx, DSUB(bz, bz_ip)));
      tz = DSUB(DADD(DMUL(cJ, jz), DMUL(cx, DSUB(by, by_ip))), DMUL(cy, DSUB(bx, bx_jp)));
    }
    Ex[col + base] = DADD(Ex[col + base], tx);
    Ey[col + base] = DADD(Ey[col + base], ty);
    Ez[col + base] = DADD(Ez[col + base], tz);

    bx_kp = bx;
    by_kp = by;
    base += g.plane;
  }
}

// ---------------------------------------------------------------------------
// Host-side launchers (called from engine.cu).

static dim3 fp64_grid(const Box& b, int kchunk) {
  return dim3((b.i1 - b.i0 + 31) / 32, (b.j1 - b.j0 + 7) / 8, (b.k1 - b.k0 + kchunk - 1) / kchunk);
}

cudaError_t launch_b_fp64(const Grid& g, const Box& box, const Fp64Fields& F, const double cb[3],
                          int applications, bool fma, cudaStream_t st) {
  if (box.empty()) return cudaSuccess;
  const int kchunk = 16;
  dim3 block(32, 8), grid = fp64_grid(box, kchunk);
#define FDTD_B64(APPS, FMA)                                                                              \
  b_update_fp64<APPS, FMA><<<grid, block, 0, st>>>(g, box, F.f[0], F.f[1], F.f[2], F.f[3], F.f[4], F.f[5], \
                                                   cb[0], cb[1], cb[2], kchunk)
  if (applications == 2) {
    if (fma) FDTD_B64(2, true);
    else FDTD_B64(2, false);
  } else {
    if (fma) FDTD_B64(1, true);
    else FDTD_B64(1, false);
  }
#undef FDTD_B64
  return cudaGetLastError();
}

template <bool FMA>
static void launch_e_fp64_arith(dim3 grid, dim3 block, const Grid& g, const Box& box, const Fp64Fields& F,
                                const double ce[3], double cJ, bool dense_j, const SourceSet& ss, int64_t step,
                                int kchunk, cudaStream_t st) {
  const bool src = ss.count > 0;
#define FDTD_E64(DJ, SRC)                                                                          \
  e_update_fp64<DJ, SRC, FMA><<<grid, block, 0, st>>>(g, box, F.f[3], F.f[4], F.f[5], F.f[6], F.f[7], \
                                                      F.f[8], F.f[0], F.f[1], F.f[2], cJ, ce[0],   \
                                                      ce[1], ce[2], kchunk, ss, step)
  if (dense_j && src) FDTD_E64(true, true);
  else if (dense_j) FDTD_E64(true, false);
  else if (src) FDTD_E64(false, true);
  else FDTD_E64(false, false);
#undef FDTD_E64
}

cudaError_t launch_e_fp64(const Grid& g, const Box& box, const Fp64Fields& F, const double ce[3], double cJ,
                          bool dense_j, const SourceSet& ss, int64_t step, bool fma, cudaStream_t st) {
  if (box.empty()) return cudaSuccess;
  const int kchunk = 16;
  dim3 block(32, 8), grid = fp64_grid(box, kchunk);
  if (fma) launch_e_fp64_arith<true>(grid, block, g, box, F, ce, cJ, dense_j, ss, step, kchunk, st);
  else launch_e_fp64_arith<false>(grid, block, g, box, F, ce, cJ, dense_j, ss, step, kchunk, st);
  return cudaGetLastError();
}

}  // namespace fdtd
