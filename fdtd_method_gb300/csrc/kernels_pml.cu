// FP64 split-field PML kernels: the absorbing layer of the reference's
// FDTD_PML class (src/FDTD_kokkos/FDTD_PML_kokkos.cpp, functors
// include/FDTD_kokkos/kokkos_functors.h:247-309 for E and :343-405 for B).
//
// In the layer each field component is the sum of two split parts, each
// decaying with the conductivity along one axis and driven by the curl term
// along that axis:
//   Eyx <- Eyx a_x - b_x (Bz - Bz[i-1]),  Ezx <- Ezx a_x + b_x (By - By[i-1]),
//   Exy <- Exy a_y + b_y (Bz - Bz[j-1]),  Ezy <- Ezy a_y - b_y (Bx - Bx[j-1]),
//   Exz <- Exz a_z - b_z (By - By[k-1]),  Eyz <- Eyz a_z + b_z (Bx - Bx[k-1]),
//   Ex = Exz + Exy,  Ey = Eyx + Eyz,  Ez = Ezy + Ezx
// (B likewise with forward differences), where a = exp(-sigma c dt) and
// b = (1 - a) / (sigma d), or c dt / d where sigma = 0.  The conductivity of
// an axis depends only on the coordinate along it, so a and b come from
// per-axis tables computed on the host exactly as the reference computes them
// per cell (its exp and pow run on the host too).  Arithmetic uses the
// reference's operation order with round-to-nearest intrinsics (no FMA), so
// the results are the reference's bit for bit.
#include "engine_internal.h"

namespace fdtd {

#define DADD __dadd_rn
#define DSUB __dsub_rn
#define DMUL __dmul_rn

__global__ void __launch_bounds__(256) e_pml_fp64(Grid g, Box b, Fp64Fields F, PmlFields P, int kchunk) {
  const int i = b.i0 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.j0 + blockIdx.y * blockDim.y + threadIdx.y;
  const int k0 = b.k0 + blockIdx.z * kchunk;
  if (i >= b.i1 || j >= b.j1 || k0 >= b.k1) return;
  const int k1 = min(k0 + kchunk, b.k1);
  const double* __restrict__ Bx = F.f[3];
  const double* __restrict__ By = F.f[4];
  const double* __restrict__ Bz = F.f[5];
  double *Exy = P.split[0], *Exz = P.split[1], *Eyx = P.split[2], *Eyz = P.split[3], *Ezx = P.split[4],
         *Ezy = P.split[5];
  const int64_t col = i + (int64_t)j * g.Ni;
  const int64_t col_ip = wrap_prev(i, g.Ni) + (int64_t)j * g.Ni;
  const int64_t col_jp = i + (int64_t)wrap_prev(j, g.Nj) * g.Ni;
  const double ax = P.decay[0][i], bxc = P.coef2[0][i];
  const double ay = P.decay[1][j], byc = P.coef2[1][j];
  for (int k = k0; k < k1; ++k) {
    const int64_t base = (int64_t)k * g.plane, pbase = (int64_t)wrap_prev(k, g.Nk) * g.plane;
    const int64_t n = col + base;
    const double az = P.decay[2][k], bzc = P.coef2[2][k];
    const double bx = Bx[n], by = By[n], bz = Bz[n];
    const double eyx = DSUB(DMUL(Eyx[n], ax), DMUL(bxc, DSUB(bz, Bz[col_ip + base])));
    const double ezx = DADD(DMUL(Ezx[n], ax), DMUL(bxc, DSUB(by, By[col_ip + base])));
    const double exy = DADD(DMUL(Exy[n], ay), DMUL(byc, DSUB(bz, Bz[col_jp + base])));
    const double ezy = DSUB(DMUL(Ezy[n], ay), DMUL(byc, DSUB(bx, Bx[col_jp + base])));
    const double exz = DSUB(DMUL(Exz[n], az), DMUL(bzc, DSUB(by, By[col + pbase])));
    const double eyz = DADD(DMUL(Eyz[n], az), DMUL(bzc, DSUB(bx, Bx[col + pbase])));
    Eyx[n] = eyx;
    Ezx[n] = ezx;
    Exy[n] = exy;
    Ezy[n] = ezy;
    Exz[n] = exz;
    Eyz[n] = eyz;
    F.f[0][n] = DADD(exz, exy);
    F.f[1][n] = DADD(eyx, eyz);
    F.f[2][n] = DADD(ezy, ezx);
  }
}

__global__ void __launch_bounds__(256) b_pml_fp64(Grid g, Box b, Fp64Fields F, PmlFields P, int kchunk) {
  const int i = b.i0 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.j0 + blockIdx.y * blockDim.y + threadIdx.y;
  const int k0 = b.k0 + blockIdx.z * kchunk;
  if (i >= b.i1 || j >= b.j1 || k0 >= b.k1) return;
  const int k1 = min(k0 + kchunk, b.k1);
  const double* __restrict__ Ex = F.f[0];
  const double* __restrict__ Ey = F.f[1];
  const double* __restrict__ Ez = F.f[2];
  double *Bxy = P.split[6], *Bxz = P.split[7], *Byx = P.split[8], *Byz = P.split[9], *Bzx = P.split[10],
         *Bzy = P.split[11];
  const int64_t col = i + (int64_t)j * g.Ni;
  const int64_t col_in = wrap_next(i, g.Ni) + (int64_t)j * g.Ni;
  const int64_t col_jn = i + (int64_t)wrap_next(j, g.Nj) * g.Ni;
  const double ax = P.decay[0][i], bxc = P.coef2[0][i];
  const double ay = P.decay[1][j], byc = P.coef2[1][j];
  for (int k = k0; k < k1; ++k) {
    const int64_t base = (int64_t)k * g.plane, nbase = (int64_t)wrap_next(k, g.Nk) * g.plane;
    const int64_t n = col + base;
    const double az = P.decay[2][k], bzc = P.coef2[2][k];
    const double ex = Ex[n], ey = Ey[n], ez = Ez[n];
    const double byx = DADD(DMUL(Byx[n], ax), DMUL(bxc, DSUB(Ez[col_in + base], ez)));
    const double bzx = DSUB(DMUL(Bzx[n], ax), DMUL(bxc, DSUB(Ey[col_in + base], ey)));
    const double bxy = DSUB(DMUL(Bxy[n], ay), DMUL(byc, DSUB(Ez[col_jn + base], ez)));
    const double bzy = DADD(DMUL(Bzy[n], ay), DMUL(byc, DSUB(Ex[col_jn + base], ex)));
    const double bxz = DADD(DMUL(Bxz[n], az), DMUL(bzc, DSUB(Ey[col + nbase], ey)));
    const double byz = DSUB(DMUL(Byz[n], az), DMUL(bzc, DSUB(Ex[col + nbase], ex)));
    Byx[n] = byx;
    Bzx[n] = bzx;
    Bxy[n] = bxy;
    Bzy[n] = bzy;
    Bxz[n] = bxz;
    Byz[n] = byz;
    F.f[3][n] = DADD(bxy, bxz);
    F.f[4][n] = DADD(byz, byx);
    F.f[5][n] = DADD(bzx, bzy);
  }
}

static dim3 pml_grid(const Box& b, int kchunk) {
  return dim3((b.i1 - b.i0 + 31) / 32, (b.j1 - b.j0 + 7) / 8, (b.k1 - b.k0 + kchunk - 1) / kchunk);
}

cudaError_t launch_e_pml_fp64(const Grid& g, const Box& box, const Fp64Fields& F, const PmlFields& P,
                              cudaStream_t st) {
  if (box.empty()) return cudaSuccess;
  const int kchunk = 16;
  e_pml_fp64<<<pml_grid(box, kchunk), dim3(32, 8), 0, st>>>(g, box, F, P, kchunk);
  return cudaGetLastError();
}

cudaError_t launch_b_pml_fp64(const Grid& g, const Box& box, const Fp64Fields& F, const PmlFields& P,
                              cudaStream_t st) {
  if (box.empty()) return cudaSuccess;
  const int kchunk = 16;
  b_pml_fp64<<<pml_grid(box, kchunk), dim3(32, 8), 0, st>>>(g, box, F, P, kchunk);
  return cudaGetLastError();
}

}  // namespace fdtd
