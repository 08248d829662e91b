/*
 * ORACLE — CPU restatement of the reference's Yee FDTD step.
 *
 * Test infrastructure only.  The parity tests, the engine's smoke check and
 * the CPU-baseline leg of the benchmark call this code as the checker; the
 * engine never links it and never falls back to it.
 *
 * Parity is pinned: the tests compare every function below against the
 * reference's own Kokkos-path sources compiled unmodified against the host
 * Kokkos stand-in (oracle/_ref, built by oracle/Makefile) and against the
 * golden numbers recorded from that build under tests/golden/.
 *
 * What it restates (file:line in Amazingkivas/FDTD_Method):
 *   periodic wrap             include/FDTD_kokkos/kokkos_functors.h:13-20
 *   E update (UpdateEField)   include/FDTD_kokkos/kokkos_functors.h:64-90
 *   B update (UpdateBField)   include/FDTD_kokkos/kokkos_functors.h:128-151
 *   coefficients              src/FDTD_kokkos/FDTD_kokkos.cpp:45-55
 *   parameter validation      src/FDTD_kokkos/FDTD_kokkos.cpp:7-12
 *   update_fields = B/2,E,B/2 src/FDTD_kokkos/FDTD_kokkos.cpp:91-104
 *   current box source        perf-tests/kokkos_sample/kokkos_sample.cpp:88-129
 *   OpenMP solver twin        src/FDTD/FDTD.cpp:63-157 (timed CPU path only)
 *   PML (split-field layer)   src/FDTD_kokkos/FDTD_PML_kokkos.cpp:22-189,
 *                             include/FDTD_kokkos/kokkos_functors.h:154-415
 *
 * Arithmetic is written in the reference's evaluation order and must be built
 * with -ffp-contract=off so that no multiply-add is fused (the reference's
 * stock x86-64 build has no FMA either); the results are then bit-identical
 * to the reference's on every host.  The loops are the reference's three
 * full-grid sweeps per step, parallelised over k with OpenMP, so the same code
 * also serves as the timed CPU port of the reference.
 *
 * Field order everywhere: EX, EY, EZ, BX, BY, BZ, JX, JY, JZ
 * (include/Enums.h:5); flat index i + j*Ni + k*Ni*Nj, x fastest.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Speed of light and pi exactly as the reference defines them
 * (include/Constants.h:6,11); the truncated pi is deliberate. */
#define ORACLE_C 3e10
#define ORACLE_PI 3.14159265358

typedef struct {
    int Ni, Nj, Nk;
    double ax, bx, ay, by, az, bz;
    double dx, dy, dz;
} oracle_params; /* include/Structures.h:23-38 */

/* One separable current source:
 *   J_c(i,j,k, step) += amp[step] * gx[(i-i0) mod Ni] * gy[...] * gz[...]
 * for every component c in comp_mask (bit 0 = Jx, 1 = Jy, 2 = Jz) and every
 * cell of the (periodically wrapped) box of extent ni x nj x nk at (i0,j0,k0).
 * The product is formed left to right, as the reference's sample driver forms
 * sin(t) * cos^2(x) * cos^2(y) * cos^2(z) (kokkos_sample.cpp:100-103).  Steps
 * at or past n_amp contribute nothing. */
typedef struct {
    int comp_mask;
    int i0, j0, k0;
    int ni, nj, nk;
    const double* gx;
    const double* gy;
    const double* gz;
    const double* amp;
    long n_amp;
} oracle_source;

int oracle_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* src/FDTD_kokkos/FDTD_kokkos.cpp:7-12 and :45-55.  coef = {cEx, cEy, cEz,
 * cBx, cBy, cBz, cJ}.  Returns -1 (the reference throws invalid_argument) for
 * a non-positive size or time step. */
int oracle_coefficients(const oracle_params* p, double dt, double coef[7]) {
    if (p->Ni <= 0 || p->Nj <= 0 || p->Nk <= 0 || dt <= 0) return -1;
    const double cdt = ORACLE_C * dt;
    coef[0] = cdt / p->dx;
    coef[1] = cdt / p->dy;
    coef[2] = cdt / p->dz;
    coef[3] = cdt / (2.0 * p->dx);
    coef[4] = cdt / (2.0 * p->dy);
    coef[5] = cdt / (2.0 * p->dz);
    coef[6] = -4.0 * ORACLE_PI * dt;
    return 0;
}

/* include/FDTD_kokkos/kokkos_functors.h:13-20: -1 -> N-1, N -> 0, others unchanged. */
static inline long wrap(long i, long N) {
    const long minus_one = (i < 0);
    const long at_n = (i == N);
    return (N - 1) * minus_one + i * !(minus_one || at_n);
}

/* A box of cells [i0,i1) x [j0,j1) x [k0,k1): the ranges the reference's
 * functors take (kokkos_functors.h:45-63 and :109-127). */
typedef struct { long i0, i1, j0, j1, k0, k1; } oracle_box;

/* include/FDTD_kokkos/kokkos_functors.h:128-151 over a box. */
void oracle_update_B_box(long Ni, long Nj, long Nk, oracle_box b,
                         const double* Ex, const double* Ey, const double* Ez,
                         double* Bx, double* By, double* Bz,
                         double cx, double cy, double cz) {
    const long plane = Ni * Nj;
#pragma omp parallel for schedule(static)
    for (long k = b.k0; k < b.k1; ++k) {
        const long kn = wrap(k + 1, Nk);
        for (long j = b.j0; j < b.j1; ++j) {
            const long jn = wrap(j + 1, Nj);
            for (long i = b.i0; i < b.i1; ++i) {
                const long in = wrap(i + 1, Ni);
                const long idx = i + j * Ni + k * plane;
                const long i_n = in + j * Ni + k * plane;
                const long j_n = i + jn * Ni + k * plane;
                const long k_n = i + j * Ni + kn * plane;
                Bx[idx] += cz * (Ey[k_n] - Ey[idx]) - cy * (Ez[j_n] - Ez[idx]);
                By[idx] += cx * (Ez[i_n] - Ez[idx]) - cz * (Ex[k_n] - Ex[idx]);
                Bz[idx] += cy * (Ex[j_n] - Ex[idx]) - cx * (Ey[i_n] - Ey[idx]);
            }
        }
    }
}

/* The same over the whole grid. */
void oracle_update_B(long Ni, long Nj, long Nk,
                     const double* Ex, const double* Ey, const double* Ez,
                     double* Bx, double* By, double* Bz,
                     double cx, double cy, double cz) {
    const oracle_box all = {0, Ni, 0, Nj, 0, Nk};
    oracle_update_B_box(Ni, Nj, Nk, all, Ex, Ey, Ez, Bx, By, Bz, cx, cy, cz);
}

/* include/FDTD_kokkos/kokkos_functors.h:64-90 over a box.  A null J pointer
 * set means J == 0 (the term cJ*0 = -0 leaves every sum unchanged). */
void oracle_update_E_box(long Ni, long Nj, long Nk, oracle_box b,
                         const double* Bx, const double* By, const double* Bz,
                         const double* Jx, const double* Jy, const double* Jz,
                         double* Ex, double* Ey, double* Ez,
                         double cJ, double cx, double cy, double cz) {
    const long plane = Ni * Nj;
#pragma omp parallel for schedule(static)
    for (long k = b.k0; k < b.k1; ++k) {
        const long kp = wrap(k - 1, Nk);
        for (long j = b.j0; j < b.j1; ++j) {
            const long jp = wrap(j - 1, Nj);
            for (long i = b.i0; i < b.i1; ++i) {
                const long ip = wrap(i - 1, Ni);
                const long idx = i + j * Ni + k * plane;
                const long i_p = ip + j * Ni + k * plane;
                const long j_p = i + jp * Ni + k * plane;
                const long k_p = i + j * Ni + kp * plane;
                const double jx = Jx ? Jx[idx] : 0.0;
                const double jy = Jy ? Jy[idx] : 0.0;
                const double jz = Jz ? Jz[idx] : 0.0;
                Ex[idx] += cJ * jx + cy * (Bz[idx] - Bz[j_p]) - cz * (By[idx] - By[k_p]);
                Ey[idx] += cJ * jy + cz * (Bx[idx] - Bx[k_p]) - cx * (Bz[idx] - Bz[i_p]);
                Ez[idx] += cJ * jz + cx * (By[idx] - By[i_p]) - cy * (Bx[idx] - Bx[j_p]);
            }
        }
    }
}

/* The same over the whole grid. */
void oracle_update_E(long Ni, long Nj, long Nk,
                     const double* Bx, const double* By, const double* Bz,
                     const double* Jx, const double* Jy, const double* Jz,
                     double* Ex, double* Ey, double* Ez,
                     double cJ, double cx, double cy, double cz) {
    const oracle_box all = {0, Ni, 0, Nj, 0, Nk};
    oracle_update_E_box(Ni, Nj, Nk, all, Bx, By, Bz, Jx, Jy, Jz, Ex, Ey, Ez, cJ, cx, cy, cz);
}

/* Adds every active source's contribution for time step `step` into the three
 * J arrays (perf-tests/kokkos_sample/kokkos_sample.cpp:91-108 writes the same
 * product into a box of Jx, Jy, Jz before each update_fields). */
void oracle_add_sources(long Ni, long Nj, long Nk, double* J[3],
                        const oracle_source* src, int nsrc, long step) {
    for (int s = 0; s < nsrc; ++s) {
        const oracle_source* q = &src[s];
        if (step < 0 || step >= q->n_amp) continue;
        const double a = q->amp[step];
#pragma omp parallel for schedule(static)
        for (long dk = 0; dk < q->nk; ++dk) {
            const long k = (q->k0 + dk) % Nk;
            for (long dj = 0; dj < q->nj; ++dj) {
                const long j = (q->j0 + dj) % Nj;
                for (long di = 0; di < q->ni; ++di) {
                    const long i = (q->i0 + di) % Ni;
                    const long idx = i + j * Ni + k * Ni * Nj;
                    const double v = a * q->gx[di] * q->gy[dj] * q->gz[dk];
                    for (int c = 0; c < 3; ++c)
                        if (q->comp_mask & (1 << c)) J[c][idx] = J[c][idx] + v;
                }
            }
        }
    }
}

/* src/FDTD_kokkos/FDTD_kokkos.cpp:91-104 repeated `steps` times.
 * f = the nine arrays in component order; f[6..8] may be null (J == 0).
 * With sources, step s (counted from step0) uses J_eff = J + sum of sources,
 * formed in jwork[3] (three scratch arrays of Ni*Nj*Nk doubles). */
void oracle_run(long Ni, long Nj, long Nk, double* f[9], const double coef[7],
                const oracle_source* src, int nsrc, long step0, int steps,
                double* jwork[3]) {
    const long n = Ni * Nj * Nk;
    for (int s = 0; s < steps; ++s) {
        const double* J[3] = {f[6], f[7], f[8]};
        if (nsrc > 0) {
            for (int c = 0; c < 3; ++c) {
                if (f[6 + c]) memcpy(jwork[c], f[6 + c], sizeof(double) * n);
                else memset(jwork[c], 0, sizeof(double) * n);
            }
            oracle_add_sources(Ni, Nj, Nk, jwork, src, nsrc, step0 + s);
            J[0] = jwork[0];
            J[1] = jwork[1];
            J[2] = jwork[2];
        }
        oracle_update_B(Ni, Nj, Nk, f[0], f[1], f[2], f[3], f[4], f[5], coef[3], coef[4], coef[5]);
        oracle_update_E(Ni, Nj, Nk, f[3], f[4], f[5], J[0], J[1], J[2], f[0], f[1], f[2],
                        coef[6], coef[0], coef[1], coef[2]);
        oracle_update_B(Ni, Nj, Nk, f[0], f[1], f[2], f[3], f[4], f[5], coef[3], coef[4], coef[5]);
    }
}

/* The reference sample driver's loop (perf-tests/kokkos_sample/kokkos_sample.cpp:88-113):
 * before each update_fields, write the sources' values into their boxes of
 * the dense J arrays f[6..8] (which must exist and be zero outside the
 * boxes), then run the three sweeps.  Same results as oracle_run with zero
 * dense J, at the reference driver's cost; used as the timed CPU baseline. */
void oracle_run_driver(long Ni, long Nj, long Nk, double* f[9], const double coef[7],
                       const oracle_source* src, int nsrc, long step0, int steps) {
    double* J[3] = {f[6], f[7], f[8]};
    for (int s = 0; s < steps; ++s) {
        const long step = step0 + s;
        for (int q = 0; q < nsrc; ++q) {
            const oracle_source* b = &src[q];
#pragma omp parallel for schedule(static)
            for (long dk = 0; dk < b->nk; ++dk) {
                const long k = (b->k0 + dk) % Nk;
                for (long dj = 0; dj < b->nj; ++dj) {
                    const long j = (b->j0 + dj) % Nj;
                    for (long di = 0; di < b->ni; ++di) {
                        const long idx = (b->i0 + di) % Ni + j * Ni + k * Ni * Nj;
                        for (int c = 0; c < 3; ++c)
                            if (b->comp_mask & (1 << c)) J[c][idx] = 0.0;
                    }
                }
            }
        }
        oracle_add_sources(Ni, Nj, Nk, J, src, nsrc, step);
        oracle_update_B(Ni, Nj, Nk, f[0], f[1], f[2], f[3], f[4], f[5], coef[3], coef[4], coef[5]);
        oracle_update_E(Ni, Nj, Nk, f[3], f[4], f[5], J[0], J[1], J[2], f[0], f[1], f[2],
                        coef[6], coef[0], coef[1], coef[2]);
        oracle_update_B(Ni, Nj, Nk, f[0], f[1], f[2], f[3], f[4], f[5], coef[3], coef[4], coef[5]);
    }
}

/* ------------------------------------------------------------------------
 * The reference's OpenMP solver twin, FDTD_openmp::FDTD
 * (src/FDTD/FDTD.cpp:63-157): the second timed CPU path of the benchmark.
 *
 * Its loops differ from the Kokkos path's: OpenMP over k, the plane and row
 * offsets and the wrapped neighbour rows computed once per k and per j, and
 * an `omp simd` loop over i (FDTD.cpp:64-97 E, :99-130 B).  Its E update adds
 * cur_coef * Jx to all three components (FDTD.cpp:82-90), so it is the
 * Kokkos path only at J = 0; this restatement keeps that line, so it gives
 * the twin's results and streams the twin's bytes (Jx read, Jy and Jz not).
 * f = the nine arrays in component order (f[6] must exist). */
static void twin_update_E(long Ni, long Nj, long Nk, double* f[9], const double coef[7]) {
    const double* Bx = f[3];
    const double* By = f[4];
    const double* Bz = f[5];
    const double* Jx = f[6];
    double* Ex = f[0];
    double* Ey = f[1];
    double* Ez = f[2];
    const double cJ = coef[6], cx = coef[0], cy = coef[1], cz = coef[2];
    const long plane = Ni * Nj;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < Nk; ++k) {
        const long zk = k * plane, zp = wrap(k - 1, Nk) * plane;
        for (long j = 0; j < Nj; ++j) {
            const long row = zk + j * Ni;           /* (., j, k) */
            const long row_jp = zk + wrap(j - 1, Nj) * Ni;  /* (., j-1, k) */
            const long row_kp = zp + j * Ni;        /* (., j, k-1) */
#pragma omp simd
            for (long i = 0; i < Ni; ++i) {
                const long c = row + i, ip = row + wrap(i - 1, Ni);
                const long jp = row_jp + i, kp = row_kp + i;
                Ex[c] += cJ * Jx[c] + cy * (Bz[c] - Bz[jp]) - cz * (By[c] - By[kp]);
                Ey[c] += cJ * Jx[c] + cz * (Bx[c] - Bx[kp]) - cx * (Bz[c] - Bz[ip]);
                Ez[c] += cJ * Jx[c] + cx * (By[c] - By[ip]) - cy * (Bx[c] - Bx[jp]);
            }
        }
    }
}

static void twin_update_B(long Ni, long Nj, long Nk, double* f[9], const double coef[7]) {
    const double* Ex = f[0];
    const double* Ey = f[1];
    const double* Ez = f[2];
    double* Bx = f[3];
    double* By = f[4];
    double* Bz = f[5];
    const double cx = coef[3], cy = coef[4], cz = coef[5];
    const long plane = Ni * Nj;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < Nk; ++k) {
        const long zk = k * plane, zn = wrap(k + 1, Nk) * plane;
        for (long j = 0; j < Nj; ++j) {
            const long row = zk + j * Ni;           /* (., j, k) */
            const long row_jn = zk + wrap(j + 1, Nj) * Ni;  /* (., j+1, k) */
            const long row_kn = zn + j * Ni;        /* (., j, k+1) */
#pragma omp simd
            for (long i = 0; i < Ni; ++i) {
                const long c = row + i, in = row + wrap(i + 1, Ni);
                const long jn = row_jn + i, kn = row_kn + i;
                Bx[c] += cz * (Ey[kn] - Ey[c]) - cy * (Ez[jn] - Ez[c]);
                By[c] += cx * (Ez[in] - Ez[c]) - cz * (Ex[kn] - Ex[c]);
                Bz[c] += cy * (Ex[jn] - Ex[c]) - cx * (Ey[in] - Ey[c]);
            }
        }
    }
}

/* FDTD_openmp::FDTD::update_fields (src/FDTD/FDTD.cpp:153-157) `steps` times. */
void oracle_twin_run(long Ni, long Nj, long Nk, double* f[9], const double coef[7], int steps) {
    for (int s = 0; s < steps; ++s) {
        twin_update_B(Ni, Nj, Nk, f, coef);
        twin_update_E(Ni, Nj, Nk, f, coef);
        twin_update_B(Ni, Nj, Nk, f, coef);
    }
}

/* ------------------------------------------------------------------------
 * PML: the reference's split-field absorbing layer (class FDTD_PML).
 *
 * Layer thickness per axis: (int)(N * pml_percent) cells at both ends
 * (FDTD_PML_kokkos.cpp:71-73).  The conductivity of an axis depends only on
 * the distance d (in cells) into the layer: sigma = SGm * (d / pml)^4 with
 * SGm = -(4 + 1)/2 * ln(R) / (pml * dx) and R = 1e-12
 * (FDTD_PML_kokkos.cpp:108-116, :132-136, kokkos_functors.h:182-189); the
 * distance is pml - i in the lower layer and i + 1 + pml - N in the upper one
 * (FDTD_PML_kokkos.cpp:109-127), and sigma is zero outside the layer (the
 * reference leaves those cells unset: its first touch is commented out,
 * FDTD_PML_kokkos.cpp:47-69; zero is what its arrays hold on a fresh
 * allocation).  E and B use the same conductivity.
 *
 * The split fields Exy, Exz, Eyx, Eyz, Ezx, Ezy, Bxy, Bxz, Byx, Byz, Bzx, Bzy
 * start at zero and live on the whole grid (as the reference's arrays). */
#define ORACLE_PML_N 4.0
#define ORACLE_PML_R 1e-12

/* Layer thickness of each axis. */
void oracle_pml_sizes(const oracle_params* p, double pml_percent, int pml[3]) {
    pml[0] = (int)((double)p->Ni * pml_percent);
    pml[1] = (int)((double)p->Nj * pml_percent);
    pml[2] = (int)((double)p->Nk * pml_percent);
}

/* Conductivity profile of one axis of n cells with a layer of `pml` cells and
 * spacing d: sig[0..n-1] (zero outside the two layers). */
static void pml_sigma_axis(long n, int pml, double d, double* sig) {
    for (long i = 0; i < n; ++i) sig[i] = 0.0;
    if (pml <= 0) return;
    const double sgm = -(ORACLE_PML_N + 1.0) / 2.0 * log(ORACLE_PML_R) / ((double)pml * d);
    for (long i = 0; i < pml; ++i)
        sig[i] = sgm * pow((double)(pml - i) / (double)pml, ORACLE_PML_N);
    for (long i = n - pml; i < n; ++i)
        sig[i] = sgm * pow((double)(i + 1 + pml - n) / (double)pml, ORACLE_PML_N);
}

void oracle_pml_sigma(const oracle_params* p, double pml_percent, double* sx, double* sy, double* sz) {
    int pml[3];
    oracle_pml_sizes(p, pml_percent, pml);
    pml_sigma_axis(p->Ni, pml[0], p->dx, sx);
    pml_sigma_axis(p->Nj, pml[1], p->dy, sy);
    pml_sigma_axis(p->Nk, pml[2], p->dz, sz);
}

/* kokkos_functors.h:211-213 (decay over one step) and the curl coefficient
 * of :279-292 / :375-388. */
static inline double pml_decay(double sigma, double dt) { return exp(-sigma * dt * ORACLE_C); }
static inline double pml_coef2(double sigma, double dt, double d) {
    if (sigma != 0.0) return (1.0 - pml_decay(sigma, dt)) / (sigma * d);
    return ORACLE_C * dt / d;
}

/* kokkos_functors.h:261-309: split-field E update over a box. */
static void pml_update_E(long Ni, long Nj, long Nk, oracle_box b, double* f[9], double* s[12],
                         const double* sig[3], double dt, double dx, double dy, double dz) {
    const long plane = Ni * Nj;
    double *Ex = f[0], *Ey = f[1], *Ez = f[2];
    const double *Bx = f[3], *By = f[4], *Bz = f[5];
    double *Exy = s[0], *Exz = s[1], *Eyx = s[2], *Eyz = s[3], *Ezx = s[4], *Ezy = s[5];
#pragma omp parallel for schedule(static)
    for (long k = b.k0; k < b.k1; ++k) {
        const long kp = wrap(k - 1, Nk);
        for (long j = b.j0; j < b.j1; ++j) {
            const long jp = wrap(j - 1, Nj);
            for (long i = b.i0; i < b.i1; ++i) {
                const long ip = wrap(i - 1, Ni);
                const long idx = i + j * Ni + k * plane;
                const long i_p = ip + j * Ni + k * plane;
                const long j_p = i + jp * Ni + k * plane;
                const long k_p = i + j * Ni + kp * plane;
                const double c2x = pml_coef2(sig[0][i], dt, dx);
                const double c2y = pml_coef2(sig[1][j], dt, dy);
                const double c2z = pml_coef2(sig[2][k], dt, dz);
                const double ax = pml_decay(sig[0][i], dt), ay = pml_decay(sig[1][j], dt),
                             az = pml_decay(sig[2][k], dt);
                Eyx[idx] = Eyx[idx] * ax - c2x * (Bz[idx] - Bz[i_p]);
                Ezx[idx] = Ezx[idx] * ax + c2x * (By[idx] - By[i_p]);
                Exy[idx] = Exy[idx] * ay + c2y * (Bz[idx] - Bz[j_p]);
                Ezy[idx] = Ezy[idx] * ay - c2y * (Bx[idx] - Bx[j_p]);
                Exz[idx] = Exz[idx] * az - c2z * (By[idx] - By[k_p]);
                Eyz[idx] = Eyz[idx] * az + c2z * (Bx[idx] - Bx[k_p]);
                Ex[idx] = Exz[idx] + Exy[idx];
                Ey[idx] = Eyx[idx] + Eyz[idx];
                Ez[idx] = Ezy[idx] + Ezx[idx];
            }
        }
    }
}

/* kokkos_functors.h:357-405: split-field B update over a box. */
static void pml_update_B(long Ni, long Nj, long Nk, oracle_box b, double* f[9], double* s[12],
                         const double* sig[3], double dt, double dx, double dy, double dz) {
    const long plane = Ni * Nj;
    const double *Ex = f[0], *Ey = f[1], *Ez = f[2];
    double *Bx = f[3], *By = f[4], *Bz = f[5];
    double *Bxy = s[6], *Bxz = s[7], *Byx = s[8], *Byz = s[9], *Bzx = s[10], *Bzy = s[11];
#pragma omp parallel for schedule(static)
    for (long k = b.k0; k < b.k1; ++k) {
        const long kn = wrap(k + 1, Nk);
        for (long j = b.j0; j < b.j1; ++j) {
            const long jn = wrap(j + 1, Nj);
            for (long i = b.i0; i < b.i1; ++i) {
                const long in = wrap(i + 1, Ni);
                const long idx = i + j * Ni + k * plane;
                const long i_n = in + j * Ni + k * plane;
                const long j_n = i + jn * Ni + k * plane;
                const long k_n = i + j * Ni + kn * plane;
                const double c2x = pml_coef2(sig[0][i], dt, dx);
                const double c2y = pml_coef2(sig[1][j], dt, dy);
                const double c2z = pml_coef2(sig[2][k], dt, dz);
                const double ax = pml_decay(sig[0][i], dt), ay = pml_decay(sig[1][j], dt),
                             az = pml_decay(sig[2][k], dt);
                Byx[idx] = Byx[idx] * ax + c2x * (Ez[i_n] - Ez[idx]);
                Bzx[idx] = Bzx[idx] * ax - c2x * (Ey[i_n] - Ey[idx]);
                Bxy[idx] = Bxy[idx] * ay - c2y * (Ez[j_n] - Ez[idx]);
                Bzy[idx] = Bzy[idx] * ay + c2y * (Ex[j_n] - Ex[idx]);
                Bxz[idx] = Bxz[idx] * az + c2z * (Ey[k_n] - Ey[idx]);
                Byz[idx] = Byz[idx] * az - c2z * (Ex[k_n] - Ex[idx]);
                Bx[idx] = Bxy[idx] + Bxz[idx];
                By[idx] = Byz[idx] + Byx[idx];
                Bz[idx] = Bzx[idx] + Bzy[idx];
            }
        }
    }
}

/* The six layer slabs of FDTD_PML::update_fields (FDTD_PML_kokkos.cpp:170-186):
 * they tile everything outside the main box exactly once. */
void oracle_pml_slabs(long Ni, long Nj, long Nk, const int pml[3], oracle_box out[6]) {
    const long pi = pml[0], pj = pml[1], pk = pml[2];
    const oracle_box s[6] = {
        {0, Ni - pi, 0, Nj, 0, pk},             /* part_from_start i, all j, lower k */
        {pi, Ni - pi, 0, pj, pk, Nk - pk},      /* main i, lower j, main k           */
        {0, pi, 0, Nj, pk, Nk},                 /* lower i, all j, part_from_end k   */
        {pi, Ni, 0, Nj, Nk - pk, Nk},           /* part_from_end i, all j, upper k   */
        {pi, Ni - pi, Nj - pj, Nj, pk, Nk - pk},/* main i, upper j, main k           */
        {Ni - pi, Ni, 0, Nj, 0, Nk - pk}};      /* upper i, all j, part_from_start k */
    for (int q = 0; q < 6; ++q) out[q] = s[q];
}

/* FDTD_PML::update_fields (FDTD_PML_kokkos.cpp:162-189) repeated `steps` times:
 * B/2 on the main box; the split-field B update on the six slabs (a whole
 * step: its coefficient is c dt/d); E on the main box (with current); the
 * split-field E update on the slabs; B/2 on the main box.  f as in oracle_run
 * (f[6..8] may be null); split = the twelve split fields; sig = the three
 * conductivity profiles (oracle_pml_sigma).  Sources as in oracle_run. */
void oracle_pml_run(long Ni, long Nj, long Nk, double* f[9], const double coef[7], const int pml[3],
                    const double* sig[3], double dt, double dx, double dy, double dz, double* split[12],
                    const oracle_source* src, int nsrc, long step0, int steps, double* jwork[3]) {
    const long n = Ni * Nj * Nk;
    const oracle_box main_box = {pml[0], Ni - pml[0], pml[1], Nj - pml[1], pml[2], Nk - pml[2]};
    oracle_box slab[6];
    oracle_pml_slabs(Ni, Nj, Nk, pml, slab);
    for (int s = 0; s < steps; ++s) {
        const double* J[3] = {f[6], f[7], f[8]};
        if (nsrc > 0) {
            for (int c = 0; c < 3; ++c) {
                if (f[6 + c]) memcpy(jwork[c], f[6 + c], sizeof(double) * n);
                else memset(jwork[c], 0, sizeof(double) * n);
            }
            oracle_add_sources(Ni, Nj, Nk, jwork, src, nsrc, step0 + s);
            J[0] = jwork[0];
            J[1] = jwork[1];
            J[2] = jwork[2];
        }
        oracle_update_B_box(Ni, Nj, Nk, main_box, f[0], f[1], f[2], f[3], f[4], f[5], coef[3], coef[4], coef[5]);
        for (int q = 0; q < 6; ++q) pml_update_B(Ni, Nj, Nk, slab[q], f, split, sig, dt, dx, dy, dz);
        oracle_update_E_box(Ni, Nj, Nk, main_box, f[3], f[4], f[5], J[0], J[1], J[2], f[0], f[1], f[2],
                            coef[6], coef[0], coef[1], coef[2]);
        for (int q = 0; q < 6; ++q) pml_update_E(Ni, Nj, Nk, slab[q], f, split, sig, dt, dx, dy, dz);
        oracle_update_B_box(Ni, Nj, Nk, main_box, f[0], f[1], f[2], f[3], f[4], f[5], coef[3], coef[4], coef[5]);
    }
}

/* Field diagnostics (new; the reference has none).  Neumaier-compensated FP64
 * sums over all cells:
 *   out[0..5] = sum Ex^2, Ey^2, Ez^2, Bx^2, By^2, Bz^2
 *   out[6..8] = sum (Ey Bz - Ez By), (Ez Bx - Ex Bz), (Ex By - Ey Bx)
 *   out[9]    = number of non-finite values among the six fields
 * Energy and Poynting integrals follow by the factors dV/(8 pi) and
 * c dV/(4 pi). */
void oracle_field_sums(long n, const double* f[6], double out[10]) {
    double s[9], c[9];
    long bad = 0;
    for (int q = 0; q < 9; ++q) s[q] = c[q] = 0.0;
    for (long i = 0; i < n; ++i) {
        double v[9];
        const double ex = f[0][i], ey = f[1][i], ez = f[2][i];
        const double bx = f[3][i], by = f[4][i], bz = f[5][i];
        v[0] = ex * ex; v[1] = ey * ey; v[2] = ez * ez;
        v[3] = bx * bx; v[4] = by * by; v[5] = bz * bz;
        v[6] = ey * bz - ez * by;
        v[7] = ez * bx - ex * bz;
        v[8] = ex * by - ey * bx;
        for (int q = 0; q < 6; ++q) bad += !isfinite(f[q][i]);
        for (int q = 0; q < 9; ++q) {
            const double t = s[q] + v[q];
            if (fabs(s[q]) >= fabs(v[q])) c[q] += (s[q] - t) + v[q];
            else c[q] += (v[q] - t) + s[q];
            s[q] = t;
        }
    }
    for (int q = 0; q < 9; ++q) out[q] = s[q] + c[q];
    out[9] = (double)bad;
}
