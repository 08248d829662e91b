// GPU twin of the reference's coarray program (coarray/fdtd.F90): the grid
// split into z slabs as its images split it (init_decomposition, :149-164),
// stepped with its halo exchange (next_Ex/Ey, pred_Bx/By, :86-102) as device
// copies between slabs on one GPU.  The current is the program's box
// (init_currents, :184-204): sin(2 pi t dt/TT) cos^2(2 pi x/Tx) cos^2(2 pi y/Ty)
// cos^2(2 pi z/Tz) in Jx, Jy, Jz for min(TT/dt, iterations) steps, then none.
// Prints the image count, the execution time and the same 10 x 10 slice of
// Ex at plane Nk/2+1 (print_full_E_slice, :292-302).
// Usage: fdtd_coarray_sample [N iterations slabs]  (default 512 25 4).
//
// The arithmetic is the engine's FP64 drop-in (the Kokkos functors' operation
// order), so the slab run prints what one whole-grid handle prints.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <vector>

#include "fdtd_gb300.hpp"

using namespace FDTD_gb300;

static int run(int n, int iterations, int images) {
  const double C = FDTD_const::C, PI = FDTD_const::PI;
  const double dx = C, dt = 0.2, TT = 8.0, Tx = 4 * C, Ty = 4 * C, Tz = 4 * C;
  const int current_time = std::min(static_cast<int>(TT / dt), iterations);
  const double bnd = n / 2.0 * dx;
  // the program's 1-based box bounds, as 0-based cell indices
  const int start[3] = {static_cast<int>(std::floor((-Tx / 4.0 + bnd) / dx)),
                        static_cast<int>(std::floor((-Ty / 4.0 + bnd) / dx)),
                        static_cast<int>(std::floor((-Tz / 4.0 + bnd) / dx))};
  const int stop[3] = {static_cast<int>(std::floor((Tx / 4.0 + bnd) / dx)),
                       static_cast<int>(std::floor((Ty / 4.0 + bnd) / dx)),
                       static_cast<int>(std::floor((Tz / 4.0 + bnd) / dx))};
  const double period[3] = {Tx, Ty, Tz};
  std::vector<double> g[3];
  for (int a = 0; a < 3; ++a)
    for (int v = start[a]; v <= stop[a]; ++v) g[a].push_back(std::pow(std::cos(2.0 * PI * v * dx / period[a]), 2.0));
  std::vector<double> amp(current_time);
  for (int t = 0; t < current_time; ++t) amp[t] = std::sin(2.0 * PI * (t + 1) * dt / TT);

  Parameters params{n, n, n, -bnd, bnd, -bnd, bnd, -bnd, bnd, dx, dx, dx};
  Slabs method(params, dt, images);
  if (current_time > 0) {
    fdtd_source s{};
    s.comp_mask = 7;
    s.i0 = ((start[0] % n) + n) % n;
    s.j0 = ((start[1] % n) + n) % n;
    s.k0 = ((start[2] % n) + n) % n;
    s.ni = static_cast<int>(g[0].size());
    s.nj = static_cast<int>(g[1].size());
    s.nk = static_cast<int>(g[2].size());
    s.gx = g[0].data();
    s.gy = g[1].data();
    s.gz = g[2].data();
    s.amp = amp.data();
    s.n_amp = current_time;
    method.add_source(s);
  }

  std::cout << "Running on " << images << " images" << std::endl;
  auto t0 = std::chrono::high_resolution_clock::now();
  method.step(iterations);
  method.fence();
  auto t1 = std::chrono::high_resolution_clock::now();
  std::printf("Total execution time: %.2f seconds\n", std::chrono::duration<double>(t1 - t0).count());

  std::vector<double> ex(static_cast<std::size_t>(n) * n * n);
  method.copy_field_to_host(Component::EX, ex.data());
  const long k = n / 2;  // plane Nk/2+1 (1-based)
  for (int j = n / 2 - 5; j <= n / 2 + 4; ++j) {
    for (int i = n / 2 - 5; i <= n / 2 + 4; ++i)
      std::printf("%12.5f", ex[i + static_cast<long>(j) * n + k * static_cast<long>(n) * n]);
    std::printf("\n");
  }
  return 0;
}

int main(int argc, char* argv[]) {
  try {
    if (argc == 1) return run(512, 25, 4);
    if (argc == 4) return run(std::atoi(argv[1]), std::atoi(argv[2]), std::atoi(argv[3]));
    std::cout << "ERROR: Incorrect number of parameters" << std::endl;
    return 1;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 2;
  }
}
