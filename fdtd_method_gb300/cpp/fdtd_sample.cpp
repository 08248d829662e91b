// GPU twin of the reference's sample driver
// (perf-tests/kokkos_sample/kokkos_sample.cpp): a box current
// sin(2 pi t/T) cos^2(2 pi x/Tx) cos^2(2 pi y/Ty) cos^2(2 pi z/Tz) in Jx, Jy, Jz
// for period/dt steps, then a free run; prints the execution time and the same
// 10 x 10 slice of Ex.  Usage: fdtd_sample [N iters [pml]]  (default 32 100).
// With "pml" it also runs the same source on FDTD_PML(params, dt, 0.2) and
// prints its execution time, as the reference's sample does under
// __PML_TEST__ (perf-tests/sample/sample.cpp:93-123).
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "fdtd_gb300.hpp"

using namespace FDTD_gb300;

static void spherical_wave(int n, int it, bool with_pml) {
  CurrentParameters cur_param{8, 4, 0.2};
  const double T = cur_param.period;
  const double Tx = cur_param.period_x, Ty = cur_param.period_y, Tz = cur_param.period_z;
  cur_param.iterations = static_cast<int>(static_cast<double>(cur_param.period) / cur_param.dt);

  const double d = FDTD_const::C;
  const double boundary = static_cast<double>(n) / 2.0 * d;
  Parameters params{n, n, n, -boundary, boundary, -boundary, boundary, -boundary, boundary, d, d, d};
  FDTD method(params, cur_param.dt);

  const int cur_time = std::min(cur_param.iterations, it);
  const int start[3] = {static_cast<int>(std::floor((-Tx / 4.0 - params.ax) / params.dx)),
                        static_cast<int>(std::floor((-Ty / 4.0 - params.ay) / params.dy)),
                        static_cast<int>(std::floor((-Tz / 4.0 - params.az) / params.dz))};
  const int stop[3] = {static_cast<int>(std::floor((Tx / 4.0 - params.ax) / params.dx)),
                       static_cast<int>(std::floor((Ty / 4.0 - params.ay) / params.dy)),
                       static_cast<int>(std::floor((Tz / 4.0 - params.az) / params.dz))};
  const double period[3] = {Tx, Ty, Tz};
  const double step[3] = {params.dx, params.dy, params.dz};
  std::vector<double> g[3];
  for (int a = 0; a < 3; ++a)
    for (int v = start[a]; v < stop[a]; ++v)
      g[a].push_back(std::pow(std::cos(2.0 * FDTD_const::PI * (v * step[a]) / period[a]), 2.0));
  std::vector<double> amp(cur_time);
  for (int t = 0; t < cur_time; ++t) amp[t] = std::sin(2.0 * FDTD_const::PI * ((t + 1) * cur_param.dt) / T);

  if (!g[0].empty() && !g[1].empty() && !g[2].empty() && cur_time > 0) {
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
    s.n_amp = cur_time;
    method.add_source(s);
  }

  auto t0 = std::chrono::high_resolution_clock::now();
  method.step(it);
  method.fence();
  auto t1 = std::chrono::high_resolution_clock::now();
  std::chrono::duration<double> elapsed = t1 - t0;
  std::cout << "Execution time: " << elapsed.count() << " s" << std::endl;

  if (with_pml) {
    FDTD_PML pml_method(params, cur_param.dt, 0.2);
    if (!g[0].empty() && !g[1].empty() && !g[2].empty() && cur_time > 0) {
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
      s.n_amp = cur_time;
      pml_method.add_source(s);
    }
    auto p0 = std::chrono::high_resolution_clock::now();
    pml_method.step(it);
    pml_method.fence();
    auto p1 = std::chrono::high_resolution_clock::now();
    std::chrono::duration<double> elapsed_pml = p1 - p0;
    std::cout << "Execution time (PML): " << elapsed_pml.count() << " s" << std::endl;
    double sums[FDTD_DIAG_COUNT];
    pml_method.field_sums(sums);
    double e2 = 0.0;
    for (int c = 0; c < 6; ++c) e2 += sums[c];
    std::cout << "PML field square sum: " << std::scientific << std::setprecision(6) << e2 << std::endl;
  }

  auto& Ex_device = method.get_field(Component::EX);
  auto Ex_host = create_mirror_view(Ex_device);
  deep_copy(Ex_host, Ex_device);
  const int i = params.Nk / 2;
  for (int j = params.Nj / 2 - 5; j < params.Nj / 2 + 5; j++) {
    for (int k = params.Ni / 2 - 5; k < params.Ni / 2 + 5; k++) {
      const long index = i + static_cast<long>(j) * params.Ni + static_cast<long>(k) * params.Ni * params.Nj;
      std::cout << std::setw(12) << std::fixed << std::setprecision(5) << Ex_host(index);
    }
    std::cout << std::endl;
  }
  std::cout << std::endl;
}

int main(int argc, char* argv[]) {
  try {
    if (argc == 1) {
      spherical_wave(32, 100, false);
    } else if (argc == 3) {
      spherical_wave(std::atoi(argv[1]), std::atoi(argv[2]), false);
    } else if (argc == 4 && std::string(argv[3]) == "pml") {
      spherical_wave(std::atoi(argv[1]), std::atoi(argv[2]), true);
    } else {
      std::cout << "ERROR: Incorrect number of parameters" << std::endl;
      return 1;
    }
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 2;
  }
  return 0;
}
