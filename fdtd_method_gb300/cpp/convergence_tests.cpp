// The reference's 12 convergence tests (unit-tests/test_FDTD_method_kokkos.cpp:7-201,
// with its helper Test_FDTD, src/FDTD_kokkos/test_FDTD_kokkos.cpp:7-161),
// restated against the drop-in class of fdtd_gb300.hpp: a plane wave along
// one axis run at (N, dt) and (2N, dt/2); the ratio of the max-abs errors
// must be 4 +- 0.1.  Prints one line per test:
//   NEAR <name> <ratio %.17g> 4 0.1 <PASS|FAIL>
// and exits non-zero if any test fails.
#include <cmath>
#include <cstdio>
#include <functional>
#include <stdexcept>

#include "fdtd_gb300.hpp"

using namespace FDTD_gb300;

namespace {

const FP default_time = 5e-13;

FP initial_func(FP x, const FP size[2]) {
  return std::sin(2.0 * FDTD_const::PI * (x - size[0]) / (size[1] - size[0]));
}
FP true_func(FP x, FP t, const FP size[2]) {
  return std::sin(2.0 * FDTD_const::PI * (x - size[0] - FDTD_const::C * t) / (size[1] - size[0]));
}

FP sign_of(Component e, Component b) {
  if ((e == Component::EX && b == Component::BZ) || (e == Component::EZ && b == Component::BY) ||
      (e == Component::EY && b == Component::BX))
    return -1.0;
  if ((e == Component::EY && b == Component::BZ) || (e == Component::EZ && b == Component::BX) ||
      (e == Component::EX && b == Component::BY))
    return 1.0;
  throw std::logic_error("ERROR: invalid selected fields");
}
int axis_of(Component e, Component b) {
  if ((e == Component::EY && b == Component::BZ) || (e == Component::EZ && b == Component::BY)) return 0;
  if ((e == Component::EX && b == Component::BZ) || (e == Component::EZ && b == Component::BX)) return 1;
  if ((e == Component::EX && b == Component::BY) || (e == Component::EY && b == Component::BX)) return 2;
  throw std::logic_error("ERROR: invalid selected fields");
}

FP run_once(Component test_field, SelectedFields sel, int Ni, int Nj, int Nk, int iters) {
  Parameters p{Ni, Nj, Nk, 0.0, 1.0, 0.0, 2.0, 0.0, 3.0, (1 - 0) / static_cast<FP>(Ni),
               (2 - 0) / static_cast<FP>(Nj), (3 - 0) / static_cast<FP>(Nk)};
  const FP dt = default_time / static_cast<FP>(iters);
  FDTD method(p, dt);
  const int axis = axis_of(sel.selected_E, sel.selected_B);
  FP sign = sign_of(sel.selected_E, sel.selected_B);
  const int n[3] = {Ni, Nj, Nk};
  const FP d[3] = {p.dx, p.dy, p.dz};
  const FP size[3][2] = {{p.ax, p.bx}, {p.ay, p.by}, {p.az, p.bz}};
  const long stride[3] = {1, Ni, static_cast<long>(Ni) * Nj};

  // initial filling (test_FDTD_kokkos.cpp:7-66)
  auto& E = method.get_field(sel.selected_E);
  auto& B = method.get_field(sel.selected_B);
  auto e_host = create_mirror_view(E);
  auto b_host = create_mirror_view(B);
  const FP d_b = d[axis] / 2.0;
  for (long idx = 0; idx < static_cast<long>(e_host.size()); ++idx) {
    const long q = (idx / stride[axis]) % n[axis];
    const FP u = static_cast<FP>(q) * d[axis];
    e_host(idx) = sign * initial_func(u, size[axis]);
    b_host(idx) = initial_func(d_b + u, size[axis]);
  }
  deep_copy(E, e_host);
  deep_copy(B, b_host);

  for (int t = 0; t < iters; t++) method.update_fields();

  // max-abs error along one grid line (test_FDTD_kokkos.cpp:103-161)
  auto& F = method.get_field(test_field);
  auto f_host = create_mirror_view(F);
  deep_copy(f_host, F);
  FP u = 0.0;
  if (static_cast<int>(test_field) > static_cast<int>(Component::EZ)) {
    sign = 1.0;
    u = d[axis] / 2.0;
  }
  FP worst = 0.0;
  for (int q = 0; q < n[axis]; ++q, u += d[axis]) {
    const FP err = std::fabs(sign * f_host(q * stride[axis]) - true_func(u, default_time, size[axis]));
    if (err > worst) worst = err;
  }
  return worst;
}

FP run_test(Component test_field, SelectedFields sel, int Ni, int Nj, int Nk) {
  return run_once(test_field, sel, Ni, Nj, Nk, 16) / run_once(test_field, sel, 2 * Ni, 2 * Nj, 2 * Nk, 32);
}

struct Case {
  const char* name;
  Component field;
  SelectedFields sel;
  int n[3];
};

}  // namespace

int main() {
  using C = Component;
  const Case cases[] = {
      {"x_axis_EY", C::EY, {C::EY, C::BZ}, {16, 8, 4}}, {"x_axis_BZ", C::BZ, {C::EY, C::BZ}, {16, 8, 4}},
      {"x_axis_EZ", C::EZ, {C::EZ, C::BY}, {16, 8, 4}}, {"x_axis_BY", C::BY, {C::EZ, C::BY}, {16, 8, 4}},
      {"y_axis_EX", C::EX, {C::EX, C::BZ}, {8, 16, 4}}, {"y_axis_BZ", C::BZ, {C::EX, C::BZ}, {8, 16, 4}},
      {"y_axis_EZ", C::EZ, {C::EZ, C::BX}, {8, 16, 4}}, {"y_axis_BX", C::BX, {C::EZ, C::BX}, {8, 16, 4}},
      {"z_axis_EX", C::EX, {C::EX, C::BY}, {4, 8, 16}}, {"z_axis_BY", C::BY, {C::EX, C::BY}, {4, 8, 16}},
      {"z_axis_EY", C::EY, {C::EY, C::BX}, {4, 8, 16}}, {"z_axis_BX", C::BX, {C::EY, C::BX}, {4, 8, 16}},
  };
  int failed = 0;
  for (const Case& c : cases) {
    const FP r = run_test(c.field, c.sel, c.n[0], c.n[1], c.n[2]);
    const bool ok = std::fabs(r - 4.0) <= 0.1;
    std::printf("NEAR Convergence_kokkos.%s %.17g 4 0.1 %s\n", c.name, r, ok ? "PASS" : "FAIL");
    failed += ok ? 0 : 1;
  }
  std::printf("SUMMARY 12 tests, %d failed\n", failed);
  return failed ? 1 : 0;
}
