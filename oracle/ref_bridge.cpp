// C entry points over the reference's own FDTD classes, compiled from the
// reference's unmodified sources against the host Kokkos stand-in in
// kokkos_shim/.  Test infrastructure only (the oracle): tests and the CPU
// baseline call these to obtain the reference's results and timings on the
// same inputs the CUDA engine gets.  Nothing here is part of the engine.
//
// Wrapped reference interfaces:
//   FDTD_kokkos::FDTD           include/FDTD_kokkos/FDTD_kokkos.h:7-36
//   FDTD_kokkos::FDTD_PML       include/FDTD_kokkos/FDTD_PML_kokkos.h:10-33
//   FDTD_openmp::FDTD           include/FDTD/FDTD.h:9-41      (REF_WITH_OPENMP_TWIN)
//   run_test_kokkos             unit-tests/test_FDTD_method_kokkos.cpp:18-69
#include <cstring>
#include <exception>
#include <string>

#include "FDTD_PML_kokkos.h"
#include "FDTD_kokkos.h"
#ifdef REF_WITH_OPENMP_TWIN
#include "FDTD.h"
#endif

using FDTD_enums::Component;

// Defined in the reference's unit-test source, linked in unmodified.
FP run_test_kokkos(Component test_field, FDTD_struct::SelectedFields current_fields,
                   int Ni, int Nj, int Nk);

namespace {
thread_local std::string g_err;
FDTD_struct::Parameters make_params(const int n[3], const double b[9]) {
  FDTD_struct::Parameters p{n[0], n[1], n[2], b[0], b[1], b[2], b[3], b[4], b[5], b[6], b[7], b[8]};
  return p;
}
}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

// n = {Ni,Nj,Nk}; b = {ax,bx,ay,by,az,bz,dx,dy,dz}.  Returns nullptr and sets
// the error text when the reference constructor throws.
void* ref_kokkos_create(const int* n, const double* b, double dt) {
  try {
    return new FDTD_kokkos::FDTD(make_params(n, b), dt);
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void ref_kokkos_destroy(void* h) { delete static_cast<FDTD_kokkos::FDTD*>(h); }

// The PML subclass, handed out as its FDTD base (update_fields is virtual,
// get_field is the base's); destroyed through its own type.
void* ref_kokkos_pml_create(const int* n, const double* b, double dt, double pml_percent) {
  try {
    FDTD_kokkos::FDTD* base = new FDTD_kokkos::FDTD_PML(make_params(n, b), dt, pml_percent);
    return base;
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void ref_kokkos_pml_destroy(void* h) {
  delete static_cast<FDTD_kokkos::FDTD_PML*>(static_cast<FDTD_kokkos::FDTD*>(h));
}

void ref_kokkos_update_fields(void* h, int steps) {
  auto* f = static_cast<FDTD_kokkos::FDTD*>(h);
  for (int s = 0; s < steps; ++s) f->update_fields();
}
void ref_kokkos_zeroed_currents(void* h) { static_cast<FDTD_kokkos::FDTD*>(h)->zeroed_currents(); }

// dir = 0: field -> host buffer; dir = 1: host buffer -> field.  Returns 0, or
// -2 with the reference's logic_error text for an invalid component.
int ref_kokkos_field(void* h, int comp, double* buf, long n, int dir) {
  try {
    auto& fld = static_cast<FDTD_kokkos::FDTD*>(h)->get_field(static_cast<Component>(comp));
    if (static_cast<long>(fld.size()) != n) { g_err = "size mismatch"; return -1; }
    if (dir == 0) std::memcpy(buf, fld.data(), sizeof(double) * n);
    else std::memcpy(fld.data(), buf, sizeof(double) * n);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -2;
  }
}

// The reference's own convergence experiment; returns err(N)/err(2N).
double ref_run_test_kokkos(int test_field, int sel_E, int sel_B, int Ni, int Nj, int Nk) {
  FDTD_struct::SelectedFields sf{static_cast<Component>(sel_E), static_cast<Component>(sel_B)};
  return run_test_kokkos(static_cast<Component>(test_field), sf, Ni, Nj, Nk);
}

#ifdef REF_WITH_OPENMP_TWIN
void* ref_omp_create(const int* n, const double* b, double dt) {
  try {
    return new FDTD_openmp::FDTD(make_params(n, b), dt);
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void ref_omp_destroy(void* h) { delete static_cast<FDTD_openmp::FDTD*>(h); }
void ref_omp_update_fields(void* h, int steps) {
  auto* f = static_cast<FDTD_openmp::FDTD*>(h);
  for (int s = 0; s < steps; ++s) f->update_fields();
}
int ref_omp_field(void* h, int comp, double* buf, long n, int dir) {
  try {
    auto& fld = static_cast<FDTD_openmp::FDTD*>(h)->get_field(static_cast<Component>(comp));
    if (static_cast<long>(fld.size()) != n) { g_err = "size mismatch"; return -1; }
    if (dir == 0) std::memcpy(buf, fld.data(), sizeof(double) * n);
    else std::memcpy(fld.data(), buf, sizeof(double) * n);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -2;
  }
}
#endif
}
