// fdtd_gb300.hpp — header-only C++ drop-in for the reference's Kokkos solver
// class FDTD_kokkos::FDTD (Amazingkivas/FDTD_Method,
// include/FDTD_kokkos/FDTD_kokkos.h:7-36), over the C ABI in fdtd_gb300.h.
//
// Same names, argument meaning and error behaviour:
//   FDTD(Parameters, FP dt)     throws std::invalid_argument("ERROR: invalid parameters")
//                               (src/FDTD_kokkos/FDTD_kokkos.cpp:7-12)
//   Field& get_field(Component) throws std::logic_error("ERROR: Invalid field component")
//                               (src/FDTD_kokkos/FDTD_kokkos.cpp:75-89)
//   virtual void update_fields() one step B/2, E, B/2 (src/FDTD_kokkos/FDTD_kokkos.cpp:91-104)
//   void zeroed_currents()      (src/FDTD_kokkos/FDTD_kokkos.cpp:69-73)
// Fields live on the GPU: a Field handle aliases the solver's device array as
// the reference's View does; host access goes through create_mirror_view +
// deep_copy, as the reference sample does (perf-tests/kokkos_sample/kokkos_sample.cpp:135-139).
#pragma once

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "fdtd_gb300.h"

namespace FDTD_gb300 {

using FP = double;  // include/FP.h:3

namespace FDTD_const {  // include/Constants.h:4-12
const double C = 3e10;
const double R = 1e-12;
const double EPS0 = 1.0;
const double MU0 = EPS0;
const double N = 4.0;
const double PI = 3.14159265358;
}  // namespace FDTD_const

enum class Component { EX, EY, EZ, BX, BY, BZ, JX, JY, JZ };  // include/Enums.h:5
enum class Axis { X, Y, Z };                                   // include/Enums.h:6

enum class Precision { FP64 = FDTD_PRECISION_FP64, FP32 = FDTD_PRECISION_FP32,
                       FP32_COMP = FDTD_PRECISION_FP32_COMP, FP16_SCALED = FDTD_PRECISION_FP16_SCALED };

struct SelectedFields {  // include/Structures.h:8-11
  Component selected_E;
  Component selected_B;
};

struct CurrentParameters {  // include/Structures.h:13-21
  int period;
  int m;
  FP dt;
  int iterations;
  FP period_x = static_cast<FP>(m) * FDTD_const::C;
  FP period_y = static_cast<FP>(m) * FDTD_const::C;
  FP period_z = static_cast<FP>(m) * FDTD_const::C;
};

struct Parameters {  // include/Structures.h:23-38
  int Ni;
  int Nj;
  int Nk;
  FP ax;
  FP bx;
  FP ay;
  FP by;
  FP az;
  FP bz;
  FP dx;
  FP dy;
  FP dz;
};

// Throws the reference's exception type for a C-ABI status.
inline void check(int rc) {
  if (rc == FDTD_OK) return;
  const std::string msg = fdtd_last_error();
  if (rc == FDTD_ERR_INVALID_ARGUMENT) throw std::invalid_argument(msg);
  if (rc == FDTD_ERR_LOGIC) throw std::logic_error(msg);
  throw std::runtime_error(msg);
}

class FDTD;

// A component of a solver's state (the reference's Kokkos::View member).
class Field {
 public:
  Field() = default;
  // Device address of the Ni*Nj*Nk doubles (FP64 form only).
  double* data() const {
    double* p = nullptr;
    check(fdtd_get_field(h_, static_cast<int>(comp_), &p));
    return p;
  }
  std::size_t size() const { return n_; }
  std::size_t extent(int) const { return n_; }
  Component component() const { return comp_; }
  fdtd_handle* handle() const { return h_; }

 private:
  friend class FDTD;
  Field(fdtd_handle* h, Component c, std::size_t n) : h_(h), comp_(c), n_(n) {}
  fdtd_handle* h_ = nullptr;
  Component comp_ = Component::EX;
  std::size_t n_ = 0;
};

// Host copy of a Field (Kokkos::create_mirror_view).
class HostMirror {
 public:
  explicit HostMirror(std::size_t n = 0) : v_(n) {}
  double& operator()(long i) { return v_[static_cast<std::size_t>(i)]; }
  double operator()(long i) const { return v_[static_cast<std::size_t>(i)]; }
  double& operator[](long i) { return v_[static_cast<std::size_t>(i)]; }
  double* data() { return v_.data(); }
  const double* data() const { return v_.data(); }
  std::size_t size() const { return v_.size(); }

 private:
  std::vector<double> v_;
};

inline HostMirror create_mirror_view(const Field& f) { return HostMirror(f.size()); }
// Kokkos::deep_copy(host, device) / deep_copy(device, host)
inline void deep_copy(HostMirror& dst, const Field& src) {
  check(fdtd_copy_field_to_host(src.handle(), static_cast<int>(src.component()), dst.data(), dst.size()));
}
inline void deep_copy(const Field& dst, const HostMirror& src) {
  check(fdtd_copy_field_from_host(dst.handle(), static_cast<int>(dst.component()), src.data(), src.size()));
}

class FDTD {
 public:
  FDTD(Parameters parameters, FP dt, Precision precision = Precision::FP64) : parameters_(parameters), dt_(dt) {
    fdtd_params p{parameters.Ni, parameters.Nj, parameters.Nk, parameters.ax, parameters.bx, parameters.ay,
                  parameters.by, parameters.az, parameters.bz, parameters.dx, parameters.dy, parameters.dz};
    check(fdtd_create(&p, dt, static_cast<int>(precision), &h_));
    const std::size_t n = static_cast<std::size_t>(parameters.Ni) * parameters.Nj * parameters.Nk;
    for (int c = 0; c < 9; ++c) fields_[c] = Field(h_, static_cast<Component>(c), n);
  }
  FDTD(const FDTD&) = delete;
  FDTD& operator=(const FDTD&) = delete;
  virtual ~FDTD() { fdtd_destroy(h_); }

 protected:
  // For subclasses that create their handle with another constructor.
  FDTD(Parameters parameters, FP dt, fdtd_handle* h) : parameters_(parameters), dt_(dt), h_(h) {
    const std::size_t n = static_cast<std::size_t>(parameters.Ni) * parameters.Nj * parameters.Nk;
    for (int c = 0; c < 9; ++c) fields_[c] = Field(h_, static_cast<Component>(c), n);
  }
  static fdtd_handle* create_pml(const Parameters& parameters, FP dt, FP pml_percent) {
    fdtd_params p{parameters.Ni, parameters.Nj, parameters.Nk, parameters.ax, parameters.bx, parameters.ay,
                  parameters.by, parameters.az, parameters.bz, parameters.dx, parameters.dy, parameters.dz};
    fdtd_handle* h = nullptr;
    check(fdtd_create_pml(&p, dt, pml_percent, FDTD_PRECISION_FP64, &h));
    return h;
  }

 public:

  Field& get_field(Component c) {
    const int i = static_cast<int>(c);
    if (i < 0 || i > 8) throw std::logic_error("ERROR: Invalid field component");
    return fields_[i];
  }

  virtual void update_fields() { check(fdtd_update_fields(h_)); }
  void zeroed_currents() { check(fdtd_zeroed_currents(h_)); }

  // Extensions.
  void step(int64_t n) { check(fdtd_step(h_, n)); }
  void fence() { check(fdtd_synchronize(h_)); }
  int add_source(const fdtd_source& s) {
    int idx = -1;
    check(fdtd_add_source(h_, &s, &idx));
    return idx;
  }
  void field_sums(double out[FDTD_DIAG_COUNT]) { check(fdtd_field_sums(h_, out)); }
  // FP64 form: DFMA-contracted sweeps (true) or the reference's arithmetic
  // bit for bit (false, the default).
  void set_fp64_arith(bool contracted) {
    check(fdtd_set_fp64_arith(h_, contracted ? FDTD_FP64_CONTRACTED : FDTD_FP64_BITWISE));
  }
  const Parameters& parameters() const { return parameters_; }
  FP dt() const { return dt_; }
  fdtd_handle* handle() const { return h_; }

 private:
  Parameters parameters_;
  FP dt_;
  fdtd_handle* h_ = nullptr;
  Field fields_[9];
};

// Replaces FDTD_kokkos::FDTD_PML (include/FDTD_kokkos/FDTD_PML_kokkos.h:10-33):
// the same solver with a split-field absorbing layer of (int)(N * pml_percent)
// cells on every face; update_fields follows FDTD_PML::update_fields.
class FDTD_PML : public FDTD {
 public:
  FDTD_PML(Parameters parameters, FP dt, FP pml_percent)
      : FDTD(parameters, dt, create_pml(parameters, dt, pml_percent)) {}
  void update_fields() override { check(fdtd_update_fields(handle())); }
};

// A periodic grid stepped as z slabs on one GPU: the decomposition of the
// reference's coarray program (coarray/fdtd.F90:149-164: the first Nk mod n
// slabs get one plane more) with its halo exchange (:86-102) as device
// copies.  Results equal one FDTD of the whole grid in the same precision,
// bit for bit.  The FP32-arithmetic forms run one fused sweep per step
// (FDTD_SWEEP_STEP) unless `fused` is false; the FP64 form runs the split
// sweeps.
class Slabs {
 public:
  Slabs(Parameters parameters, FP dt, int n_slabs, Precision precision = Precision::FP64, bool fused = true)
      : parameters_(parameters), defer_(precision != Precision::FP64), fused_(fused && defer_) {
    if (n_slabs <= 0 || n_slabs > parameters.Nk) throw std::invalid_argument("need 1 <= slabs <= Nk");
    fdtd_params p{parameters.Ni, parameters.Nj, parameters.Nk, parameters.ax, parameters.bx, parameters.ay,
                  parameters.by, parameters.az, parameters.bz, parameters.dx, parameters.dy, parameters.dz};
    const int base = parameters.Nk / n_slabs, extra = parameters.Nk % n_slabs;
    int k = 0;
    for (int s = 0; s < n_slabs; ++s) {
      const int size = base + (s < extra ? 1 : 0);
      fdtd_handle* h = nullptr;
      const int rc = fdtd_slab_create(&p, dt, static_cast<int>(precision), k, k + size, &h);
      if (rc != FDTD_OK) {
        release();
        check(rc);
      }
      slabs_.push_back(h);
      bounds_.push_back({k, k + size});
      k += size;
    }
  }
  Slabs(const Slabs&) = delete;
  Slabs& operator=(const Slabs&) = delete;
  ~Slabs() { release(); }

  int size() const { return static_cast<int>(slabs_.size()); }
  // Planes [first, second) of slab s.
  std::pair<int, int> bounds(int s) const { return bounds_.at(s); }
  fdtd_handle* slab(int s) const { return slabs_.at(s); }

  // A source in whole-grid coordinates; every slab keeps its part.
  void add_source(const fdtd_source& src) {
    for (fdtd_handle* h : slabs_) check(fdtd_add_source(h, &src, nullptr));
  }
  // n update_fields steps: exchange E, B/2, then per step exchange B, E,
  // exchange E, B (the trailing and leading B halves of consecutive steps in
  // one sweep).  The FP32-arithmetic forms leave the last step's trailing
  // half pending, as a whole-grid handle does, and the next call's first
  // sweep applies it with that call's leading half.  Fused: an exchange,
  // then per step one fused sweep and an exchange.
  void step(int64_t n) {
    if (n <= 0) return;
    if (fused_) {
      exchange(FDTD_HALO_STEP);
      for (int64_t s = 0; s < n; ++s) {
        sweep(FDTD_SWEEP_STEP);
        exchange(FDTD_HALO_STEP);
      }
      pending_ = true;
      return;
    }
    exchange(FDTD_HALO_E);
    sweep(pending_ ? FDTD_SWEEP_B_DOUBLE : FDTD_SWEEP_B_HALF);
    for (int64_t s = 0; s < n; ++s) {
      exchange(FDTD_HALO_B);
      sweep(FDTD_SWEEP_E);
      exchange(FDTD_HALO_E);
      sweep(s + 1 < n ? FDTD_SWEEP_B_DOUBLE : (defer_ ? FDTD_SWEEP_B_DEFER : FDTD_SWEEP_B_HALF));
    }
    pending_ = defer_;
  }
  void fence() {
    for (fdtd_handle* h : slabs_) check(fdtd_synchronize(h));
  }
  // Whole-grid copies (Ni*Nj*Nk values, flat index i + j*Ni + k*Ni*Nj).
  void copy_field_to_host(Component c, double* host) const {
    const std::size_t plane = static_cast<std::size_t>(parameters_.Ni) * parameters_.Nj;
    for (std::size_t s = 0; s < slabs_.size(); ++s)
      check(fdtd_copy_field_to_host(slabs_[s], static_cast<int>(c), host + plane * bounds_[s].first,
                                    plane * (bounds_[s].second - bounds_[s].first)));
  }
  void copy_field_from_host(Component c, const double* host) {
    const std::size_t plane = static_cast<std::size_t>(parameters_.Ni) * parameters_.Nj;
    for (std::size_t s = 0; s < slabs_.size(); ++s)
      check(fdtd_copy_field_from_host(slabs_[s], static_cast<int>(c), host + plane * bounds_[s].first,
                                      plane * (bounds_[s].second - bounds_[s].first)));
    if (static_cast<int>(c) < FDTD_JX) pending_ = false;  // each slab applied its pending half first
  }
  const Parameters& parameters() const { return parameters_; }

 private:
  void exchange(int halo) { check(fdtd_slab_exchange(slabs_.data(), size(), halo)); }
  void sweep(int kind) {
    for (fdtd_handle* h : slabs_) check(fdtd_slab_sweep(h, kind));
  }
  void release() {
    for (fdtd_handle* h : slabs_) fdtd_destroy(h);
    slabs_.clear();
  }
  Parameters parameters_;
  bool defer_;            // leave the last trailing B half pending (not FP64)
  bool fused_;            // one fused sweep per step (FP32-arithmetic forms)
  bool pending_ = false;  // a trailing B half step is pending on every slab
  std::vector<fdtd_handle*> slabs_;
  std::vector<std::pair<int, int>> bounds_;
};

}  // namespace FDTD_gb300
