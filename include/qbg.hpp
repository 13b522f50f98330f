/*
 * qbg.hpp -- header-only C++17 layer over the C ABI of qbg.h for C++ hosts
 * (the reference is a C++ program).  It owns plans and operator pairs with
 * RAII, turns status codes into exceptions carrying the status and the
 * library's message, and gives the ETRS forward/backward operator pair a C++
 * interface:
 *
 *   qbg::Basis basis(cell, ecut);                   // Basis::resize
 *   qbg::Plan plan(basis, 120, 120, 120, QBG_PREC_MIXED_DF32);
 *   plan.set_vlocal(v_r); plan.set_nonlocal(...);
 *   qbg::TDPropagation td(plan, ld, nst, occ, dt, nsteps, K);
 *   std::vector<double> J = td.forward(psi_dev, A);          // (nsteps+1) x 3
 *   std::vector<double> ga = td.backward(dLdJ, e, grad_v_dev); // nsteps+1
 *
 * Device arrays stay raw pointers (the caller owns its memory, as qball owns
 * its SlaterDet blocks); host arrays are std::vector.  No state beyond the
 * C handles lives here.
 */
#ifndef QBG_HPP
#define QBG_HPP

#include <array>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "qbg.h"

namespace qbg {

class Error : public std::runtime_error {
 public:
  Error(qbg_status s, const std::string& what)
      : std::runtime_error(what + ": " + (qbg_last_error() ? qbg_last_error() : "")),
        status_(s) {}
  qbg_status status() const { return status_; }

 private:
  qbg_status status_;
};

inline void check(qbg_status s, const char* what) {
  if (s != QBG_OK) throw Error(s, what);
}

// Full-sphere basis at k = 0 (Basis::resize) in the reference's rod order.
struct Basis {
  std::array<double, 9> cell{};
  double ecut = 0.0;
  double omega = 0.0;
  int ngw = 0, nrods = 0;
  std::array<int, 3> np{};
  std::vector<int> rod_h, rod_k, rod_lmin, rod_size;
  std::vector<double> kpg2, kpgx;

  Basis(const std::array<double, 9>& a, double ecut_ha) : cell(a), ecut(ecut_ha) {
    int info[12] = {0};
    check(qbg_basis_dims(cell.data(), ecut, info), "qbg_basis_dims");
    ngw = info[0];
    nrods = info[1];
    np = {info[2], info[3], info[4]};
    rod_h.resize(nrods);
    rod_k.resize(nrods);
    rod_lmin.resize(nrods);
    rod_size.resize(nrods);
    kpg2.resize(ngw);
    kpgx.resize(3 * (size_t)ngw);
    check(qbg_basis_fill(cell.data(), ecut, rod_h.data(), rod_k.data(), rod_lmin.data(),
                         rod_size.data(), nullptr, kpg2.data(), kpgx.data()),
          "qbg_basis_fill");
    const double* a0 = &cell[0];
    const double* a1 = &cell[3];
    const double* a2 = &cell[6];
    const double cx = a1[1] * a2[2] - a1[2] * a2[1];
    const double cy = a1[2] * a2[0] - a1[0] * a2[2];
    const double cz = a1[0] * a2[1] - a1[1] * a2[0];
    omega = a0[0] * cx + a0[1] * cy + a0[2] * cz;
    if (omega < 0) omega = -omega;
  }

  qbg_basis_desc desc() const {
    qbg_basis_desc d;
    d.ngw = ngw;
    d.nrods = nrods;
    d.rod_h = rod_h.data();
    d.rod_k = rod_k.data();
    d.rod_lmin = rod_lmin.data();
    d.rod_size = rod_size.data();
    d.kpgx = kpgx.data();
    d.omega = omega;
    return d;
  }
};

// FourierTransform + the Hamiltonian operators of one system (qbg_plan).
class Plan {
 public:
  Plan(const Basis& b, int np0, int np1, int np2, int precision = QBG_PREC_FP64)
      : ngw_(b.ngw), n_((long long)np0 * np1 * np2) {
    const qbg_basis_desc d = b.desc();
    check(qbg_plan_create(&d, np0, np1, np2, precision, &h_), "qbg_plan_create");
  }
  ~Plan() {
    if (h_) qbg_plan_destroy(h_);
  }
  Plan(const Plan&) = delete;
  Plan& operator=(const Plan&) = delete;
  Plan(Plan&& o) noexcept : h_(std::exchange(o.h_, nullptr)), ngw_(o.ngw_), n_(o.n_) {}
  Plan& operator=(Plan&& o) noexcept {
    if (this != &o) {
      if (h_) qbg_plan_destroy(h_);
      h_ = std::exchange(o.h_, nullptr);
      ngw_ = o.ngw_;
      n_ = o.n_;
    }
    return *this;
  }

  qbg_plan* get() const { return h_; }
  int ngw() const { return ngw_; }
  long long grid_points() const { return n_; }

  void set_chunk(int n) { check(qbg_plan_set_chunk(h_, n), "qbg_plan_set_chunk"); }
  void set_vlocal(const double* v_r) { check(qbg_set_vlocal(h_, v_r), "qbg_set_vlocal"); }
  void set_nonlocal(const std::vector<int>& na, const std::vector<int>& lmax,
                    const std::vector<double>& rc, const std::vector<double>& wt,
                    const std::vector<double>& tau) {
    check(qbg_set_nonlocal(h_, (int)na.size(), na.data(), lmax.data(), rc.data(), wt.data(),
                           tau.data()),
          "qbg_set_nonlocal");
  }
  // Real pseudopotential projector tables (NonLocalPotential::update_twnl's
  // arrays, species after species; see qbg_set_nonlocal_tables)
  void set_nonlocal_tables(const std::vector<int>& na, const std::vector<int>& npr,
                           const std::vector<int>& lproj, const std::vector<double>& wt,
                           const std::vector<double>& twnl, const std::vector<double>& tau) {
    check(qbg_set_nonlocal_tables(h_, (int)na.size(), na.data(), npr.data(), lproj.data(),
                                  wt.data(), twnl.data(), tau.data()),
          "qbg_set_nonlocal_tables");
  }
  // projector GEMMs of the plain FP64 form: QBG_GEMM_OZAKI (slices 6 or 7) or
  // QBG_GEMM_SIMT
  void set_fp64_gemm(int mode, int slices = 7) {
    check(qbg_plan_set_fp64_gemm(h_, mode, slices), "qbg_plan_set_fp64_gemm");
  }
  void set_vector_potential(const std::array<double, 3>& A) {
    check(qbg_set_vector_potential(h_, A.data()), "qbg_set_vector_potential");
  }
  void backward(const double* c, int ldc, double* f, int nbatch, void* stream = nullptr) {
    check(qbg_backward(h_, c, ldc, f, nbatch, stream), "qbg_backward");
  }
  void forward(double* f, double* c, int ldc, int nbatch, void* stream = nullptr) {
    check(qbg_forward(h_, f, c, ldc, nbatch, stream), "qbg_forward");
  }
  // H psi; returns E_nl when occ is given (synchronises), else 0
  double hpsi(const double* psi, int ld, double* out, int nst, const double* occ = nullptr,
              void* stream = nullptr) {
    double enl = 0.0;
    check(qbg_hpsi(h_, psi, ld, out, nst, occ, occ ? &enl : nullptr, stream), "qbg_hpsi");
    return enl;
  }
  // rho(r) (device, N doubles); returns the electron count (synchronises)
  double density(const double* psi, int ld, int nst, const double* occ, double* rho,
                 double weight = 1.0, void* stream = nullptr) {
    double nel = 0.0;
    check(qbg_density(h_, psi, ld, nst, occ, weight, rho, &nel, stream), "qbg_density");
    return nel;
  }
  std::array<double, 3> current(const double* psi, int ld, int nst, const double* occ,
                                double nel, void* stream = nullptr) {
    std::array<double, 3> J{};
    check(qbg_current(h_, psi, ld, nst, occ, nel, J.data(), stream), "qbg_current");
    return J;
  }
  void etrs_step(double* psi, int ld, int nst, const double* occ, double dt,
                 const double* A_t = nullptr, const double* A_tdt = nullptr,
                 void* stream = nullptr) {
    check(qbg_etrs_step(h_, psi, ld, nst, occ, dt, A_t, A_tdt, nullptr, nullptr, stream),
          "qbg_etrs_step");
  }

 private:
  qbg_plan* h_ = nullptr;
  int ngw_ = 0;
  long long n_ = 0;
};

// Checkpointed forward/backward operator pair over nsteps fixed-potential
// ETRS steps (qbg_td_*).
class TDPropagation {
 public:
  TDPropagation(Plan& plan, int ld, int nst, const std::vector<double>& occ, double dt,
                int nsteps, int K)
      : nsteps_(nsteps) {
    if ((int)occ.size() < nst) throw std::invalid_argument("TDPropagation: occ has < nst entries");
    check(qbg_td_create(plan.get(), ld, nst, occ.data(), dt, nsteps, K, &h_), "qbg_td_create");
  }
  ~TDPropagation() {
    if (h_) qbg_td_destroy(h_);
  }
  TDPropagation(const TDPropagation&) = delete;
  TDPropagation& operator=(const TDPropagation&) = delete;

  // psi (device) advanced in place; A: (nsteps+1) x 3; returns J: (nsteps+1) x 3
  std::vector<double> forward(double* psi, const std::vector<double>& A,
                              void* stream = nullptr) {
    if (A.size() != 3 * (size_t)(nsteps_ + 1))
      throw std::invalid_argument("TDPropagation::forward: A must hold (nsteps+1) x 3 values");
    std::vector<double> J(3 * (size_t)(nsteps_ + 1));
    check(qbg_td_forward(h_, psi, A.data(), J.data(), stream), "qbg_td_forward");
    return J;
  }
  // dL/da_n along e (nsteps+1 values); grad_v (device, N doubles) and
  // lambda0 (device [ld x nst]) are written when non-null
  std::vector<double> backward(const std::vector<double>& dLdJ, const std::array<double, 3>& e,
                               double* grad_v = nullptr, double* lambda0 = nullptr,
                               void* stream = nullptr) {
    if (dLdJ.size() != 3 * (size_t)(nsteps_ + 1))
      throw std::invalid_argument("TDPropagation::backward: dLdJ must hold (nsteps+1) x 3 values");
    std::vector<double> ga((size_t)nsteps_ + 1);
    check(qbg_td_backward(h_, dLdJ.data(), e.data(), grad_v, ga.data(), lambda0, stream),
          "qbg_td_backward");
    return ga;
  }

 private:
  qbg_td* h_ = nullptr;
  int nsteps_ = 0;
};

}  // namespace qbg

#endif  // QBG_HPP
