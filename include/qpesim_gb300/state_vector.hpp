// state_vector.hpp - drop-in replacement of the reference header of the same name
// (cpp/state_vector.hpp). StateVector keeps its layout and constructor
// (:16-42: 2^precision blocks of C(M, e)^2 complex doubles, std::vector-backed);
// qift() (:115-179) and IdentifyPhaseAmplitudes() (:341-372) run on the GPU
// through include/qpe_gb300.h. The test-only gate methods of the reference
// (apply_gate, apply_controlled_gate, :51-113) are not part of the hot path and
// are not provided.
#ifndef STATE_VECTOR_HPP_
#define STATE_VECTOR_HPP_

#include <cassert>
#include <complex>
#include <cstdint>
#include <iostream>
#include <vector>

#include "qpe_gb300.h"
#include "util.hpp"

namespace qpesim_gb300 {
inline qpe_context* default_context();
}

class StateVector : public std::vector<std::complex<double>> {
 public:
  StateVector(unsigned precision, unsigned num_orbitals, unsigned num_occupied)
      : precision{precision}, num_orbitals_{num_orbitals}, num_occupied_{num_occupied} {
    assert(num_occupied <= num_orbitals);
    assert(precision > 0);
    n_choose_o_ = nChoosek(num_orbitals, num_occupied);
    resize((1ul << precision) * n_choose_o_ * n_choose_o_, 0);
  }

  void qift() {
    int rc = qpe_qift(qpesim_gb300::default_context(), precision, n_choose_o_ * n_choose_o_,
                      reinterpret_cast<double*>(data()));
    if (rc != QPE_OK) throw qpe_last_error();
  }

  std::vector<double> IdentifyPhaseAmplitudes() {
    std::vector<double> probs(1ul << precision, 0.0);
    int rc = qpe_identify_phase_amplitudes(qpesim_gb300::default_context(), precision, n_choose_o_ * n_choose_o_,
                                           reinterpret_cast<const double*>(data()), probs.data());
    if (rc != QPE_OK) throw qpe_last_error();
    return probs;
  }

 protected:
  unsigned precision;
  unsigned num_orbitals_;
  unsigned num_occupied_;
  uint64_t n_choose_o_;
};

namespace qpesim_gb300 {
inline qpe_context* default_context() {
  static qpe_context* ctx = [] {
    qpe_context* c = nullptr;
    if (qpe_context_create(0, &c) != QPE_OK) throw qpe_last_error();
    return c;
  }();
  return ctx;
}
}  // namespace qpesim_gb300

#endif  // STATE_VECTOR_HPP_
