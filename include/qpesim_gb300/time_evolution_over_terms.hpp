// time_evolution_over_terms.hpp - drop-in replacement of the reference header of
// the same name (cpp/time_evolution_over_terms.hpp). It keeps the entry point
//   std::complex<double> time_evolve_over_terms(StateVector&, Hamiltonian&, unsigned precision)
// (:92) and forwards it to the GB300 library (include/qpe_gb300.h): the terms come
// from the caller's Hamiltonian exactly as the reference reads them
// (PrintIndexedSegmentedHamiltonianTerms and the *_term coefficient getters, at
// the Hamiltonian's timestep), and the library applies them in the order of
// applyUnitary_reordered (:374-562) to every controlled power on the GPU. The
// iterative variant time_evolve_iqpe (:141-155) is forwarded the same way.
// A failing call throws a const char* with the library's message, the way the
// reference reports errors.
//
// Use: put this directory's files in place of the reference's
// time_evolution_over_terms.hpp and state_vector.hpp, and link libqpe_gb300.so.
#ifndef TIME_EVOLUTION_MANUAL_HPP
#define TIME_EVOLUTION_MANUAL_HPP

#include <complex>
#include <tuple>
#include <vector>

#include "hamiltonian.hpp"
#include "qpe_gb300.h"
#include "state_vector.hpp"

namespace qpesim_gb300 {

inline void put_matrix(const std::array<std::complex<double>, 4>& m, double* d) {
  d[0] = m[0].real();
  d[1] = m[0].imag();
  d[2] = m[1].real();
  d[3] = m[1].imag();
}

// The five segments with their exponentiated coefficients.
struct SegmentedTerms {
  std::vector<qpe_term> seg[5];
};

inline SegmentedTerms collect_terms(Hamiltonian& h) {
  SegmentedTerms out;
  IdxSingleVec pp, pq;
  IdxDoubleVec pqqp, pqqr, pqrs;
  std::tie(pp, pq, pqqp, pqqr, pqrs) = h.PrintIndexedSegmentedHamiltonianTerms();
  for (const auto& t : pp) {
    qpe_term x{};
    x.p = x.q = t.first.first;
    std::complex<double> c = h.pp_term(x.p);
    x.even[0] = c.real();
    x.even[1] = c.imag();
    out.seg[QPE_TERM_PP].push_back(x);
  }
  for (const auto& t : pq) {
    qpe_term x{};
    x.p = t.first.first;
    x.q = t.first.second;
    put_matrix(h.pq_term(x.p, x.q, 0), x.even);
    put_matrix(h.pq_term(x.p, x.q, 1), x.odd);
    out.seg[QPE_TERM_PQ].push_back(x);
  }
  for (const auto& t : pqqp) {
    qpe_term x{};
    std::tie(x.p, x.q, x.r, x.s) = t.first;
    std::complex<double> c = h.pqqp_term(x.p, x.q);
    x.even[0] = c.real();
    x.even[1] = c.imag();
    out.seg[QPE_TERM_PQQP].push_back(x);
  }
  for (const auto& t : pqqr) {
    qpe_term x{};
    std::tie(x.p, x.q, x.r, x.s) = t.first;
    put_matrix(h.pqqr_term(x.p, x.q, x.s, 0), x.even);
    put_matrix(h.pqqr_term(x.p, x.q, x.s, 1), x.odd);
    out.seg[QPE_TERM_PQQR].push_back(x);
  }
  for (const auto& t : pqrs) {
    qpe_term x{};
    std::tie(x.p, x.q, x.r, x.s) = t.first;
    put_matrix(h.pqrs_term(x.p, x.q, x.r, x.s, 0), x.even);
    put_matrix(h.pqrs_term(x.p, x.q, x.r, x.s, 1), x.odd);
    out.seg[QPE_TERM_PQRS].push_back(x);
  }
  return out;
}

}  // namespace qpesim_gb300

inline std::complex<double> time_evolve_over_terms(StateVector& state_vector, Hamiltonian& hamiltonian,
                                                   unsigned precision) {
  qpesim_gb300::SegmentedTerms T = qpesim_gb300::collect_terms(hamiltonian);
  auto ptr = [&](int k) { return T.seg[k].empty() ? nullptr : T.seg[k].data(); };
  int rc = qpe_time_evolve_over_terms(
      qpesim_gb300::default_context(), hamiltonian.num_orbitals(), hamiltonian.num_occupied(), precision,
      ptr(QPE_TERM_PP), T.seg[QPE_TERM_PP].size(), ptr(QPE_TERM_PQ), T.seg[QPE_TERM_PQ].size(), ptr(QPE_TERM_PQQP),
      T.seg[QPE_TERM_PQQP].size(), ptr(QPE_TERM_PQQR), T.seg[QPE_TERM_PQQR].size(), ptr(QPE_TERM_PQRS),
      T.seg[QPE_TERM_PQRS].size(), reinterpret_cast<double*>(state_vector.data()));
  if (rc != QPE_OK) throw qpe_last_error();
  return std::complex<double>();
}

// time_evolve_iqpe (:141-155): block 1 evolved in place, num_of_applications
// sweeps in applyUnitary's term order (:174-372).
inline void time_evolve_iqpe(StateVector& state_vector, Hamiltonian& hamiltonian, unsigned num_of_applications) {
  qpesim_gb300::SegmentedTerms T = qpesim_gb300::collect_terms(hamiltonian);
  auto ptr = [&](int k) { return T.seg[k].empty() ? nullptr : T.seg[k].data(); };
  // The register's precision from its size: 2^precision blocks of C(M, e)^2.
  uint64_t c = 1;
  for (unsigned i = 1; i <= hamiltonian.num_occupied(); ++i)
    c = c * (hamiltonian.num_orbitals() - hamiltonian.num_occupied() + i) / i;
  unsigned precision = 0;
  while ((c * c << (precision + 1)) <= state_vector.size()) ++precision;
  int rc = qpe_time_evolve_iqpe(
      qpesim_gb300::default_context(), hamiltonian.num_orbitals(), hamiltonian.num_occupied(), precision,
      ptr(QPE_TERM_PP), T.seg[QPE_TERM_PP].size(), ptr(QPE_TERM_PQ), T.seg[QPE_TERM_PQ].size(), ptr(QPE_TERM_PQQP), T.seg[QPE_TERM_PQQP].size(), ptr(QPE_TERM_PQQR),
      T.seg[QPE_TERM_PQQR].size(), ptr(QPE_TERM_PQRS), T.seg[QPE_TERM_PQRS].size(), num_of_applications,
      reinterpret_cast<double*>(state_vector.data()));
  if (rc != QPE_OK) throw qpe_last_error();
}

#endif  // TIME_EVOLUTION_MANUAL_HPP
