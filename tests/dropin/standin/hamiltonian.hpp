// hamiltonian.hpp (test stand-in) - a Hamiltonian class with the interface of the
// reference's (cpp/hamiltonian.hpp:24-184) that the drop-in headers and the
// drop-in driver call, backed by the library's own term compiler
// (include/qpe_gb300_hamiltonian.h). It lets the drop-in headers
// (include/qpesim_gb300/) be built and run where the reference sources are not
// present, such as a GPU host; where they are, the same driver is built against
// the reference's own hamiltonian.cc instead. Errors are thrown as const char*,
// the way the reference reports them.
#ifndef QPE_DROPIN_STANDIN_HAMILTONIAN_HPP_
#define QPE_DROPIN_STANDIN_HAMILTONIAN_HPP_

#include <array>
#include <complex>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "qpe_gb300.h"
#include "qpe_gb300_hamiltonian.h"
#include "state_vector.hpp"

enum class SpinIndex { HalfUp };

// Term lists as PrintIndexedSegmentedHamiltonianTerms returns them: the
// spin-orbital indices and the indexed integral value of each term.
using IdxSingleVec = std::vector<std::pair<std::pair<unsigned, unsigned>, double>>;
using IdxDoubleVec = std::vector<std::pair<std::tuple<unsigned, unsigned, unsigned, unsigned>, double>>;

class Hamiltonian {
 public:
  Hamiltonian() { check(qpe_ham_create(&h_)); }
  Hamiltonian(const Hamiltonian&) = delete;
  Hamiltonian& operator=(const Hamiltonian&) = delete;
  Hamiltonian(Hamiltonian&& o) noexcept : h_(o.h_) { o.h_ = nullptr; }
  ~Hamiltonian() {
    if (h_) qpe_ham_destroy(h_);
  }

  // Reads the file's integrals, identity, sizes and initial state (block 0 of a
  // 2^precision register, unscaled).
  StateVector IngestBroombridge(const std::string& path, unsigned precision) {
    uint32_t M = 0, e = 0;
    {
      qpe_hamiltonian* probe = nullptr;  // sizes first, so that block 0 fits
      check(qpe_ham_create(&probe));
      const int rc = qpe_ham_ingest_broombridge(probe, path.c_str(), &M, &e, nullptr, 0);
      qpe_ham_destroy(probe);
      check(rc);
    }
    StateVector sv(precision, M, e);
    const uint64_t c = nChoosek(M, e);
    check(qpe_ham_ingest_broombridge(h_, path.c_str(), &M, &e, reinterpret_cast<double*>(sv.data()), c * c));
    return sv;
  }

  void IndexTerms(SpinIndex = SpinIndex::HalfUp) { check(qpe_ham_index_terms(h_)); }
  void SetTimestep(double t) { check(qpe_ham_set_timestep(h_, t)); }
  unsigned num_orbitals() const {
    uint32_t v = 0;
    check(qpe_ham_get_num_orbitals(h_, &v));
    return v;
  }
  unsigned num_occupied() const {
    uint32_t v = 0;
    check(qpe_ham_get_num_occupied(h_, &v));
    return v;
  }

  std::tuple<IdxSingleVec, IdxSingleVec, IdxDoubleVec, IdxDoubleVec, IdxDoubleVec>
  PrintIndexedSegmentedHamiltonianTerms() const {
    size_t counts[5] = {};
    check(qpe_ham_segment_counts(h_, counts));
    IdxSingleVec pp, pq;
    IdxDoubleVec pqqp, pqqr, pqrs;
    for (int k = 0; k < 5; ++k) {
      std::vector<qpe_term> t(counts[k]);
      std::vector<double> raw(counts[k]);
      if (counts[k]) check(qpe_ham_segment_terms(h_, k, t.data(), raw.data(), counts[k]));
      for (size_t i = 0; i < counts[k]; ++i) {
        if (k == QPE_TERM_PP || k == QPE_TERM_PQ)
          (k == QPE_TERM_PP ? pp : pq).push_back({{t[i].p, t[i].q}, raw[i]});
        else
          (k == QPE_TERM_PQQP ? pqqp : (k == QPE_TERM_PQQR ? pqqr : pqrs))
              .push_back({std::make_tuple(t[i].p, t[i].q, t[i].r, t[i].s), raw[i]});
      }
    }
    return std::make_tuple(pp, pq, pqqp, pqqr, pqrs);
  }

  std::complex<double> pp_term(unsigned p) const {
    double o[2];
    check(qpe_ham_pp_term(h_, p, o));
    return {o[0], o[1]};
  }
  std::complex<double> pqqp_term(unsigned p, unsigned q) const {
    double o[2];
    check(qpe_ham_pqqp_term(h_, p, q, o));
    return {o[0], o[1]};
  }
  std::array<std::complex<double>, 4> pq_term(unsigned p, unsigned q, unsigned parity) const {
    double o[8];
    check(qpe_ham_pq_term(h_, p, q, parity, o));
    return matrix(o);
  }
  std::array<std::complex<double>, 4> pqqr_term(unsigned p, unsigned q, unsigned r, unsigned parity) const {
    double o[8];
    check(qpe_ham_pqqr_term(h_, p, q, r, parity, o));
    return matrix(o);
  }
  std::array<std::complex<double>, 4> pqrs_term(unsigned p, unsigned q, unsigned r, unsigned s,
                                                 unsigned parity) const {
    double o[8];
    check(qpe_ham_pqrs_term(h_, p, q, r, s, parity, o));
    return matrix(o);
  }

 private:
  static void check(int rc) {
    if (rc != QPE_OK) throw qpe_last_error();
  }
  static std::array<std::complex<double>, 4> matrix(const double* o) {
    return {std::complex<double>(o[0], o[1]), std::complex<double>(o[2], o[3]), std::complex<double>(o[4], o[5]),
            std::complex<double>(o[6], o[7])};
  }
  qpe_hamiltonian* h_ = nullptr;
};

#endif  // QPE_DROPIN_STANDIN_HAMILTONIAN_HPP_
