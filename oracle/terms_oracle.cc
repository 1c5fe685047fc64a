// terms_oracle.cc - TEST INFRASTRUCTURE ONLY: a CPU restatement of the
// reference's Hamiltonian term compiler (cpp/hamiltonian.cc), so that the oracle
// can turn integrals into the five segmented, exponentiated term lists on its
// own, without the product library. Only tests/ and bench.py's CPU-baseline leg
// use it, as the checker; nothing in the product links it.
//
// Pinned by tests/test_oracle_golden.py against the term lists the reference
// itself produced (tests/golden/terms_*.npz) and against the product's compiler.
//
// Data model: a spin orbital is packed into one int, spin * kSpinStride +
// orbital (1-based), so that integer order is the reference's SpinOrbital order
// (spin first, Up < Down, then orbital; cpp/types.hpp:66-78). The term maps are
// keyed by arrays of packed ints, which order lexicographically like the
// reference's std::pair / std::tuple keys, so iteration order and the order in
// which contributions are summed into each key are the reference's.
#include <array>
#include <cmath>
#include <complex>
#include <map>
#include <set>
#include <utility>
#include <vector>

#include "../include/qpe_gb300.h"

namespace orc_terms {

constexpr int kSpinStride = 1 << 12;  // orbitals are below this
inline int so(int orbital, int spin) { return spin * kSpinStride + orbital; }
inline int spin_of(int x) { return x / kSpinStride; }
inline int orb_of(int x) { return x % kSpinStride; }

using Key2 = std::array<int, 2>;
using Key4 = std::array<int, 4>;

struct Compiler {
  unsigned M = 0, occupied = 0;
  double t = 0.0;
  std::map<Key2, double> one;   // one_body_terms (cpp/hamiltonian.hpp:153)
  std::map<Key4, double> two;   // two_body_terms (:154)
  std::map<std::array<unsigned, 2>, double> ione;  // indexed_one_body_terms (:175)
  std::map<std::array<unsigned, 4>, double> itwo;  // indexed_two_body_terms (:176)
  bool bad = false;

  // _UpdateDataModel_OneBody / _TwoBody (cpp/hamiltonian.cc:623-657): zero deltas
  // are dropped; a key's value starts at 0.0 and accumulates in call order.
  void add1(const Key2& k, double d) {
    if (d == 0) return;
    double& v = one[k];
    v = v + d;
  }
  void add2(const Key4& k, double d) {
    if (d == 0) return;
    double& v = two[k];
    v = v + d;
  }

  // AddOneBodyTerm (:301-323) with _EnumerateSpinOrbitals_OneBody (:421-438).
  void add_one_body(int p, int q, double c) {
    if (c == 0) return;
    for (int s = 0; s < 2; ++s) add1({so(p, s), so(q, s)}, c);
  }

  // _ReorderPQQPTerm (:467-496). Returns false for the dropped PPQQ shapes.
  static bool reorder_pqqp(Key4& k, double& c) {
    int &p = k[0], &q = k[1], &r = k[2], &s = k[3];
    if (r == s || p == q) return false;
    c = c / 2.0;
    if (p == r) {
      std::swap(r, s);
      c *= -1.0;
    }
    if (!(p < q)) {
      std::swap(p, q);
      std::swap(r, s);
    }
    return true;
  }

  // _ReorderPQQRTerm (:498-545).
  bool reorder_pqqr(Key4& k, double& c) {
    int &p = k[0], &q = k[1], &r = k[2], &s = k[3];
    if (p == q || r == s) return false;
    c = c / 4.0;
    if (q == r) {
    } else if (q == s) {
      c *= -1.0;
      std::swap(r, s);
    } else if (p == r) {
      c *= -1.0;
      std::swap(p, q);
    } else if (p == s) {
      std::swap(p, q);
      std::swap(r, s);
    } else {
      bad = true;  // the reference throws "Unknown PQQR term"
      return false;
    }
    if (s < p) std::swap(p, s);
    return true;
  }

  // _ReorderPQRSTerm (:547-619).
  static bool reorder_pqrs(Key4& k, double& c) {
    int &p = k[0], &q = k[1], &r = k[2], &s = k[3];
    const int alphas = (spin_of(p) == 0) + (spin_of(q) == 0) + (spin_of(r) == 0) + (spin_of(s) == 0);
    c = c / 4.0;
    if (!(std::min(p, q) < std::min(r, s))) {
      std::swap(p, r);
      std::swap(q, s);
    }
    if (alphas == 2) {
      if (spin_of(q) == 0) {
        std::swap(p, q);
        c *= -1.0;
      }
      if (spin_of(r) == 0) {
        std::swap(r, s);
        c *= -1.0;
      }
    } else {
      if (orb_of(q) < orb_of(p)) {
        std::swap(p, q);
        c *= -1.0;
      }
      if (orb_of(r) < orb_of(s)) {
        std::swap(r, s);
        c *= -1.0;
      }
    }
    return true;
  }

  // AddTwoBodyTerm (:325-398): the PPPP shortcut, else the 8-fold permutation
  // set (:400-417, visited in set order), each with the spin assignments
  // (inner spin on q, r, outer on p, s; inner loop outermost, :440-463), each
  // reordered by its number of distinct spin orbitals.
  void add_two_body(int p, int q, int r, int s, double c) {
    if (c == 0) return;
    if (p == q && q == r && r == s) {
      add2({so(p, 0), so(p, 1), so(p, 1), so(p, 0)}, c);
      return;
    }
    const std::set<std::array<int, 4>> perms = {{p, q, r, s}, {s, q, r, p}, {p, r, q, s}, {s, r, q, p},
                                                {q, p, s, r}, {r, p, s, q}, {q, s, p, r}, {r, s, p, q}};
    for (const auto& x : perms) {
      for (int inner = 0; inner < 2; ++inner) {
        for (int outer = 0; outer < 2; ++outer) {
          Key4 k = {so(x[0], outer), so(x[1], inner), so(x[2], inner), so(x[3], outer)};
          const std::set<int> distinct(k.begin(), k.end());
          double cc = c;
          bool keep = false;
          if (distinct.size() == 2)
            keep = reorder_pqqp(k, cc);
          else if (distinct.size() == 3)
            keep = reorder_pqqr(k, cc);
          else if (distinct.size() == 4)
            keep = reorder_pqrs(k, cc);
          else
            bad = true;
          if (keep) add2(k, cc);
        }
      }
    }
  }

  // IndexTerms(HalfUp) (:160-197): spin * M + orbital - 1.
  void index_terms() {
    auto idx = [&](int x) { return (unsigned)(spin_of(x) * (int)M + orb_of(x) - 1); };
    for (const auto& kv : one) ione.insert({{idx(kv.first[0]), idx(kv.first[1])}, kv.second});
    for (const auto& kv : two)
      itwo.insert({{idx(kv.first[0]), idx(kv.first[1]), idx(kv.first[2]), idx(kv.first[3])}, kv.second});
  }

  // The coefficient getters (:661-783) at timestep t: exp(-i h t) for the
  // diagonal kinds; {m00, m01} = {cos(h t), -i (-1)^parity sin(h t)} for the pair
  // kinds (1 and 0 where the key has no term).
  std::complex<double> diag(double h) const {
    using namespace std::complex_literals;
    return std::exp(-1i * h * t);
  }
  void pair(double h, bool present, unsigned parity, double* out) const {
    using namespace std::complex_literals;
    std::complex<double> m00, m01;
    if (!present) {
      m00 = std::complex<double>(1.0);
      m01 = std::complex<double>(0.0);
    } else {
      m00 = std::cos(h * t);
      m01 = -1i * static_cast<std::complex<double>>(parity ? -1 : 1) * std::sin(h * t);
    }
    out[0] = m00.real();
    out[1] = m00.imag();
    out[2] = m01.real();
    out[3] = m01.imag();
  }

  // PrintIndexedSegmentedHamiltonianTerms (:253-299): pp and pq from the one-body
  // map; pqqp (q == r, p == s), pqqr (q == r, p != s) and pqrs from the two-body
  // map, each in key order; with the getters' coefficients.
  void segments(std::vector<qpe_term> seg[5], std::vector<double> raw[5]) const {
    for (const auto& kv : ione) {
      qpe_term x{};
      x.p = kv.first[0];
      x.q = kv.first[1];
      const int kind = x.p == x.q ? QPE_TERM_PP : QPE_TERM_PQ;
      if (kind == QPE_TERM_PP) {
        const std::complex<double> c = diag(kv.second);
        x.even[0] = c.real();
        x.even[1] = c.imag();
      } else {
        pair(kv.second, true, 0, x.even);
        pair(kv.second, true, 1, x.odd);
      }
      seg[kind].push_back(x);
      raw[kind].push_back(kv.second);
    }
    for (const auto& kv : itwo) {
      qpe_term x{};
      x.p = kv.first[0];
      x.q = kv.first[1];
      x.r = kv.first[2];
      x.s = kv.first[3];
      int kind;
      if (x.q == x.r) kind = x.p == x.s ? QPE_TERM_PQQP : QPE_TERM_PQQR;
      else kind = QPE_TERM_PQRS;
      if (kind == QPE_TERM_PQQP) {
        const std::complex<double> c = diag(kv.second);
        x.even[0] = c.real();
        x.even[1] = c.imag();
      } else {
        pair(kv.second, true, 0, x.even);
        pair(kv.second, true, 1, x.odd);
      }
      seg[kind].push_back(x);
      raw[kind].push_back(kv.second);
    }
  }
};

}  // namespace orc_terms

using orc_terms::Compiler;

extern "C" {

void* orc_terms_create(void) { return new Compiler(); }
void orc_terms_destroy(void* h) { delete static_cast<Compiler*>(h); }

// Spatial orbital count M (max_number_of_orbitals), electrons per spin and the
// timestep of the getters.
void orc_terms_set(void* h, unsigned M, unsigned occupied, double t) {
  Compiler* c = static_cast<Compiler*>(h);
  c->M = M;
  c->occupied = occupied;
  c->t = t;
}

// AddOneBodyTerm({p, q}, v) and AddTwoBodyTerm({p, q, r, s}, v), 1-based orbitals.
void orc_terms_add_one_body(void* h, int p, int q, double v) { static_cast<Compiler*>(h)->add_one_body(p, q, v); }
void orc_terms_add_two_body(void* h, int p, int q, int r, int s, double v) {
  static_cast<Compiler*>(h)->add_two_body(p, q, r, s, v);
}

// IndexTerms, then the five segments: counts[5], and for each segment k the
// terms into out[k] (capacity caps[k]) and their indexed values into raw[k].
// Returns 0, or 1 if a term had an unknown shape or a capacity is too small.
int orc_terms_segments(void* h, size_t counts[5], qpe_term* const* out, double* const* raw, const size_t* caps) {
  Compiler* c = static_cast<Compiler*>(h);
  if (c->bad) return 1;
  if (c->ione.empty() && c->itwo.empty()) c->index_terms();
  std::vector<qpe_term> seg[5];
  std::vector<double> rv[5];
  c->segments(seg, rv);
  for (int k = 0; k < 5; ++k) {
    counts[k] = seg[k].size();
    if (!out || !out[k]) continue;
    if (seg[k].size() > caps[k]) return 1;
    for (size_t i = 0; i < seg[k].size(); ++i) {
      out[k][i] = seg[k][i];
      if (raw && raw[k]) raw[k][i] = rv[k][i];
    }
  }
  return 0;
}

}  // extern "C"
