// hamiltonian.cpp - host-side Hamiltonian term compiler (the producer side of the
// boundary). It follows the reference's Hamiltonian class (cpp/hamiltonian.hpp,
// cpp/hamiltonian.cc) step for step: the same data model (ordered maps keyed by
// spin orbitals, then by HalfUp indices), the same accumulation order and the same
// coefficient expressions, so the term lists and coefficients it hands to the
// device program are the ones the reference would compute.
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <regex>
#include <map>
#include <new>
#include <set>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/qpe_gb300_hamiltonian.h"
#include "qpe_common.h"
#include "yaml_subset.h"

namespace qpe {

static uint64_t binom_exact(int n, int k) {
  if (k < 0 || n < 0 || k > n) return 0;
  if (k * 2 > n) k = n - k;
  uint64_t r = 1;
  for (int i = 1; i <= k; ++i) r = r * (uint64_t)(n - k + i) / (uint64_t)i;
  return r;
}

// SpinOrbital (cpp/types.hpp:33-98): ordered by spin (Up < Down), then orbital.
struct SpinOrb {
  int orbital = 0;
  int spin = 0;  // 0 = Up (alpha), 1 = Down (beta)
  bool operator<(const SpinOrb& t) const {
    if (t.spin != spin) return spin < t.spin;
    return orbital < t.orbital;
  }
  bool operator==(const SpinOrb& t) const { return orbital == t.orbital && spin == t.spin; }
  bool operator!=(const SpinOrb& t) const { return !(*this == t); }
  // ConvertToInt(HalfUp, M) (cpp/types.hpp:50-55).
  int half_up(int M) const { return spin * M + orbital - 1; }
};

using OneKey = std::pair<SpinOrb, SpinOrb>;
using TwoKey = std::tuple<SpinOrb, SpinOrb, SpinOrb, SpinOrb>;

struct Hamiltonian {
  double identity = 0.0;
  unsigned num_orbitals = 0;
  unsigned num_occupied = 0;
  double t = 0.0;
  std::map<OneKey, double> one_body;
  std::map<TwoKey, double> two_body;
  std::map<std::pair<unsigned, unsigned>, double> idx_one;
  std::map<std::tuple<unsigned, unsigned, unsigned, unsigned>, double> idx_two;

  // _UpdateDataModel_OneBody / _TwoBody (cpp/hamiltonian.cc:623-657).
  void update_one(const OneKey& k, double delta) {
    if (delta == 0) return;
    double existing = one_body[k];
    one_body[k] = existing + delta;
  }
  void update_two(const TwoKey& k, double delta) {
    if (delta == 0) return;
    double existing = two_body[k];
    two_body[k] = existing + delta;
  }

  // AddOneBodyTerm (:301-323) with _EnumerateSpinOrbitals_OneBody (:421-438).
  void add_one(int p, int q, double coeff) {
    if (coeff == 0) return;
    for (int spin = 0; spin < 2; ++spin) update_one(OneKey{SpinOrb{p, spin}, SpinOrb{q, spin}}, coeff);
  }

  // _ReorderPQQPTerm (:467-499).
  static bool reorder_pqqp(TwoKey& k, double& coeff) {
    SpinOrb p, q, r, s;
    std::tie(p, q, r, s) = k;
    if (r == s || p == q) return false;
    double c = coeff / 2.0;
    if (p == r) {
      std::swap(r, s);
      c *= -1.0;
    }
    if (!(p < q)) {
      std::swap(p, q);
      std::swap(r, s);
    }
    k = TwoKey{p, q, r, s};
    coeff = c;
    return true;
  }

  // _ReorderPQQRTerm (:501-548).
  static bool reorder_pqqr(TwoKey& k, double& coeff) {
    SpinOrb p, q, r, s;
    std::tie(p, q, r, s) = k;
    if (p == q || r == s) return false;
    double c = coeff / 4.0;
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
      throw Error(QPE_ERR_INVALID, "unknown pqqr term shape");
    }
    if (s < p) std::swap(p, s);
    k = TwoKey{p, q, r, s};
    coeff = c;
    return true;
  }

  // _ReorderPQRSTerm (:550-619).
  static void reorder_pqrs(TwoKey& k, double& coeff) {
    SpinOrb p, q, r, s;
    std::tie(p, q, r, s) = k;
    unsigned alphas = (p.spin == 0) + (q.spin == 0) + (r.spin == 0) + (s.spin == 0);
    double c = coeff / 4.0;
    const SpinOrb& m_pq = (q < p) ? q : p;
    const SpinOrb& m_rs = (s < r) ? s : r;
    if (!(m_pq < m_rs)) {
      std::swap(p, r);
      std::swap(q, s);
    }
    if (alphas == 2) {
      if (q.spin == 0) {
        std::swap(p, q);
        c *= -1.0;
      }
      if (r.spin == 0) {
        std::swap(r, s);
        c *= -1.0;
      }
    } else {
      if (q.orbital < p.orbital) {
        std::swap(p, q);
        c *= -1.0;
      }
      if (r.orbital < s.orbital) {
        std::swap(r, s);
        c *= -1.0;
      }
    }
    k = TwoKey{p, q, r, s};
    coeff = c;
  }

  // AddTwoBodyTerm (:325-398) with the permutations of :400-417 and the spin
  // assignments of :440-463 (outer loop over the inner pair's spin).
  void add_two(int p, int q, int r, int s, double coeff) {
    if (coeff == 0) return;
    if (p == q && q == r && r == s) {
      update_two(TwoKey{SpinOrb{p, 0}, SpinOrb{p, 1}, SpinOrb{p, 1}, SpinOrb{p, 0}}, coeff);
      return;
    }
    const int i = p, j = q, kk = r, l = s;
    std::set<std::tuple<int, int, int, int>> perms = {
        {i, j, kk, l}, {l, j, kk, i}, {i, kk, j, l}, {l, kk, j, i},
        {j, i, l, kk}, {kk, i, l, j}, {j, l, i, kk}, {kk, l, i, j}};
    for (const auto& pm : perms) {
      int a, b, c, d;
      std::tie(a, b, c, d) = pm;
      for (int inner = 0; inner < 2; ++inner)
        for (int outer = 0; outer < 2; ++outer) {
          TwoKey key{SpinOrb{a, outer}, SpinOrb{b, inner}, SpinOrb{c, inner}, SpinOrb{d, outer}};
          std::set<SpinOrb> uniq{std::get<0>(key), std::get<1>(key), std::get<2>(key), std::get<3>(key)};
          double cf = coeff;
          bool keep = true;
          if (uniq.size() == 2)
            keep = reorder_pqqp(key, cf);
          else if (uniq.size() == 3)
            keep = reorder_pqqr(key, cf);
          else if (uniq.size() == 4)
            reorder_pqrs(key, cf);
          else
            throw Error(QPE_ERR_INVALID, "unknown two-body term type");
          if (keep) update_two(key, cf);
        }
    }
  }

  // IndexTerms(HalfUp) (:160-197): std::map::insert keeps the first value per key.
  void index_terms() {
    const int M = (int)num_orbitals;
    for (const auto& kv : one_body) {
      std::pair<unsigned, unsigned> key((unsigned)kv.first.first.half_up(M), (unsigned)kv.first.second.half_up(M));
      idx_one.insert(std::make_pair(key, kv.second));
    }
    for (const auto& kv : two_body) {
      SpinOrb p, q, r, s;
      std::tie(p, q, r, s) = kv.first;
      std::tuple<unsigned, unsigned, unsigned, unsigned> key((unsigned)p.half_up(M), (unsigned)q.half_up(M),
                                                            (unsigned)r.half_up(M), (unsigned)s.half_up(M));
      idx_two.insert(std::make_pair(key, kv.second));
    }
  }

  // Coefficient getters (:661-783). The expressions are kept as the reference
  // writes them so that the floating-point results are the same.
  std::complex<double> pp_term(unsigned p) const {
    using namespace std::complex_literals;
    auto it = idx_one.find(std::make_pair(p, p));
    if (it == idx_one.end()) return std::complex<double>(1.0);
    return std::exp(-1i * it->second * t);
  }
  void rot(double coeff, unsigned parity, std::complex<double> out[4]) const {
    using namespace std::complex_literals;
    std::complex<double> m00 = std::cos(coeff * t);
    int sign = (parity & 1) ? -1 : 1;  // powint(-1, parity) for parity in {0, 1}
    std::complex<double> m01 = -1i * static_cast<std::complex<double>>(sign) * std::sin(coeff * t);
    out[0] = m00;
    out[1] = m01;
    out[2] = m01;
    out[3] = m00;
  }
  static void ident(std::complex<double> out[4]) {
    out[0] = out[3] = std::complex<double>(1.0);
    out[1] = out[2] = std::complex<double>(0.0);
  }
  void pq_term(unsigned p, unsigned q, unsigned parity, std::complex<double> out[4]) const {
    auto it = idx_one.find(std::make_pair(p, q));
    if (it == idx_one.end()) return ident(out);
    rot(it->second, parity, out);
  }
  std::complex<double> pqqp_term(unsigned p, unsigned q) const {
    using namespace std::complex_literals;
    auto it = idx_two.find(std::make_tuple(p, q, q, p));
    if (it == idx_two.end()) return std::complex<double>(1.0);
    return std::exp(-1i * it->second * t);
  }
  void pqqr_term(unsigned p, unsigned q, unsigned r, unsigned parity, std::complex<double> out[4]) const {
    auto it = idx_two.find(std::make_tuple(p, q, q, r));
    if (it == idx_two.end()) return ident(out);
    rot(it->second, parity, out);
  }
  void pqrs_term(unsigned p, unsigned q, unsigned r, unsigned s, unsigned parity, std::complex<double> out[4]) const {
    auto it = idx_two.find(std::make_tuple(p, q, r, s));
    if (it == idx_two.end()) return ident(out);
    rot(it->second, parity, out);
  }
};

static void put2(const std::complex<double>* m, double* dst) {
  dst[0] = m[0].real();
  dst[1] = m[0].imag();
  dst[2] = m[1].real();
  dst[3] = m[1].imag();
}

// rank of a bit string (cpp/offset_computer.hpp:16-27), for the initial state.
static int64_t colex_rank(uint64_t bv) {
  int64_t r = 0;
  int order = 1;
  for (int pos = 0; bv; ++pos, bv >>= 1)
    if (bv & 1) r += (int64_t)binom_exact(pos, order++);
  return r;
}

}  // namespace qpe

using qpe::Hamiltonian;

struct qpe_hamiltonian {
  Hamiltonian h;
};

extern "C" {

int qpe_ham_create(qpe_hamiltonian** out) {
  return qpe::guard([&] {
    if (!out) throw qpe::Error(QPE_ERR_INVALID, "null output pointer");
    *out = new qpe_hamiltonian();
  });
}

int qpe_ham_destroy(qpe_hamiltonian* h) {
  delete h;
  return QPE_OK;
}

int qpe_ham_add_one_body(qpe_hamiltonian* h, int p, int q, double coeff) {
  return qpe::guard([&] {
    if (!h || p < 1 || q < 1 || p < q) throw qpe::Error(QPE_ERR_INVALID, "one-body term needs 1-based p >= q");
    h->h.add_one(p, q, coeff);
  });
}

int qpe_ham_add_two_body(qpe_hamiltonian* h, int p, int q, int r, int s, double coeff) {
  return qpe::guard([&] {
    if (!h || p < 1 || q < 1 || r < 1 || s < 1) throw qpe::Error(QPE_ERR_INVALID, "two-body orbitals are 1-based");
    h->h.add_two(p, q, r, s, coeff);
  });
}

int qpe_ham_set_num_orbitals(qpe_hamiltonian* h, uint32_t m) {
  if (!h || m == 0 || m > 31) return qpe::fail(QPE_ERR_INVALID, "num_orbitals must be in 1..31");
  h->h.num_orbitals = m;
  return QPE_OK;
}
int qpe_ham_set_num_occupied(qpe_hamiltonian* h, uint32_t e) {
  if (!h) return qpe::fail(QPE_ERR_INVALID, "null hamiltonian");
  h->h.num_occupied = e;
  return QPE_OK;
}
int qpe_ham_set_identity(qpe_hamiltonian* h, double v) {
  if (!h) return qpe::fail(QPE_ERR_INVALID, "null hamiltonian");
  h->h.identity = v;
  return QPE_OK;
}
int qpe_ham_set_timestep(qpe_hamiltonian* h, double t) {
  if (!h) return qpe::fail(QPE_ERR_INVALID, "null hamiltonian");
  h->h.t = t;
  return QPE_OK;
}
int qpe_ham_get_num_orbitals(const qpe_hamiltonian* h, uint32_t* out) {
  if (!h || !out) return qpe::fail(QPE_ERR_INVALID, "null argument");
  *out = h->h.num_orbitals;
  return QPE_OK;
}
int qpe_ham_get_num_occupied(const qpe_hamiltonian* h, uint32_t* out) {
  if (!h || !out) return qpe::fail(QPE_ERR_INVALID, "null argument");
  *out = h->h.num_occupied;
  return QPE_OK;
}
int qpe_ham_get_identity(const qpe_hamiltonian* h, double* out) {
  if (!h || !out) return qpe::fail(QPE_ERR_INVALID, "null argument");
  *out = h->h.identity;
  return QPE_OK;
}

int qpe_ham_index_terms(qpe_hamiltonian* h) {
  return qpe::guard([&] {
    if (!h || h->h.num_orbitals == 0) throw qpe::Error(QPE_ERR_INVALID, "set num_orbitals before indexing");
    h->h.idx_one.clear();
    h->h.idx_two.clear();
    h->h.index_terms();
  });
}

// PrintIndexedSegmentedHamiltonianTerms (:253-299): pp if p == q, else pq;
// pqqp if q == r and p == s, pqqr if q == r only, pqrs otherwise.
int qpe_ham_segment_counts(const qpe_hamiltonian* h, size_t counts[5]) {
  if (!h || !counts) return qpe::fail(QPE_ERR_INVALID, "null argument");
  for (int i = 0; i < 5; ++i) counts[i] = 0;
  for (const auto& kv : h->h.idx_one) counts[kv.first.first == kv.first.second ? QPE_TERM_PP : QPE_TERM_PQ]++;
  for (const auto& kv : h->h.idx_two) {
    unsigned p, q, r, s;
    std::tie(p, q, r, s) = kv.first;
    counts[q == r ? (p == s ? QPE_TERM_PQQP : QPE_TERM_PQQR) : QPE_TERM_PQRS]++;
  }
  return QPE_OK;
}

int qpe_ham_segment_terms(const qpe_hamiltonian* h, int kind, qpe_term* out, double* raw, size_t cap) {
  return qpe::guard([&] {
    if (!h || (!out && cap)) throw qpe::Error(QPE_ERR_INVALID, "null argument");
    if (kind < 0 || kind > 4) throw qpe::Error(QPE_ERR_INVALID, "unknown term kind");
    size_t n = 0;
    auto emit = [&](unsigned p, unsigned q, unsigned r, unsigned s, double v) -> qpe_term& {
      if (n >= cap) throw qpe::Error(QPE_ERR_INVALID, "output capacity too small");
      qpe_term& t = out[n];
      std::memset(&t, 0, sizeof(t));
      t.p = p;
      t.q = q;
      t.r = r;
      t.s = s;
      if (raw) raw[n] = v;
      ++n;
      return t;
    };
    const Hamiltonian& H = h->h;
    std::complex<double> m[4];
    if (kind == QPE_TERM_PP || kind == QPE_TERM_PQ) {
      for (const auto& kv : H.idx_one) {
        unsigned p = kv.first.first, q = kv.first.second;
        if ((p == q) != (kind == QPE_TERM_PP)) continue;
        qpe_term& t = emit(p, q, 0, 0, kv.second);
        if (kind == QPE_TERM_PP) {
          std::complex<double> c = H.pp_term(p);
          t.even[0] = c.real();
          t.even[1] = c.imag();
        } else {
          H.pq_term(p, q, 0, m);
          qpe::put2(m, t.even);
          H.pq_term(p, q, 1, m);
          qpe::put2(m, t.odd);
        }
      }
    } else {
      for (const auto& kv : H.idx_two) {
        unsigned p, q, r, s;
        std::tie(p, q, r, s) = kv.first;
        int k = q == r ? (p == s ? QPE_TERM_PQQP : QPE_TERM_PQQR) : QPE_TERM_PQRS;
        if (k != kind) continue;
        qpe_term& t = emit(p, q, r, s, kv.second);
        if (k == QPE_TERM_PQQP) {
          std::complex<double> c = H.pqqp_term(p, q);
          t.even[0] = c.real();
          t.even[1] = c.imag();
        } else if (k == QPE_TERM_PQQR) {
          H.pqqr_term(p, q, s, 0, m);
          qpe::put2(m, t.even);
          H.pqqr_term(p, q, s, 1, m);
          qpe::put2(m, t.odd);
        } else {
          H.pqrs_term(p, q, r, s, 0, m);
          qpe::put2(m, t.even);
          H.pqrs_term(p, q, r, s, 1, m);
          qpe::put2(m, t.odd);
        }
      }
    }
  });
}

// IngestBroombridge (cpp/hamiltonian.cc:8-144) over the project's YAML reader:
// identity, one-body rows [p, q, v] (swapped so p >= q), two-body rows
// [i, l, j, k, v] -> AddTwoBodyTerm(i, j, k, l), the orbital count as the largest
// index seen, and the first initial-state suggestion with its Jordan-Wigner signs
// (operators applied right to left; each one flips the sign once per occupied
// orbital below it), addressed at C(M, e) * rank(alpha) + rank(beta).
int qpe_ham_ingest_broombridge(qpe_hamiltonian* hh, const char* path, uint32_t* num_orbitals, uint32_t* num_occupied,
                               double* block0, size_t cap) {
  return qpe::guard([&] {
    if (!hh || !path) throw qpe::Error(QPE_ERR_INVALID, "null argument");
    Hamiltonian& H = hh->h;
    std::shared_ptr<const qpe_yaml::Value> doc;
    try {
      doc = qpe_yaml::load_file(path);
    } catch (const std::exception& e) {
      throw qpe::Error(QPE_ERR_INVALID, e.what());
    }
    auto need = [](const qpe_yaml::Value* v, const char* what) {
      if (!v) throw qpe::Error(QPE_ERR_INVALID, std::string("Broombridge file lacks ") + what);
      return v;
    };
    auto num = [&](const qpe_yaml::Value* v, const char* what) {
      need(v, what);
      if (v->kind != qpe_yaml::Value::Scalar) throw qpe::Error(QPE_ERR_INVALID, std::string(what) + " is not a number");
      return std::strtod(v->scalar.c_str(), nullptr);
    };
    const qpe_yaml::Value* sets = need(doc->get("integral_sets"), "integral_sets");
    const qpe_yaml::Value* ints = need(sets->at(0), "integral_sets[0]");
    H.identity = num(need(ints->get("coulomb_repulsion"), "coulomb_repulsion")->get("value"), "coulomb_repulsion") +
                 num(need(ints->get("energy_offset"), "energy_offset")->get("value"), "energy_offset");
    const qpe_yaml::Value* ham = need(ints->get("hamiltonian"), "hamiltonian");
    unsigned maxorb = H.num_orbitals;
    const qpe_yaml::Value* ob = need(need(ham->get("one_electron_integrals"), "one_electron_integrals")->get("values"),
                                     "one_electron_integrals.values");
    for (const auto& row : ob->seq) {
      unsigned p = (unsigned)num(row->at(0), "index"), q = (unsigned)num(row->at(1), "index");
      const double v = num(row->at(2), "value");
      if (q > p) std::swap(p, q);
      H.add_one((int)p, (int)q, v);
      maxorb = std::max(maxorb, std::max(p, q));
    }
    const qpe_yaml::Value* tb = need(need(ham->get("two_electron_integrals"), "two_electron_integrals")->get("values"),
                                     "two_electron_integrals.values");
    for (const auto& row : tb->seq) {
      const unsigned i = (unsigned)num(row->at(0), "index"), l = (unsigned)num(row->at(1), "index");
      const unsigned j = (unsigned)num(row->at(2), "index"), k = (unsigned)num(row->at(3), "index");
      H.add_two((int)i, (int)j, (int)k, (int)l, num(row->at(4), "value"));
      maxorb = std::max(maxorb, std::max(std::max(i, j), std::max(k, l)));
    }
    if (maxorb == 0 || maxorb > 31) throw qpe::Error(QPE_ERR_UNSUPPORTED, "orbital count must be in 1..31");
    H.num_orbitals = maxorb;
    // Initial state (cpp/hamiltonian.cc:54-139).
    std::vector<std::pair<uint64_t, double>> amps;
    const qpe_yaml::Value* sugg = ints->get("initial_state_suggestions");
    const qpe_yaml::Value* sup = nullptr;
    if (sugg && sugg->at(0) && sugg->at(0)->get("state")) sup = sugg->at(0)->get("state")->get("superposition");
    static const std::regex pat(R"(\((\d+)([ab])\)(\+*))");
    if (sup) {
      for (const auto& basis : sup->seq) {
        if (basis->kind != qpe_yaml::Value::Seq || basis->seq.size() < 2) continue;
        double coeff = num(basis->at(0), "coefficient");
        unsigned electrons = 0;
        uint64_t bv = 0;
        for (size_t t = basis->seq.size() - 1; t-- > 1;) {  // operators, right to left
          std::smatch m;
          const std::string& txt = basis->seq[t]->scalar;
          if (!std::regex_match(txt, m, pat)) throw qpe::Error(QPE_ERR_INVALID, "bad operator " + txt);
          const unsigned orb = (unsigned)std::stoi(m[1]) - 1;
          const bool up = m[2] == "a";
          const bool raise = m[3] == "+";
          const unsigned idx = up ? orb : orb + maxorb;
          if (idx >= 64) throw qpe::Error(QPE_ERR_INVALID, "orbital index out of range");
          if (raise) {
            if ((bv >> idx) & 1) throw qpe::Error(QPE_ERR_INVALID, "creation on an occupied orbital");
            bv += 1ull << idx;
            ++electrons;
          } else {
            if (!((bv >> idx) & 1)) throw qpe::Error(QPE_ERR_INVALID, "annihilation on an empty orbital");
            bv -= 1ull << idx;
            --electrons;
          }
          for (unsigned pos = 0; pos < idx; ++pos)
            if ((bv >> pos) & 1) coeff *= -1.0;
        }
        H.num_occupied = electrons / 2;
        const uint64_t beta = bv >> maxorb, alpha = bv & ((1ull << maxorb) - 1);
        const uint64_t addr = qpe::binom_exact((int)maxorb, (int)H.num_occupied) * (uint64_t)qpe::colex_rank(alpha) +
                              (uint64_t)qpe::colex_rank(beta);
        amps.emplace_back(addr, coeff);
      }
    }
    if (num_orbitals) *num_orbitals = H.num_orbitals;
    if (num_occupied) *num_occupied = H.num_occupied;
    if (block0) {
      const uint64_t C = qpe::binom_exact((int)H.num_orbitals, (int)H.num_occupied);
      if (cap < C * C) throw qpe::Error(QPE_ERR_INVALID, "block0 capacity below C(M, e)^2");
      std::memset(block0, 0, 2 * C * C * sizeof(double));
      for (const auto& a : amps) {
        if (a.first >= C * C) throw qpe::Error(QPE_ERR_INVALID, "initial state outside the register");
        block0[2 * a.first] = a.second;
        block0[2 * a.first + 1] = 0.0;
      }
    }
  });
}

int qpe_ham_pp_term(const qpe_hamiltonian* h, uint32_t p, double out[2]) {
  if (!h || !out) return qpe::fail(QPE_ERR_INVALID, "null argument");
  std::complex<double> c = h->h.pp_term(p);
  out[0] = c.real();
  out[1] = c.imag();
  return QPE_OK;
}
static void put4(const std::complex<double>* m, double* out) {
  for (int i = 0; i < 4; ++i) {
    out[2 * i] = m[i].real();
    out[2 * i + 1] = m[i].imag();
  }
}
int qpe_ham_pq_term(const qpe_hamiltonian* h, uint32_t p, uint32_t q, uint32_t parity, double out[8]) {
  if (!h || !out) return qpe::fail(QPE_ERR_INVALID, "null argument");
  std::complex<double> m[4];
  h->h.pq_term(p, q, parity, m);
  put4(m, out);
  return QPE_OK;
}
int qpe_ham_pqqp_term(const qpe_hamiltonian* h, uint32_t p, uint32_t q, double out[2]) {
  if (!h || !out) return qpe::fail(QPE_ERR_INVALID, "null argument");
  std::complex<double> c = h->h.pqqp_term(p, q);
  out[0] = c.real();
  out[1] = c.imag();
  return QPE_OK;
}
int qpe_ham_pqqr_term(const qpe_hamiltonian* h, uint32_t p, uint32_t q, uint32_t r, uint32_t parity,
                      double out[8]) {
  if (!h || !out) return qpe::fail(QPE_ERR_INVALID, "null argument");
  std::complex<double> m[4];
  h->h.pqqr_term(p, q, r, parity, m);
  put4(m, out);
  return QPE_OK;
}
int qpe_ham_pqrs_term(const qpe_hamiltonian* h, uint32_t p, uint32_t q, uint32_t r, uint32_t s,
                      uint32_t parity, double out[8]) {
  if (!h || !out) return qpe::fail(QPE_ERR_INVALID, "null argument");
  std::complex<double> m[4];
  h->h.pqrs_term(p, q, r, s, parity, m);
  put4(m, out);
  return QPE_OK;
}

}  // extern "C"
