// program_build.cpp - host compiler from segmented Hamiltonian terms to a device
// program (tables + ops + passes), see program.h for the pass model.
#include "program_build.h"

#include <algorithm>
#include <map>
#include <string>
#include <tuple>

#include "qpe_common.h"

namespace qpe {

uint64_t binom(int n, int k) {
  if (k < 0 || n < 0 || k > n) return 0;
  if (k * 2 > n) k = n - k;
  uint64_t r = 1;
  for (int i = 1; i <= k; ++i) r = r * (uint64_t)(n - k + i) / (uint64_t)i;
  return r;
}

namespace {

struct AbsOp {
  char cls;            // 'A' column-local, 'B' row-local, 'D' diagonal, 'X' mixed ABBA
  int ta = -1, tb = -1;
  int na = 0, nb = 0;  // D: occupied alpha/beta orbitals; A: beta cond bits; B: alpha cond bits
  uint8_t abit[2] = {0, 0}, bbit[2] = {0, 0};
  uint32_t coef = 0;
  uint64_t touches = 0;
};

struct Builder {
  HostProgram& P;
  std::map<std::tuple<int, int, int, int, int, int>, int> reg;  // (kind, spin, o0..o3)

  explicit Builder(HostProgram& p) : P(p) {}

  int weight_of(int spin) const { return spin ? (int)P.nb : (int)P.na; }

  int table(AxisKind kind, int spin, int o0, int o1 = 0, int o2 = 0, int o3 = 0) {
    auto key = std::make_tuple((int)kind, spin, o0, o1, o2, o3);
    auto it = reg.find(key);
    if (it != reg.end()) return it->second;
    AxisTable t{};
    t.kind = kind;
    t.nbits = (uint8_t)P.M;
    t.weight = (uint8_t)weight_of(spin);
    int nocc = 0;
    switch (kind) {
      case AX_N: t.nfixed = 1; nocc = 1; break;
      case AX_NN: t.nfixed = 2; nocc = 2; break;
      case AX_CA: t.nfixed = 2; nocc = 1; break;
      case AX_CNA: t.nfixed = 3; nocc = 2; break;
      case AX_CCAA: t.nfixed = 4; nocc = 2; break;
    }
    t.o[0] = (uint8_t)o0;
    t.o[1] = (uint8_t)o1;
    t.o[2] = (uint8_t)o2;
    t.o[3] = (uint8_t)o3;
    uint64_t cnt = binom((int)P.M - t.nfixed, weight_of(spin) - nocc);
    if (cnt > 0x7fffffffull) throw Error(QPE_ERR_UNSUPPORTED, "index table too large");
    t.count = (uint32_t)cnt;
    const bool pairs = kind == AX_CA || kind == AX_CNA || kind == AX_CCAA;
    uint64_t words = cnt * (pairs ? 2 : 1);
    if (pairs && (P.pool_words & 1)) ++P.pool_words;  // pair entries are read as 8-byte words
    if (P.pool_words + words > 0xffffffffull) throw Error(QPE_ERR_UNSUPPORTED, "index pool too large");
    t.offset = (uint32_t)P.pool_words;
    P.pool_words += words;
    P.tables.push_back(t);
    int id = (int)P.tables.size() - 1;
    reg.emplace(key, id);
    return id;
  }

  uint64_t cnt(int id) const { return id < 0 ? 0 : P.tables[id].count; }
  // Lines of one spin whose string has all `nbits` given orbitals occupied.
  uint64_t lines_with(int spin, int nbits) const {
    return binom((int)P.M - nbits, weight_of(spin) - nbits);
  }

  uint32_t add_coef(const qpe_term& t) {
    uint32_t id = (uint32_t)(P.coefs.size() / 8);
    for (int i = 0; i < 4; ++i) P.coefs.push_back(t.even[i]);
    for (int i = 0; i < 4; ++i) P.coefs.push_back(t.odd[i]);
    return id;
  }

  void check_index(unsigned v) const {
    if (v >= 2 * P.M) throw Error(QPE_ERR_INVALID, "term index out of range: " + std::to_string(v));
  }

  // The dispatch of applyUnitary_reordered (:374-562) for one term, including the
  // early returns for fewer than two electrons of a spin (:593, :849, :991, :1080).
  bool lower(int kind, const qpe_term& t, AbsOp& op) {
    const unsigned M = P.M;
    op = AbsOp{};
    switch (kind) {
      case QPE_TERM_PP: {  // updatePP_AA / updatePP_BB
        check_index(t.p);
        op.cls = 'D';
        if (t.p < M) { op.na = 1; op.abit[0] = (uint8_t)t.p; }
        else { op.nb = 1; op.bbit[0] = (uint8_t)(t.p - M); }
        break;
      }
      case QPE_TERM_PQQP: {  // updatePQQP_AA / _BB / _AB
        check_index(t.p); check_index(t.q);
        if (t.p >= t.q) throw Error(QPE_ERR_INVALID, "pqqp term needs p < q");
        op.cls = 'D';
        if (t.q < M) {
          if (P.na < 2) return false;
          op.na = 2; op.abit[0] = (uint8_t)t.p; op.abit[1] = (uint8_t)t.q;
        } else if (t.p >= M) {
          if (P.nb < 2) return false;
          op.nb = 2; op.bbit[0] = (uint8_t)(t.p - M); op.bbit[1] = (uint8_t)(t.q - M);
        } else {
          op.na = 1; op.abit[0] = (uint8_t)t.p;
          op.nb = 1; op.bbit[0] = (uint8_t)(t.q - M);
        }
        break;
      }
      case QPE_TERM_PQ: {  // updatePQ_AA: discoverCA(p, q); updatePQ_BB
        check_index(t.p); check_index(t.q);
        if (t.p <= t.q || (t.p < M) != (t.q < M)) throw Error(QPE_ERR_INVALID, "pq term needs p > q of one spin");
        if (t.p < M) { op.cls = 'A'; op.ta = table(AX_CA, 0, t.p, t.q); }
        else { op.cls = 'B'; op.tb = table(AX_CA, 1, t.p - M, t.q - M); }
        break;
      }
      case QPE_TERM_PQQR: {  // key (p, q, q, r): r in t.s
        const unsigned p = t.p, q = t.q, r = t.s;
        check_index(p); check_index(q); check_index(r);
        if (t.r != q || r <= p || (p < M) != (r < M) || q == p || q == r)
          throw Error(QPE_ERR_INVALID, "malformed pqqr term");
        if (p < M && q < M) {  // AAAA
          if (P.na < 2) return false;
          op.cls = 'A'; op.ta = table(AX_CNA, 0, p, q, r);
        } else if (p >= M && q >= M) {  // BBBB
          if (P.nb < 2) return false;
          op.cls = 'B'; op.tb = table(AX_CNA, 1, p - M, q - M, r - M);
        } else if (q >= M) {  // ABBA: alpha CA(p, r), beta strings with q
          op.cls = 'A'; op.ta = table(AX_CA, 0, p, r);
          op.nb = 1; op.bbit[0] = (uint8_t)(q - M);
        } else {  // BAAB: alpha strings with q, beta CA(p, r)
          op.cls = 'B'; op.tb = table(AX_CA, 1, p - M, r - M);
          op.na = 1; op.abit[0] = (uint8_t)q;
        }
        break;
      }
      case QPE_TERM_PQRS: {
        const unsigned p = t.p, q = t.q, r = t.r, s = t.s;
        check_index(p); check_index(q); check_index(r); check_index(s);
        if (p < M && q < M && r < M && s < M) {
          if (P.na < 2) return false;
          if (p == q || p == r || p == s || q == r || q == s || r == s) throw Error(QPE_ERR_INVALID, "pqrs orbitals repeat");
          op.cls = 'A'; op.ta = table(AX_CCAA, 0, p, q, r, s);
        } else if (p >= M && q >= M && r >= M && s >= M) {
          if (P.nb < 2) return false;
          if (p == q || p == r || p == s || q == r || q == s || r == s) throw Error(QPE_ERR_INVALID, "pqrs orbitals repeat");
          op.cls = 'B'; op.tb = table(AX_CCAA, 1, p - M, q - M, r - M, s - M);
        } else {
          if (!(p < M && s < M && q >= M && r >= M) || p == s || q == r)
            throw Error(QPE_ERR_INVALID, "mixed pqrs term must be alpha p, s and beta q, r");
          op.cls = 'X'; op.ta = table(AX_CA, 0, p, s); op.tb = table(AX_CA, 1, q - M, r - M);
        }
        break;
      }
      default:
        throw Error(QPE_ERR_INVALID, "unknown term kind");
    }
    op.coef = add_coef(t);
    // Amplitude-term updates of this application (pair = 2, diagonal = 1).
    switch (op.cls) {
      case 'D': op.touches = lines_with(0, op.na) * lines_with(1, op.nb); break;
      case 'A': op.touches = 2 * cnt(op.ta) * lines_with(1, op.nb); break;
      case 'B': op.touches = 2 * cnt(op.tb) * lines_with(0, op.na); break;
      case 'X': op.touches = 2 * cnt(op.ta) * cnt(op.tb); break;
    }
    return true;
  }

  int list_table(int spin, int n, const uint8_t* bits) {
    if (n == 1) return table(AX_N, spin, bits[0]);
    return table(AX_NN, spin, bits[0], bits[1]);
  }

  DevOp encode(const AbsOp& a, uint32_t pass_type) {
    DevOp d{};
    const double* rec = &P.coefs[8 * (size_t)a.coef];
    if (a.cls == 'D') {
      d.gen = OP_INLINE;
      d.c0 = rec[0];
      d.c1 = rec[1];
    } else if (rec[1] == 0.0 && rec[2] == 0.0 && rec[5] == 0.0 && rec[6] == 0.0 && rec[4] == rec[0] &&
               rec[7] == -rec[3]) {
      // m00 = (c, 0) for both parities, m01 = (0, t) for parity 0 and (0, -t) for 1
      d.gen = OP_INLINE;
      d.c0 = rec[0];
      d.c1 = rec[3];
    } else {
      d.gen = a.coef;
    }
    auto tab_ref = [&](int id) {
      d.tab = P.tables[id].offset;
      d.count = P.tables[id].count;
    };
    if (pass_type == PASS_COL) {
      if (a.cls == 'A') {
        d.kind = OPK_PAIR; tab_ref(a.ta);
        d.ncond = (uint8_t)a.nb; d.cb0 = a.bbit[0]; d.cb1 = a.bbit[1];
      } else {  // D
        if (a.na == 0) { d.kind = OPK_DIAG_ALL; d.count = (uint32_t)P.Ca; }
        else { d.kind = OPK_DIAG_LIST; tab_ref(list_table(0, a.na, a.abit)); }
        d.ncond = (uint8_t)a.nb; d.cb0 = a.bbit[0]; d.cb1 = a.bbit[1];
      }
    } else if (pass_type == PASS_ROW) {
      if (a.cls == 'B') {
        d.kind = OPK_PAIR; tab_ref(a.tb);
        d.ncond = (uint8_t)a.na; d.cb0 = a.abit[0]; d.cb1 = a.abit[1];
      } else {  // D
        if (a.nb == 0) { d.kind = OPK_DIAG_ALL; d.count = (uint32_t)P.Cb; }
        else { d.kind = OPK_DIAG_LIST; tab_ref(list_table(1, a.nb, a.bbit)); }
        d.ncond = (uint8_t)a.na; d.cb0 = a.abit[0]; d.cb1 = a.abit[1];
      }
    } else {  // MIX
      d.kind = OPK_PAIR; tab_ref(a.ta);
    }
    return d;
  }

  // Groups consecutive applications into passes (program.h).
  void segment(const std::vector<AbsOp>& seq) {
    bool open = false;
    Pass cur{};
    int cur_mix = -1;
    auto close = [&]() {
      if (open) {
        cur.op1 = (uint32_t)P.ops.size();
        P.passes.push_back(cur);
      }
      open = false;
    };
    auto start = [&](uint32_t type) {
      close();
      cur = Pass{};
      cur.type = type;
      cur.op0 = (uint32_t)P.ops.size();
      open = true;
    };
    for (const AbsOp& a : seq) {
      uint32_t want;
      if (a.cls == 'A') want = PASS_COL;
      else if (a.cls == 'B') want = PASS_ROW;
      else if (a.cls == 'D') want = (open && cur.type != PASS_MIX) ? cur.type : (uint32_t)PASS_COL;
      else want = PASS_MIX;
      if (!open || cur.type != want || (want == PASS_MIX && cur_mix != a.tb)) {
        start(want);
        if (want == PASS_MIX) {
          cur_mix = a.tb;
          cur.mixtab = P.tables[a.tb].offset;
          cur.mixcount = P.tables[a.tb].count;
        }
      }
      P.ops.push_back(encode(a, want));
    }
    close();
  }
};

}  // namespace

// The application order of applyUnitary_reordered (:374-562).
static void reordered_sweep(Builder& B, const TermArrays& T, std::vector<AbsOp>& sweep) {
  const unsigned M = B.P.M;
  AbsOp op;
  for (size_t i = 0; i < T.n[QPE_TERM_PP]; ++i)
    if (B.lower(QPE_TERM_PP, T.t[QPE_TERM_PP][i], op)) sweep.push_back(op);
  for (size_t i = 0; i < T.n[QPE_TERM_PQQP]; ++i)
    if (B.lower(QPE_TERM_PQQP, T.t[QPE_TERM_PQQP][i], op)) sweep.push_back(op);
  for (size_t i = 0; i < T.n[QPE_TERM_PQ]; ++i) {
    const qpe_term& pq = T.t[QPE_TERM_PQ][i];
    if (B.lower(QPE_TERM_PQ, pq, op)) sweep.push_back(op);
    // :453-465: every pqqr (p_, q_, q_, r_) with p_ == q and r_ == p, in map order.
    for (size_t j = 0; j < T.n[QPE_TERM_PQQR]; ++j) {
      const qpe_term& t = T.t[QPE_TERM_PQQR][j];
      if (t.p == pq.q && t.s == pq.p && B.lower(QPE_TERM_PQQR, t, op)) sweep.push_back(op);
    }
  }
  // pqqr terms no pq term picks up are never applied (:465); they are still
  // validated so that malformed input is reported.
  for (size_t j = 0; j < T.n[QPE_TERM_PQQR]; ++j) {
    const qpe_term& t = T.t[QPE_TERM_PQQR][j];
    if (t.p >= 2 * M || t.q >= 2 * M || t.s >= 2 * M) throw Error(QPE_ERR_INVALID, "pqqr index out of range");
  }
  for (size_t i = 0; i < T.n[QPE_TERM_PQRS]; ++i)
    if (B.lower(QPE_TERM_PQRS, T.t[QPE_TERM_PQRS][i], op)) sweep.push_back(op);
}

void build_program(HostProgram& P, unsigned M, unsigned na, unsigned nb, const TermArrays& T,
                   unsigned order, unsigned steps) {
  const bool au_order = (order & QPE_PROGRAM_APPLY_UNITARY_ORDER) != 0;
  order &= ~QPE_PROGRAM_APPLY_UNITARY_ORDER;
  if (M == 0 || M > 31) throw Error(QPE_ERR_INVALID, "num_orbitals must be in 1..31");
  if (na == 0 || nb == 0 || na > M || nb > M) throw Error(QPE_ERR_INVALID, "electrons per spin must be in 1..M");
  if (order != 1 && order != 2) throw Error(QPE_ERR_INVALID, "trotter_order must be 1 or 2");
  if (steps == 0 || steps > 4096) throw Error(QPE_ERR_INVALID, "steps_per_power must be in 1..4096");
  P = HostProgram{};
  P.M = M;
  P.na = na;
  P.nb = nb;
  P.Ca = binom((int)M, (int)na);
  P.Cb = binom((int)M, (int)nb);
  if (P.Ca > 0x7fffffffull || P.Cb > 0x7fffffffull) throw Error(QPE_ERR_UNSUPPORTED, "string space too large");
  P.order = order;
  P.steps = steps;
  P.apply_unitary_order = au_order;
  Builder B(P);

  std::vector<AbsOp> sweep;
  AbsOp op;
  if (au_order) {
    // The order of applyUnitary (:174-372): each segment whole, in map order.
    for (int kind : {QPE_TERM_PP, QPE_TERM_PQ, QPE_TERM_PQQP, QPE_TERM_PQQR, QPE_TERM_PQRS})
      for (size_t i = 0; i < T.n[kind]; ++i)
        if (B.lower(kind, T.t[kind][i], op)) sweep.push_back(op);
  } else {
    reordered_sweep(B, T, sweep);
  }

  P.ops_per_sweep = (uint32_t)sweep.size();
  for (const AbsOp& a : sweep) P.touches_per_sweep += a.touches;
  // One forward sweep is stored. A controlled power runs it `steps` times; a
  // second-order step runs it forward and then backward (the passes in reverse
  // order, each pass's terms in reverse order): segmenting the reversed term
  // list gives the same passes reversed, so the backward sweep needs no copy.
  P.touches_per_power = P.touches_per_sweep * steps * order;
  B.segment(sweep);
  if (P.pool_words == 0) P.pool_words = 1;
}

}  // namespace qpe
