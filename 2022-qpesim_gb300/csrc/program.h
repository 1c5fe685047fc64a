// program.h - the device-facing form of one Hamiltonian's Trotter step.
//
// A sweep (one first-order Trotter step, applyUnitary_reordered in
// cpp/time_evolution_over_terms.hpp:374-562) is compiled into a list of passes.
// Each pass is a run of consecutive term applications that share a "line"
// decomposition of the Ca x Cb block, so that the block splits into independent
// tiles the pass can process without synchronising with other tiles:
//   PASS_COL: lines are columns (fixed beta string). Terms that change only alpha
//             occupations (pq, pqqr AAAA/ABBA, pqrs AAAA) and every diagonal term
//             act on each column separately.
//   PASS_ROW: lines are rows (fixed alpha string): the mirror image for beta.
//   PASS_MIX: consecutive pqrs ABBA terms with the same beta pair (q, r); a tile is
//             the two columns b01 (r occupied) and b10 (q occupied) that the beta
//             pair table pairs up, over all rows.
// Inside a tile the terms are applied in the reference order. The per-term index
// sets come from device-built tables equal to the expanded run tables of the
// discover*_BVs routines (:1160-1411), entry for entry.
#ifndef QPE_PROGRAM_H_
#define QPE_PROGRAM_H_

#include <stdint.h>

namespace qpe {

enum AxisKind : uint8_t { AX_N = 0, AX_NN = 1, AX_CA = 2, AX_CNA = 3, AX_CCAA = 4 };

// One device index table over the strings of one spin.
//   AX_N    o = {q}           list: strings with q occupied               (discoverN_BVs)
//   AX_NN   o = {p, r}        list: strings with p and r occupied         (discoverNN_BVs)
//   AX_CA   o = {p, r}        pairs: 01 side r occupied, 10 side p        (discoverCA_BVs)
//   AX_CNA  o = {p, q, r}     pairs: q occupied; 01 side r, 10 side p     (discoverCNA_BVs)
//   AX_CCAA o = {p, q, r, s}  pairs: 01 side r, s; 10 side p, q           (discoverCCAA_BVs)
// Pair entries take two words: (i01 | parity << 31, i10). List entries one word.
struct AxisTable {
  uint8_t kind;
  uint8_t nbits;   // orbitals of the spin (M)
  uint8_t weight;  // electrons of the spin
  uint8_t nfixed;
  uint8_t o[4];
  uint32_t count;   // entries
  uint32_t offset;  // first word in the pool
};

// One term application inside a pass. `cond` bits (ncond of them) must all be
// occupied in the line's own string for the term to act on that line (e.g. the
// spectator q of a pqqr ABBA term, or the beta orbitals of a diagonal term
// applied in a column pass). The coefficients are inline: for a pair term with a
// real m00 = c0 and an imaginary m01 = i * c1 for parity 0 and -i * c1 for parity 1
// (every term of the reference's getters: cos and -sin of h t), `c0`, `c1`; for a
// diagonal term its complex coefficient (c0, c1). Any other pair matrix keeps its
// 8-double record (even m00, m01, odd m00, m01) at index `gen` of the program's
// coefficient array; gen == OP_INLINE marks the inline form.
constexpr uint32_t OP_INLINE = 0xffffffffu;
struct alignas(16) DevOp {
  uint32_t tab;    // word offset of the table (unused for OPK_DIAG_ALL)
  uint32_t count;  // table entries (OPK_DIAG_ALL: line length)
  uint8_t kind;
  uint8_t ncond;
  uint8_t cb0, cb1;
  uint32_t gen;    // OP_INLINE, or the coefficient record of a general pair matrix
  double c0, c1;
};
static_assert(sizeof(DevOp) == 32, "DevOp layout");

enum OpKind : uint8_t { OPK_PAIR = 0, OPK_DIAG_LIST = 1, OPK_DIAG_ALL = 2 };

enum PassType : uint8_t { PASS_COL = 0, PASS_ROW = 1, PASS_MIX = 2 };

// The chunked term runners of the tile passes (tile_ops.cuh) set up kPairChunk
// terms at a time, each covering up to kPairTrips entries per thread.
constexpr uint32_t kPairChunk = 4;
constexpr uint32_t kPairTrips = 3;

// Column-pair passes as update units (mix_units.h): words before a warp
// program's gather entries, the amplitudes one warp gathers (two per lane), the
// most terms a scheduled window may have, and the slot of a pass without a
// schedule.
constexpr uint32_t kMixWpHeader = 4;
constexpr uint32_t kMixWarpAmps = 64;
constexpr uint32_t kMixMaxLevels = 24;
constexpr uint32_t kMixNoSchedule = 0xffffffffu;

struct Pass {
  uint32_t type;
  uint32_t op0, op1;
  uint32_t mixtab;    // PASS_MIX: word offset of the beta CA pair table
  uint32_t mixcount;  // PASS_MIX: its entries (= tiles)
};

}  // namespace qpe

#endif  // QPE_PROGRAM_H_
