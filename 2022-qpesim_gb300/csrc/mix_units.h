// mix_units.h - runs of column-pair (MIX) passes as independent update units, for
// the resident kernel with the block spread over a cluster (k_resident_lean).
//
// Every term of a MIX pass pairs amplitude (a, b01) with (a', b10) for each row
// pair (a, a') of its alpha table and each column pair (b01, b10) of the pass's
// beta table. Take a window of consecutive MIX passes and join the two amplitudes
// of every such pair: the window's updates split into connected components, and
// updates of different components touch disjoint amplitudes. So a component (a
// "unit") can run on its own for the whole window: gather its amplitudes, apply
// the window's terms in order (level k = the window's term k; within a level every
// update is on its own pair of amplitudes), scatter them back. The updates that
// touch one amplitude keep their order and each keeps the tile runner's
// arithmetic, so the results are bit-identical; a window of w passes needs one
// gather, one scatter and one cluster barrier instead of w of each.
//
// The host grows each window while its units still fit (at most 24 updates per
// level and 192 amplitudes per unit; the kernel's warps and stages) and packs the
// units into warp programs: small units share a warp (their updates at each
// level on its 8 quads of lanes, their amplitudes, up to 64, on its own range of
// the group's stage), large ones take a team of two
// or three warps of one three-warp group, which then synchronises by the group's
// named barrier. Units go to the CTA with the least work per level.
//
// Per pass (MixUnits::pass_slot): kMixNoSchedule (the pass runs by tiles), or the
// window's block of warp programs (bits 0-19) and its number of passes (bits
// 20-27), the same for every pass of the window. A sweep meets a window at its
// first pass (forward) or its last (reversed), runs it, and skips its other passes.
//
// Warp program (kMixWpHeader + kMixWarpAmps + 8 * levels words, a multiple of 4):
//   w[0]                     nelem (bits 0-6, <= 64) | team warps (bits 7-8; 0: idle)
//                            | levels (bits 9-16)
//   w[1]                     first term of the window (its op index)
//   w[kMixWpHeader + l]      gather entry l (lane l % 32): row | col << 11 | stage index << 22
//   w[kMixWpHeader + kMixWarpAmps + 8 k + u]
//                            update of quad u at level k: left stage index
//                            | right stage index << 10 | parity << 20 | valid << 21
#ifndef QPE_MIX_UNITS_H_
#define QPE_MIX_UNITS_H_

#include <stdint.h>

#include <vector>

#include "program_build.h"

namespace qpe {

struct MixUnits {
  uint32_t wp_words = 0;             // words per warp program
  uint32_t warps_per_cta = 0;
  uint32_t cluster = 0;
  uint32_t scheduled = 0;            // MIX passes with a schedule
  uint32_t windows = 0;              // blocks of warp programs
  std::vector<uint32_t> pass_slot;   // per pass, as above
  std::vector<uint32_t> words;       // blocks [window][cta][warp][wp_words]
};

// Words of one warp program (windows of at most kMixMaxLevels terms).
uint32_t mix_wp_words(const HostProgram& hp);

// Builds the windows and unit schedules of the MIX passes of `hp` whose terms are
// inline pair terms, windows of at most max_window passes. `pool` is the
// program's index pool as built on the device. Passes whose units do not fit keep
// the tile runner. Returns false when no pass could be scheduled.
bool build_mix_units(const HostProgram& hp, const uint32_t* pool, uint32_t K, uint32_t warps_per_cta,
                     uint32_t stage_elems, uint32_t max_window, MixUnits& out);

// Row and column passes as per-line programs (k_resident_lean, strategy 7).
//
// A row or column pass applies its terms to every line (row or column)
// separately, in order, each term on the line only if the line's own string has
// the term's condition orbitals. The host evaluates those conditions per line
// and writes, for each line, the program of the terms that apply: one level per
// term (a term whose updates exceed the team's lanes takes several levels, its
// trips, which touch disjoint amplitudes), each with the term's op index and the
// update word of every quad. The kernel then runs a line like an update unit: a
// team of three warps gathers the line into its group's stage, runs the levels
// (the next levels' words loaded ahead from global memory) and scatters it back,
// with no per-term decisions on the device. Pair updates are the quad-split
// updates of the line runner (left / right stage index, parity); diagonal
// updates are split over lane pairs (two amplitudes per word, lane h writing
// component h of v (c0 + i c1) as in the line runner).
//
// With replicas, line b of a column pass runs on replica b % replicas and row a
// of a row pass on replica (a - first row of its CTA) % replicas: the lines
// each replica exchanges afterwards. Rows run on the CTA that owns them.
//
// Line program (words):
//   w[0]   nelem (bits 0-6) | team warps (bits 7-8)     w[1] levels
//   w[kMixWpHeader + l]    gather entry l, as in a window's program
//   w[kMixWpHeader + kMixWarpAmps + 9 k]       op index | diagonal << 31
//   w[kMixWpHeader + kMixWarpAmps + 9 k + 1 + u]
//          pair: left | right << 10 | parity << 20 | valid << 21
//          diagonal: amplitude of slot 2u | of slot 2u + 1 << 10 | valid << 20 | valid << 21
//     (quad u; for a diagonal level lanes 4u, 4u + 1 take slot 2u, lanes 4u + 2,
//     4u + 3 slot 2u + 1)
struct LineUnits {
  uint32_t passes = 0;               // row and column passes with programs
  uint32_t replicas = 1;
  std::vector<uint32_t> pass_slot;   // per pass: its block of program offsets, or kMixNoSchedule
  std::vector<uint32_t> offs;        // blocks [slot][replica][cta][warp]: word offset of the
                                     // warp's program, or kMixNoSchedule (idle)
  std::vector<uint32_t> words;
};

// Builds the line programs of every row and column pass of `hp` whose terms are
// inline (general pair matrices keep the line runner). strA / strB: the line
// strings by rank (the device's tables); pool: the index pool.
bool build_line_units(const HostProgram& hp, const uint32_t* pool, const uint32_t* strA, const uint32_t* strB,
                      uint32_t K, uint32_t warps_per_cta, uint32_t rows_per_cta, uint32_t replicas,
                      uint32_t stage_elems, LineUnits& out);

}  // namespace qpe

#endif  // QPE_MIX_UNITS_H_
