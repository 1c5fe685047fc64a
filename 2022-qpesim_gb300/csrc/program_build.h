// program_build.h - host-side program representation and its builder.
#ifndef QPE_PROGRAM_BUILD_H_
#define QPE_PROGRAM_BUILD_H_

#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "../../include/qpe_gb300.h"
#include "program.h"

namespace qpe {

// The five segmented term arrays, indexed by QPE_TERM_*.
struct TermArrays {
  const qpe_term* t[5];
  size_t n[5];
};

struct HostProgram {
  unsigned M = 0, na = 0, nb = 0;
  uint64_t Ca = 0, Cb = 0;
  unsigned order = 1, steps = 1;
  bool apply_unitary_order = false;  // applyUnitary's term order (iterative QPE)
  std::vector<AxisTable> tables;
  uint64_t pool_words = 0;
  std::vector<DevOp> ops;      // one forward Trotter sweep
  std::vector<double> coefs;   // 8 doubles per term record (general matrices)
  std::vector<Pass> passes;    // one forward Trotter sweep
  uint32_t ops_per_sweep = 0;
  uint64_t touches_per_sweep = 0;
  uint64_t touches_per_power = 0;
};

uint64_t binom(int n, int k);

void build_program(HostProgram& P, unsigned M, unsigned na, unsigned nb, const TermArrays& T,
                   unsigned order, unsigned steps);

}  // namespace qpe

#endif  // QPE_PROGRAM_BUILD_H_
