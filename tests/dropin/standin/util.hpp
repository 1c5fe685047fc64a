// util.hpp (test stand-in) - the one helper of the reference's cpp/util.hpp that
// the drop-in headers and the drop-in driver use, for building them where the
// reference sources are absent: nChoosek (cpp/util.hpp:49-60), the number of
// k-element subsets of n elements.
#ifndef QPE_DROPIN_STANDIN_UTIL_HPP_
#define QPE_DROPIN_STANDIN_UTIL_HPP_

#include <cstdint>

inline uint64_t nChoosek(uint64_t n, uint64_t k) {
  if (k > n) return 0;
  uint64_t r = 1;
  for (uint64_t i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

#endif  // QPE_DROPIN_STANDIN_UTIL_HPP_
