// qpe_common.h - error plumbing shared by the C ABI implementation files.
// Every exported function converts exceptions into an int status plus a
// thread-local message (qpe_last_error), so no exception crosses the C ABI.
#ifndef QPE_COMMON_H_
#define QPE_COMMON_H_

#include <exception>
#include <new>
#include <stdexcept>
#include <string>

#include "../../include/qpe_gb300.h"

namespace qpe {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

inline int fail(int code, const std::string& msg) {
  set_last_error(msg);
  return code;
}

template <class F>
int guard(F&& f) {
  try {
    f();
    return QPE_OK;
  } catch (const Error& e) {
    return fail(e.code, e.what());
  } catch (const std::bad_alloc&) {
    return fail(QPE_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(QPE_ERR_INVALID, e.what());
  } catch (...) {
    return fail(QPE_ERR_INVALID, "unknown error");
  }
}

}  // namespace qpe

#endif  // QPE_COMMON_H_
