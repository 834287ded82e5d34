// kmc_abi_guard.h -- C++ exceptions stop at the C ABI.
//
// Every exported function returns a status (include/cntkmc.h), but its C++ body can throw: a host
// vector sized from the caller's arguments (std::bad_alloc, std::length_error), or a standard
// library call.  An exception must not unwind into a C caller (it would end the process in
// std::terminate), so each exported definition is a function-try-block whose handler turns the
// exception being handled into a status:
//   std::bad_alloc, std::length_error  -> KMC_ERR_NOMEM ("host allocation failed")
//   any other exception                 -> KMC_ERR_ARG, with its what() as the message.
#pragma once
#include <exception>
#include <new>
#include <stdexcept>

#include "../../include/cntkmc.h"

namespace kmc {

// The status of the exception being handled; *what gets a message that stays valid until the
// enclosing handler ends.  Call it only inside a catch handler.
inline int abi_status(const char** what) noexcept {
  try {
    throw;
  } catch (const std::bad_alloc&) {
    *what = "host allocation failed";
    return KMC_ERR_NOMEM;
  } catch (const std::length_error&) {
    *what = "host allocation failed (size too large)";
    return KMC_ERR_NOMEM;
  } catch (const std::exception& e) {
    *what = e.what();
    return KMC_ERR_ARG;
  } catch (...) {
    *what = "unknown C++ exception";
    return KMC_ERR_ARG;
  }
}

// abi_status for entry points with a context: the message "<fn>: <what>" goes to the context's
// kmc_last_error (when it can be stored).  Defined in cntkmc_api.cu.
int abi_fail(kmc_ctx* c, const char* fn) noexcept;

}  // namespace kmc
