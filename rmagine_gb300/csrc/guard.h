// The exception guard of the C entry points (host code only).
#pragma once

#include <exception>
#include <new>
#include <string>

namespace rmg {

int fail(int status, const std::string& msg);

// Runs the body of a C entry point: no C++ exception may cross the C ABI, so
// a failed host allocation becomes RMG_ERR_OOM and any other exception
// RMG_ERR_CUDA, with the message in rmg_last_error().
template <typename F>
int guarded(const char* what, F&& body) {
  try {
    return body();
  } catch (const std::bad_alloc&) {
    return fail(RMG_ERR_OOM, std::string(what) + ": host allocation failed");
  } catch (const std::exception& e) {
    return fail(RMG_ERR_CUDA, std::string(what) + ": " + e.what());
  } catch (...) {
    return fail(RMG_ERR_CUDA, std::string(what) + ": unexpected exception");
  }
}

}  // namespace rmg
