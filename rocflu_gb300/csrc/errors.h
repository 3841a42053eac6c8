// Last-error message of the C ABI (rflu_gpu_last_error) and the helper that
// records it; every failing entry point returns a negative RFLU_ERR_* code.
#pragma once
#include <string>

namespace rflu {
std::string &lastError();
inline int fail(int code, const std::string &msg) {
  lastError() = msg;
  return code;
}
}  // namespace rflu
