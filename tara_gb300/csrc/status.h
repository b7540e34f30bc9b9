// The thread-local status behind tara_last_error / tara_last_error_message
// (defined in solver2d.cu), for host code with and without CUDA.
#pragma once
#include <string>

namespace tara {

int set_error(int code, const std::string& msg);
int set_ok();

// The status across a cleanup that records its own: a public destroy reports
// success, so a create that fails, or a driver that leaves a run on an error,
// saves the error before freeing its handle and restores it after.
struct ErrorState {
  int code;
  std::string msg;
};
ErrorState save_error();
void restore_error(const ErrorState& s);

}  // namespace tara
