// errors.h -- the library's per-thread error message (read through phx_last_error()).
#pragma once

#include <string>

namespace phx {

// Records msg as this thread's last error and returns code.
int set_last_error(int code, const std::string& msg);

}  // namespace phx
