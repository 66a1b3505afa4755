// rt_error.h — the calling thread's last-error message (rt_last_error_string),
// for translation units that are plain host C++.
#pragma once

#include <cstdint>

namespace rt {

// Records printf-style `fmt` as the calling thread's last error; returns code.
int32_t report_error(int32_t code, const char* fmt, ...);

}  // namespace rt
