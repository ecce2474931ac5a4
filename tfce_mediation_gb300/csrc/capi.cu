// Library-wide C-ABI pieces: version and per-thread error message.
#include <cstring>

#include "common.cuh"

namespace tfgb {

namespace {
thread_local char g_err[512] = {0};
}

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

void clear_error() { g_err[0] = '\0'; }

}  // namespace tfgb

extern "C" {

int tfce_version(void) { return 100; }  // 0.1.0

const char* tfce_last_error(void) { return tfgb::g_err; }

}  // extern "C"
