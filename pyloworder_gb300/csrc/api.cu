// Library-wide C-ABI entries: version and per-thread error string.
#include "plom_common.cuh"

namespace plom {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

const char* last_error() { return g_err; }

}  // namespace plom

extern "C" const char* plom_last_error_string(void) { return plom::last_error(); }
extern "C" int plom_version(void) { return 100; }
