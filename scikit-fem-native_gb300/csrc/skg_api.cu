// Library-wide C ABI entry points: version and per-thread last error.
#include <string>

#include "skg_common.cuh"

namespace skg {
namespace {
thread_local std::string g_last_error;
}
void set_last_error(const std::string &msg) { g_last_error = msg; }
}  // namespace skg

extern "C" int skg_version(void) { return 100; }

extern "C" const char *skg_last_error(void) { return skg::g_last_error.c_str(); }
