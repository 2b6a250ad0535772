// Error reporting and version entry points of the C ABI.
#include "common.cuh"

#include <atomic>
#include <string.h>

namespace fgb {

static thread_local char g_err[1024] = {0};
static std::atomic<long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

}  // namespace fgb

extern "C" {

const char* fgb_last_error(void) { return fgb::g_err; }

const char* fgb_version(void) { return "fluxgb 0.1 sm_103a"; }

long long fgb_launch_count(void) { return fgb::g_launches.load(std::memory_order_relaxed); }

}  // extern "C"
