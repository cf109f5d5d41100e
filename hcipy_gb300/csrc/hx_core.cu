// Library-wide state: per-thread error text, launch counter, host-side fault injection.
#include "hx_common.cuh"

#include <atomic>
#include <cstdarg>
#include <cstdlib>

namespace {
thread_local char g_error[1024] = "";
std::atomic<long long> g_launches{0};
}  // namespace

namespace hx {

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
}

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

bool fault_injected(const char* site) {
    const char* env = getenv("HX_FAULT");
    if (env == nullptr || site == nullptr) return false;
    if (strstr(env, site) == nullptr) return false;
    set_error("fault injected at '%s' (HX_FAULT=%s)", site, env);
    return true;
}

}  // namespace hx

extern "C" {

const char* hx_last_error(void) { return g_error; }

int hx_version(void) { return 100; }

long long hx_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

}  // extern "C"
