// Library-wide state: per-thread error text, launch counter, host-side fault injection, kernel timing.
#include "hx_common.cuh"

#include <atomic>
#include <cstdarg>
#include <cstdlib>
#include <mutex>
#include <vector>

namespace {
thread_local char g_error[1024] = "";
std::atomic<long long> g_launches{0};

struct TraceRecord {
    int kind;
    double work;
    cudaEvent_t start, stop;
};
std::atomic<bool> g_trace_on{false};
std::mutex g_trace_mu;
std::vector<TraceRecord> g_trace;
}  // namespace

namespace hx {

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
}

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

bool trace_on() { return g_trace_on.load(std::memory_order_relaxed); }

int trace_begin(int kind, double work, cudaStream_t stream) {
    TraceRecord r{kind, work, nullptr, nullptr};
    if (cudaEventCreate(&r.start) != cudaSuccess) return -1;
    if (cudaEventCreate(&r.stop) != cudaSuccess) {
        cudaEventDestroy(r.start);
        return -1;
    }
    cudaEventRecord(r.start, stream);
    std::lock_guard<std::mutex> lock(g_trace_mu);
    g_trace.push_back(r);
    return (int)g_trace.size() - 1;
}

void trace_end(int record, cudaStream_t stream) {
    std::lock_guard<std::mutex> lock(g_trace_mu);
    if (record >= 0 && record < (int)g_trace.size()) cudaEventRecord(g_trace[record].stop, stream);
}

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

int hx_trace_enable(int on) {
    g_trace_on.store(on != 0, std::memory_order_relaxed);
    return HX_OK;
}

int hx_trace_read(int kind, long long* launches, double* total_ms, double* total_work, int reset) {
    long long n = 0;
    double ms = 0.0, work = 0.0;
    std::lock_guard<std::mutex> lock(g_trace_mu);
    for (const TraceRecord& r : g_trace) {
        if (r.kind != kind) continue;
        float t = 0.0f;
        if (cudaEventSynchronize(r.stop) != cudaSuccess || cudaEventElapsedTime(&t, r.start, r.stop) != cudaSuccess) {
            hx::set_error("hx_trace_read: %s", cudaGetErrorString(cudaGetLastError()));
            return HX_ERR_CUDA;
        }
        ++n;
        ms += t;
        work += r.work;
    }
    if (reset) {
        std::vector<TraceRecord> keep;
        for (const TraceRecord& r : g_trace) {
            if (r.kind == kind) {
                cudaEventDestroy(r.start);
                cudaEventDestroy(r.stop);
            } else {
                keep.push_back(r);
            }
        }
        g_trace.swap(keep);
    }
    if (launches) *launches = n;
    if (total_ms) *total_ms = ms;
    if (total_work) *total_work = work;
    return HX_OK;
}

}  // extern "C"
