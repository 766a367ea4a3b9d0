// Launch accounting and optional per-kernel CUDA-event timing (the GPU
// analogue of the reference's @timer, dedalus/utils/timer.py:29-65).
//
// Every kernel launch in the library goes through kt_begin / kt_end.  The
// launch counter is always on; event timing only when dd_timing_enable(1):
// then each launch is bracketed by two events on its own stream and
// dd_timing_report() synchronises them and sums the device time per label.
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "dd_common.cuh"
#include "timing.cuh"

namespace dd {

namespace {
struct Pending {
    const char* label;
    cudaEvent_t a, b;
};
struct Stat {
    long long count = 0;
    double ms = 0.0;
};
std::mutex g_mu;
bool g_on = false;
long long g_launches = 0;
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_pool;
std::unordered_map<std::string, Stat> g_stats;

cudaEvent_t take_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

void drain_locked() {
    for (auto& p : g_pending) {
        cudaEventSynchronize(p.b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.a, p.b);
        Stat& s = g_stats[p.label];
        s.count += 1;
        s.ms += ms;
        g_pool.push_back(p.a);
        g_pool.push_back(p.b);
    }
    g_pending.clear();
}
}  // namespace

int kt_begin(const char* label, cudaStream_t st) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_launches += 1;
    if (!g_on) return -1;
    if (g_pending.size() > 100000) drain_locked();
    Pending p{label, take_event(), take_event()};
    cudaEventRecord(p.a, st);
    g_pending.push_back(p);
    return (int)g_pending.size() - 1;
}

void kt_end(int slot, cudaStream_t st) {
    if (slot < 0) return;
    std::lock_guard<std::mutex> lk(g_mu);
    if (slot < (int)g_pending.size()) cudaEventRecord(g_pending[slot].b, st);
}

}  // namespace dd

using namespace dd;

extern "C" {

int dd_timing_enable(int on) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_on = on != 0;
    return DD_OK;
}

int dd_timing_reset(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    drain_locked();
    g_stats.clear();
    return DD_OK;
}

long long dd_launch_count(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_launches;
}

int dd_timing_report(char* buf, size_t len) {
    DD_CHECK_ARG(buf && len > 0, "dd_timing_report: null buffer");
    std::lock_guard<std::mutex> lk(g_mu);
    drain_locked();
    std::string out;
    char line[256];
    for (auto& kv : g_stats) {
        snprintf(line, sizeof(line), "%s %lld %.6f\n", kv.first.c_str(), kv.second.count, kv.second.ms);
        out += line;
    }
    DD_CHECK_ARG(out.size() + 1 <= len, "dd_timing_report: buffer too small (%zu bytes needed)", out.size() + 1);
    memcpy(buf, out.c_str(), out.size() + 1);
    return DD_OK;
}

}  // extern "C"
