// Launch accounting and optional per-kernel-class timing.
//
// Every kernel launch of the library goes through prof_before/prof_after.
// A global counter always counts launches.  When timing is enabled,
// CUDA events are recorded on the launching stream around each launch and
// the algorithmic flop count of the launch is stored with them, so a caller
// (the benchmark) can read per-class device time and achieved throughput
// without an external profiler.
#include <atomic>
#include <mutex>
#include <vector>

#include "sgb_internal.cuh"

namespace sgb {

namespace {

struct Rec {
    int kclass;
    cudaEvent_t a, b;
    double flops;
    double issued;
};

std::atomic<long long> g_launches{0};
constexpr unsigned kAllClasses = (1u << SGB_KCLASS_COUNT) - 1u;
std::atomic<unsigned> g_mask{0};  // kernel classes timed
std::mutex g_mu;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;
thread_local cudaEvent_t t_start = nullptr;

cudaEvent_t get_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void recycle_locked() {
    for (auto& r : g_recs) {
        g_pool.push_back(r.a);
        g_pool.push_back(r.b);
    }
    g_recs.clear();
}

}  // namespace

namespace {
constexpr long long kDefaultSpin = 1ll << 22;
std::atomic<long long> g_spin{kDefaultSpin};
}  // namespace

long long spin_limit() { return g_spin.load(std::memory_order_relaxed); }

bool capturing(cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(s, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone;
}

void prof_before(cudaStream_t s, int kclass) {
    const unsigned mask = g_mask.load(std::memory_order_relaxed);
    if (mask == 0) return;
    // launches that do not name their class are timed only when all are
    if (kclass >= 0 ? !(mask & (1u << kclass)) : mask != kAllClasses) return;
    if (capturing(s)) return;
    std::lock_guard<std::mutex> lk(g_mu);
    t_start = get_event();
    cudaEventRecord(t_start, s);
}

void prof_after(int kclass, cudaStream_t s, double flops, double issued) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (t_start == nullptr) return;
    std::lock_guard<std::mutex> lk(g_mu);
    cudaEvent_t e = get_event();
    cudaEventRecord(e, s);
    g_recs.push_back(Rec{kclass, t_start, e, flops, issued});
    t_start = nullptr;
}

}  // namespace sgb

using namespace sgb;

extern "C" {

long long sgb_launch_count(void) { return g_launches.load(); }

long long sgb_debug_spin_limit(long long polls) {
    if (polls < 0) return g_spin.load();
    if (polls > (1ll << 40)) polls = 1ll << 40;
    return g_spin.exchange(polls);
}

int sgb_profile_enable(int on) { return sgb_profile_enable_classes(on ? kAllClasses : 0u); }

int sgb_profile_enable_classes(unsigned mask) {
    std::lock_guard<std::mutex> lk(g_mu);
    recycle_locked();
    g_mask.store(mask & kAllClasses);
    return SGB_OK;
}

int sgb_profile_read(int kclass, long long* launches, double* ms, double* flops) {
    if (kclass < 0 || kclass >= SGB_KCLASS_COUNT || !launches || !ms || !flops) return SGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_mu);
    long long n = 0;
    double t = 0.0, f = 0.0;
    for (auto& r : g_recs) {
        if (r.kclass != kclass) continue;
        if (cudaEventSynchronize(r.b) != cudaSuccess) return SGB_ERR_CUDA;
        float x = 0.f;
        if (cudaEventElapsedTime(&x, r.a, r.b) != cudaSuccess) return SGB_ERR_CUDA;
        ++n;
        t += x;
        f += r.flops;
    }
    *launches = n;
    *ms = t;
    *flops = f;
    return SGB_OK;
}

int sgb_profile_read_issued(int kclass, double* issued) {
    if (kclass < 0 || kclass >= SGB_KCLASS_COUNT || !issued) return SGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_mu);
    double f = 0.0;
    for (auto& r : g_recs)
        if (r.kclass == kclass) f += r.issued;
    *issued = f;
    return SGB_OK;
}

}  // extern "C"
