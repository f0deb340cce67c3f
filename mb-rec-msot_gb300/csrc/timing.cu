// timing.cu -- kernel launch counter and optional CUDA-event timing of the
// hot kernels (used by the benchmark to measure the dominant kernel's
// duration live, and by tests).  Off by default: when disabled a timed scope
// costs one branch.
#include <atomic>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace msot {

std::atomic<long long> g_launch_count{0};

static const char *kNames[KID_COUNT] = {"prefilter", "interp_forward", "interp_adjoint",
                                        "ir_conv", "solver_vector", "permute", "tv_prox"};

struct EventPair {
    cudaEvent_t a, b;
    int kid;
};

struct Registry {
    std::mutex mu;
    bool enabled = false;
    std::vector<EventPair> pool;
    size_t used = 0;
};

static Registry &reg() {
    static Registry r;
    return r;
}

static constexpr size_t kPoolMax = 1 << 16;

bool profiling_enabled() { return reg().enabled; }

TimedScope::TimedScope(int kid, cudaStream_t st) : kid_(kid), st_(st), slot_(-1) {
    Registry &r = reg();
    if (!r.enabled) return;
    std::lock_guard<std::mutex> g(r.mu);
    if (r.used >= kPoolMax) return;
    if (r.used == r.pool.size()) {
        EventPair e{};
        if (cudaEventCreate(&e.a) != cudaSuccess || cudaEventCreate(&e.b) != cudaSuccess) return;
        r.pool.push_back(e);
    }
    slot_ = (long)r.used++;
    r.pool[slot_].kid = kid;
    cudaEventRecord(r.pool[slot_].a, st_);
}

TimedScope::~TimedScope() {
    if (slot_ < 0) return;
    cudaEventRecord(reg().pool[slot_].b, st_);
}

}  // namespace msot

using namespace msot;

extern "C" {

long long msot_launch_count(void) { return g_launch_count.load(); }

int msot_profile_enable(int on) {
    Registry &r = reg();
    std::lock_guard<std::mutex> g(r.mu);
    r.enabled = on != 0;
    r.used = 0;
    return MSOT_OK;
}

const char *msot_profile_kernel_name(int kid) {
    return (kid >= 0 && kid < KID_COUNT) ? kNames[kid] : nullptr;
}

int msot_profile_read(int kid, int *launches, double *total_ms) {
    if (kid < 0 || kid >= KID_COUNT || !launches || !total_ms) {
        set_error("profile_read: bad arguments");
        return MSOT_EINVAL;
    }
    MSOT_CUDA_TRY(cudaDeviceSynchronize());
    Registry &r = reg();
    std::lock_guard<std::mutex> g(r.mu);
    int n = 0;
    double ms = 0.0;
    for (size_t i = 0; i < r.used; ++i) {
        if (r.pool[i].kid != kid) continue;
        float t = 0.f;
        if (cudaEventElapsedTime(&t, r.pool[i].a, r.pool[i].b) == cudaSuccess) {
            ms += t;
            ++n;
        }
    }
    *launches = n;
    *total_ms = ms;
    return MSOT_OK;
}

}  // extern "C"
