// timing.cu -- kernel launch counter and optional CUDA-event timing of the
// hot kernels (used by the benchmark to measure the dominant kernel's
// duration live, and by tests).  Off by default: when disabled a timed scope
// costs one branch.  Also the L2 gather probe (k_l2_gather_probe): the rate
// of random 32-byte loads from an L2-resident buffer, the ceiling of the DAS
// interpolation kernels.
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

// ---------------------------------------------------------------------------
// L2 gather probe: throughput of random 32-byte-sector loads from a buffer
// that stays resident in L2 -- the ceiling of the DAS kernels, whose image
// and sinogram gathers are served by L2, not HBM.
// ---------------------------------------------------------------------------
namespace msot {

__global__ void k_l2_gather_probe(const float4 *__restrict__ buf, unsigned n_sectors, int iters,
                                  unsigned seed, float *sink) {
    unsigned h = seed ^ ((blockIdx.x * blockDim.x + threadIdx.x) * 2654435761u);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = 0; i < iters; ++i) {
        h = h * 1664525u + 1013904223u;
        const unsigned s = h % n_sectors;
        const float4 a = __ldg(buf + 2 * (size_t)s), b = __ldg(buf + 2 * (size_t)s + 1);
        acc.x += a.x + b.x;
        acc.y += a.y + b.y;
        acc.z += a.z + b.z;
        acc.w += a.w + b.w;
    }
    if (acc.x + acc.y + acc.z + acc.w == 1234.5f) sink[0] = acc.x;  // keeps the loads
}

}  // namespace msot

extern "C" int msot_l2_gather_probe(size_t buffer_bytes, double *gbs) {
    using namespace msot;
    if (!gbs || buffer_bytes < 1024 * 1024 || buffer_bytes > (size_t)96 * 1024 * 1024) {
        set_error("l2_gather_probe: buffer of 1 .. 96 MiB");
        return MSOT_EINVAL;
    }
    float4 *buf = nullptr;
    float *sink = nullptr;
    MSOT_CUDA_TRY(cudaMalloc(&buf, buffer_bytes));
    if (cudaMalloc(&sink, sizeof(float)) != cudaSuccess) {
        cudaFree(buf);
        set_error("l2_gather_probe: allocation failed");
        return MSOT_ENOMEM;
    }
    const unsigned n_sectors = (unsigned)(buffer_bytes / 32);
    int dev = 0, sms = 0;
    cudaEvent_t a = nullptr, b = nullptr;
    cudaError_t e = cudaMemset(buf, 0, buffer_bytes);
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    float ms = 0.f;
    if (e == cudaSuccess) {
        const dim3 grid((unsigned)sms * 16), block(256);
        const int iters = 64, reps = 20;
        for (int w = 0; w < 3; ++w)  // warm-up: brings the buffer into L2
            KLAUNCH(k_l2_gather_probe<<<grid, block>>>(buf, n_sectors, iters, 7u + w, sink));
        cudaEventRecord(a);
        for (int r = 0; r < reps; ++r)
            KLAUNCH(k_l2_gather_probe<<<grid, block>>>(buf, n_sectors, iters, 100u + r, sink));
        cudaEventRecord(b);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        *gbs = (double)grid.x * block.x * iters * 32.0 * reps / (ms * 1e-3) / 1e9;
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaFree(buf);
    cudaFree(sink);
    if (e != cudaSuccess) {
        set_error("l2_gather_probe: %s", cudaGetErrorString(e));
        return MSOT_ECUDA;
    }
    return MSOT_OK;
}
