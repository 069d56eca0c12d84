// C ABI: counters and the integer-pipe throughput probe used by the benchmark's
// roofline (the plain multi-limb kernels are bound by 32x32->64 multiply-adds).
#include "capi_util.cuh"
#include "gemm.cuh"
#include "sdpg.h"
#include "tc_gemm.cuh"

#include <map>
#include <mutex>
#include <vector>

namespace sdpg {
std::atomic<unsigned long long> g_kernel_launches{0};

void keep_pool_memory(int device) {
    static std::mutex mu;
    static bool done[64] = {};
    if (device < 0 || device >= 64) return;
    std::lock_guard<std::mutex> lock(mu);
    if (done[device]) return;
    cudaMemPool_t pool;
    SDPG_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t keep = UINT64_MAX;
    SDPG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    done[device] = true;
}

static std::mutex g_pinned_mu;
static std::map<size_t, std::vector<void *>> g_pinned_free;

void *pinned_acquire(size_t bytes) {
    {
        std::lock_guard<std::mutex> lock(g_pinned_mu);
        auto &v = g_pinned_free[bytes];
        if (!v.empty()) {
            void *p = v.back();
            v.pop_back();
            return p;
        }
    }
    void *p = nullptr;
    SDPG_CUDA(cudaMallocHost(&p, bytes));
    return p;
}

void pinned_release(void *p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> lock(g_pinned_mu);
    g_pinned_free[bytes].push_back(p);
}
}  // namespace sdpg

using namespace sdpg;

namespace {

// 16 independent signed 32x32->64 multiply-add chains per thread (IMAD.WIDE), with a
// data dependence between iterations so no multiply can be hoisted or folded.
__global__ void imad_wide_probe_kernel(const int *in, long long *out, int iters) {
    int x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = in[(threadIdx.x + 7 * k) & 255];
    int y0 = in[(threadIdx.x * 3) & 255], y1 = in[(threadIdx.x * 5 + 1) & 255];
    long long acc[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) acc[k] = k;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            acc[k] += (long long)x[k] * y0;
            acc[k + 8] += (long long)x[k] * y1;
        }
        y0 = ((int)acc[3] & 0x7fff) ^ it;
        y1 = ((int)(acc[12] >> 7) & 0x7fff) + it;
    }
    long long s = 0;
#pragma unroll
    for (int k = 0; k < 16; ++k) s ^= acc[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" {

unsigned long long sdpg_launch_count(void) { return g_kernel_launches.load(); }

int sdpg_set_gemm_method(int method) {
    return sdpg_guard([&] {
        if (method < 0 || method > 2) throw sdpg_error(SDPG_ERR_ARG, "method must be 0, 1 or 2");
        const int old = g_gemm_method;
        g_gemm_method = method;
        return old;
    });
}

long long sdpg_set_tensor_wait_budget(long long cycles) {
    const long long old = g_tc_wait_cycles;
    g_tc_wait_cycles = cycles > 0 ? cycles : 0;
    return old;
}

int sdpg_tensor_error(int device, int *flag) {
    return sdpg_guard([&] {
        if (!flag) throw sdpg_error(SDPG_ERR_ARG, "null output");
        SDPG_CUDA(cudaSetDevice(device));
        SDPG_CUDA(cudaMemcpy(flag, crt_error_word(), sizeof(int), cudaMemcpyDeviceToHost));
        return (int)SDPG_OK;
    });
}

int sdpg_probe_imad_wide(int device, double *ops_per_second) {
    return sdpg_guard([&] {
        if (!ops_per_second) throw sdpg_error(SDPG_ERR_ARG, "null output");
        SDPG_CUDA(cudaSetDevice(device));
        int sms = 0;
        SDPG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        const int blocks = sms * 8, threads = 256, iters = 8192;
        DeviceBuffer in(256 * sizeof(int)), out((size_t)blocks * threads * sizeof(long long));
        int h[256];
        for (int i = 0; i < 256; ++i) h[i] = 1000003 * i + 17;
        SDPG_CUDA(cudaMemcpy(in.p, h, sizeof h, cudaMemcpyHostToDevice));
        cudaEvent_t a, b;
        SDPG_CUDA(cudaEventCreate(&a));
        SDPG_CUDA(cudaEventCreate(&b));
        imad_wide_probe_kernel<<<blocks, threads>>>((const int *)in.p, (long long *)out.p, 256);  // warm-up
        SDPG_CHECK_LAUNCH();
        float best = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            SDPG_CUDA(cudaEventRecord(a));
            imad_wide_probe_kernel<<<blocks, threads>>>((const int *)in.p, (long long *)out.p, iters);
            SDPG_CHECK_LAUNCH();
            SDPG_CUDA(cudaEventRecord(b));
            SDPG_CUDA(cudaEventSynchronize(b));
            float ms = 0;
            SDPG_CUDA(cudaEventElapsedTime(&ms, a, b));
            if (ms < best) best = ms;
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        *ops_per_second = (double)blocks * threads * iters * 16.0 / (best * 1e-3);
        return (int)SDPG_OK;
    });
}

}  // extern "C"

// ---- per-kernel timing ------------------------------------------------------------

namespace sdpg {

std::atomic<bool> g_kt_on{false};

namespace kt_detail {

struct KtPair {
    const char *name;
    int device;
    cudaEvent_t a, b;
    double work;
};

std::mutex g_kt_mu;
std::vector<KtPair> g_kt_pairs;           // recorded, not yet read
std::vector<std::pair<int, cudaEvent_t>> g_kt_free;  // (device, event) ready for reuse
thread_local std::vector<std::pair<cudaStream_t, cudaEvent_t>> t_kt_open;  // begun, not ended

cudaEvent_t kt_event(int dev) {
    {
        std::lock_guard<std::mutex> lock(g_kt_mu);
        for (size_t i = 0; i < g_kt_free.size(); ++i)
            if (g_kt_free[i].first == dev) {
                cudaEvent_t e = g_kt_free[i].second;
                g_kt_free[i] = g_kt_free.back();
                g_kt_free.pop_back();
                return e;
            }
    }
    cudaEvent_t e;
    SDPG_CUDA(cudaEventCreate(&e));
    return e;
}

bool capturing(cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(s, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone;
}

}  // namespace kt_detail

using namespace kt_detail;

void kt_begin(cudaStream_t s) {
    if (capturing(s)) return;
    int dev = 0;
    SDPG_CUDA(cudaGetDevice(&dev));
    cudaEvent_t e = kt_event(dev);
    SDPG_CUDA(cudaEventRecord(e, s));
    t_kt_open.emplace_back(s, e);
}

void kt_end(const char *name, cudaStream_t s, double work) {
    for (size_t i = t_kt_open.size(); i-- > 0;) {
        if (t_kt_open[i].first != s) continue;
        cudaEvent_t a = t_kt_open[i].second;
        t_kt_open.erase(t_kt_open.begin() + (long)i);
        int dev = 0;
        SDPG_CUDA(cudaGetDevice(&dev));
        cudaEvent_t b = kt_event(dev);
        SDPG_CUDA(cudaEventRecord(b, s));
        std::lock_guard<std::mutex> lock(g_kt_mu);
        g_kt_pairs.push_back(KtPair{name, dev, a, b, work});
        return;
    }
}

}  // namespace sdpg

extern "C" {

int sdpg_kernel_timing(int enable) {
    const bool old = sdpg::g_kt_on.exchange(enable != 0);
    return old ? 1 : 0;
}

int sdpg_kernel_times(char *buf, int cap) {
    using namespace sdpg::kt_detail;
    return sdpg_guard([&] {
        if (!buf || cap <= 0) throw sdpg_error(SDPG_ERR_ARG, "null buffer");
        std::vector<KtPair> pairs;
        {
            std::lock_guard<std::mutex> lock(g_kt_mu);
            pairs.swap(g_kt_pairs);
        }
        struct Agg {
            long long launches = 0;
            double ms = 0, work = 0;
        };
        std::map<std::string, Agg> agg;
        int dev0 = 0;
        SDPG_CUDA(cudaGetDevice(&dev0));
        for (const KtPair &p : pairs) {
            SDPG_CUDA(cudaSetDevice(p.device));
            SDPG_CUDA(cudaEventSynchronize(p.b));
            float ms = 0;
            SDPG_CUDA(cudaEventElapsedTime(&ms, p.a, p.b));
            Agg &v = agg[p.name];
            v.launches += 1;
            v.ms += ms;
            v.work += p.work;
        }
        SDPG_CUDA(cudaSetDevice(dev0));
        {
            std::lock_guard<std::mutex> lock(g_kt_mu);
            for (const KtPair &p : pairs) {
                g_kt_free.emplace_back(p.device, p.a);
                g_kt_free.emplace_back(p.device, p.b);
            }
        }
        std::string out;
        for (const auto &kv : agg) {
            char line[256];
            snprintf(line, sizeof line, "%s %lld %.6f %.6e\n", kv.first.c_str(), kv.second.launches, kv.second.ms,
                     kv.second.work);
            out += line;
        }
        if ((int)out.size() + 1 > cap) throw sdpg_error(SDPG_ERR_TOO_LARGE, "buffer too small");
        memcpy(buf, out.c_str(), out.size() + 1);
        return (int)agg.size();
    });
}

}  // extern "C"
