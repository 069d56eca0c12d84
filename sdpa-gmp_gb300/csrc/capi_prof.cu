// C ABI: counters and the integer-pipe throughput probe used by the benchmark's
// roofline (the plain multi-limb kernels are bound by 32x32->64 multiply-adds).
#include "capi_util.cuh"
#include "gemm.cuh"
#include "sdpg.h"
#include "tc_gemm.cuh"
#include "tcgen05.cuh"

#include <algorithm>
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

// ---- tensor-instruction throughput probes -------------------------------------------
//
// Which tensor instruction carries the residue GEMM was settled by these rates.
// sdpg_probe_tensor_rate(kind):
//   0  tcgen05.mma kind::f16 (fp16 x fp16 -> fp32 in tensor memory), the residue GEMM's
//      instruction: one CTA per SM; one thread issues `rounds` x 4 products of
//      M = 128, N = 256, K = 16 into one accumulator from fixed shared-memory operands
//      (no memory traffic), then waits for them on an mbarrier (bounded).
//   1  mma.sync m16n8k32 s8 x s8 -> s32, the 8-bit integer tensor instruction this target
//      accepts (ptxas rejects tcgen05.mma kind::i8 for sm_103a).
//   2  mma.sync m16n8k16 f16 x f16 -> f32, the legacy form of kind 0.
constexpr int kProbeN = 256;
constexpr int kProbeTileA = 128 * 128;  // 128 rows of one 128-byte swizzle row
constexpr int kProbeTileB = kProbeN * 128;
constexpr int kProbeSmem = kProbeTileA + kProbeTileB + 1024 + 64;
constexpr int kProbeRounds = 2048;
// shared memory requested per CTA: more than half the SM's, so each SM holds one CTA
constexpr int kProbeSmemLaunch = 120 * 1024;
static_assert(kProbeSmem <= kProbeSmemLaunch, "probe shared memory");

__global__ void __launch_bounds__(128, 1) tc_f16_rate_probe_kernel(int rounds, int *status) {
    using namespace tc;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *tA = smem, *tB = smem + kProbeTileA;
    uint64_t *bar = (uint64_t *)(tB + kProbeTileB);
    uint32_t *slot = (uint32_t *)(bar + 1);
    const int t = threadIdx.x;
    // operands: fp16 ones and zeros (the values do not matter for the rate)
    for (int i = t; i < (kProbeTileA + kProbeTileB) / 16; i += blockDim.x)
        reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0x3C003C00u, 0u, 0x00003C00u, 0u);
    if (t == 0) {
        mbar_init(smem_u32(bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (t < 32) {
        tmem_alloc(smem_u32(slot), kProbeN);
        tmem_relinquish();
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    if (t == 0) {
        const uint64_t ad = sw128_kmajor_desc(smem_u32(tA)), bd = sw128_kmajor_desc(smem_u32(tB));
        constexpr uint32_t idesc = idesc_f16_f32(128, kProbeN);
        for (int r = 0; r < rounds; ++r) {
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                tc_mma(tmem, ad + (uint64_t)(2 * kk), bd + (uint64_t)(2 * kk), idesc, (r | kk) ? 1u : 0u);
        }
        tc_commit(smem_u32(bar));
        // the products are issued: wait for them with the full budget, and once more if
        // that ran out, so none is in flight when the tensor memory is freed
        if (!mbar_wait(smem_u32(bar), 0)) {
            atomicExch(status, 1);
            mbar_wait(smem_u32(bar), 0);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (t < 32) {
        tc_fence_after();
        tmem_dealloc(tmem, kProbeN);
    }
}

// Eight independent accumulator chains per warp; each mma depends on its own previous
// result only, so the loop cannot be folded.
template <bool kInt8>
__global__ void mma_sync_rate_probe_kernel(int iters, uint32_t seed, uint32_t *out) {
    const uint32_t x = seed ^ (threadIdx.x * 0x9E3779B9u) ^ blockIdx.x;
    const uint32_t a0 = x & 0x3F3F3F3Fu, a1 = (x >> 3) & 0x3F3F3F3Fu, a2 = (x >> 5) & 0x3F3F3F3Fu,
                   a3 = (x >> 7) & 0x3F3F3F3Fu;
    const uint32_t b0 = (x * 3u) & 0x3F3F3F3Fu, b1 = (x * 5u) & 0x3F3F3F3Fu;
    uint32_t acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[j][q] = 0u;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if constexpr (kInt8) {
                asm volatile(
                    "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
                    "{%8, %9}, {%0, %1, %2, %3};"
                    : "+r"(acc[j][0]), "+r"(acc[j][1]), "+r"(acc[j][2]), "+r"(acc[j][3])
                    : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
            } else {
                // fp16 operands: the low bits of x as normal numbers in [0.5, 1)
                asm volatile(
                    "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
                    "{%8, %9}, {%0, %1, %2, %3};"
                    : "+r"(acc[j][0]), "+r"(acc[j][1]), "+r"(acc[j][2]), "+r"(acc[j][3])
                    : "r"((a0 & 0x03FF03FFu) | 0x38003800u), "r"((a1 & 0x03FF03FFu) | 0x38003800u),
                      "r"((a2 & 0x03FF03FFu) | 0x38003800u), "r"((a3 & 0x03FF03FFu) | 0x38003800u),
                      "r"((b0 & 0x03FF03FFu) | 0x38003800u), "r"((b1 & 0x03FF03FFu) | 0x38003800u));
            }
        }
    }
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) s ^= acc[j][q];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" {

unsigned long long sdpg_launch_count(void) { return g_kernel_launches.load(); }

int sdpg_probe_tensor_rate(int device, int kind, double *ops_per_second) {
    return sdpg_guard([&] {
        if (!ops_per_second) throw sdpg_error(SDPG_ERR_ARG, "null output");
        if (kind < 0 || kind > 2) throw sdpg_error(SDPG_ERR_ARG, "kind must be 0, 1 or 2");
        SDPG_CUDA(cudaSetDevice(device));
        int sms = 0;
        SDPG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        cudaEvent_t a, b;
        SDPG_CUDA(cudaEventCreate(&a));
        SDPG_CUDA(cudaEventCreate(&b));
        float best = 1e30f;
        double ops = 0;
        if (kind == 0) {
            DeviceBuffer st(sizeof(int));
            SDPG_CUDA(cudaMemset(st.p, 0, sizeof(int)));
            SDPG_CUDA(cudaFuncSetAttribute(tc_f16_rate_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           kProbeSmemLaunch));
            tc_f16_rate_probe_kernel<<<sms, 128, kProbeSmemLaunch>>>(64, (int *)st.p);  // warm-up
            SDPG_CHECK_LAUNCH();
            for (int rep = 0; rep < 3; ++rep) {
                SDPG_CUDA(cudaEventRecord(a));
                tc_f16_rate_probe_kernel<<<sms, 128, kProbeSmemLaunch>>>(kProbeRounds, (int *)st.p);
                SDPG_CHECK_LAUNCH();
                SDPG_CUDA(cudaEventRecord(b));
                SDPG_CUDA(cudaEventSynchronize(b));
                float ms = 0;
                SDPG_CUDA(cudaEventElapsedTime(&ms, a, b));
                best = std::min(best, ms);
            }
            int h = 0;
            SDPG_CUDA(cudaMemcpy(&h, st.p, sizeof(int), cudaMemcpyDeviceToHost));
            if (h) throw sdpg_error(SDPG_ERR_TIMEOUT, "tensor-rate probe: a bounded wait gave up");
            ops = (double)sms * kProbeRounds * 4 * (2.0 * 128 * kProbeN * 16);
        } else {
            const int blocks = sms * 4, threads = 256, iters = 4096;
            DeviceBuffer out((size_t)blocks * threads * sizeof(uint32_t));
            auto launch = [&](int it) {
                if (kind == 1)
                    mma_sync_rate_probe_kernel<true><<<blocks, threads>>>(it, 12345u, (uint32_t *)out.p);
                else
                    mma_sync_rate_probe_kernel<false><<<blocks, threads>>>(it, 12345u, (uint32_t *)out.p);
                SDPG_CHECK_LAUNCH();
            };
            launch(64);  // warm-up
            for (int rep = 0; rep < 3; ++rep) {
                SDPG_CUDA(cudaEventRecord(a));
                launch(iters);
                SDPG_CUDA(cudaEventRecord(b));
                SDPG_CUDA(cudaEventSynchronize(b));
                float ms = 0;
                SDPG_CUDA(cudaEventElapsedTime(&ms, a, b));
                best = std::min(best, ms);
            }
            const double per_mma = kind == 1 ? 2.0 * 16 * 8 * 32 : 2.0 * 16 * 8 * 16;
            ops = (double)blocks * (threads / 32) * iters * 8 * per_mma;
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        *ops_per_second = ops / (best * 1e-3);
        return (int)SDPG_OK;
    });
}

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
