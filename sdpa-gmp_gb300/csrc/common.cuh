// Shared host-side plumbing for the CUDA kernels: error codes, a growable
// device workspace, and launch helpers.
#pragma once
#include <atomic>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <stdexcept>
#include <string>

#include "ml.cuh"
#include "sdpg.h"

namespace sdpg {

struct sdpg_error : std::runtime_error {
    int code;
    sdpg_error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define SDPG_CUDA(call)                                                                        \
    do {                                                                                       \
        cudaError_t _e = (call);                                                               \
        if (_e != cudaSuccess)                                                                 \
            throw ::sdpg::sdpg_error(SDPG_ERR_CUDA,                                    \
                                     std::string(#call) + ": " + cudaGetErrorString(_e));       \
    } while (0)

// Every kernel launch in the library is followed by SDPG_CHECK_LAUNCH(), which also
// counts it (sdpg_launch_count reports the total).
extern std::atomic<unsigned long long> g_kernel_launches;
#define SDPG_CHECK_LAUNCH()                                                         \
    do {                                                                            \
        ::sdpg::g_kernel_launches.fetch_add(1, std::memory_order_relaxed);          \
        SDPG_CUDA(cudaGetLastError());                                              \
    } while (0)

// Per-kernel timing (sdpg_kernel_timing): while on, every launch site brackets its
// kernel with a pair of CUDA events on the launching stream (none inside a stream
// capture) and the pairs are summed per kernel name when read.
extern std::atomic<bool> g_kt_on;
void kt_begin(cudaStream_t s);
void kt_end(const char *name, cudaStream_t s, double work = 0);
#define SDPG_KT_BEGIN(s)                                                            \
    do {                                                                            \
        if (::sdpg::g_kt_on.load(std::memory_order_relaxed)) ::sdpg::kt_begin(s);   \
    } while (0)
#define SDPG_CHECK_LAUNCH_KT(name, s)                                                   \
    do {                                                                                \
        SDPG_CHECK_LAUNCH();                                                            \
        if (::sdpg::g_kt_on.load(std::memory_order_relaxed)) ::sdpg::kt_end(name, s);   \
    } while (0)
// the same, with the launch's algorithmic work (bytes or flops, per kernel) recorded
#define SDPG_CHECK_LAUNCH_KTW(name, s, work)                                                  \
    do {                                                                                      \
        SDPG_CHECK_LAUNCH();                                                                  \
        if (::sdpg::g_kt_on.load(std::memory_order_relaxed)) ::sdpg::kt_end(name, s, work);   \
    } while (0)

// Device scratch that only grows; one per problem handle (or per C-ABI call).  With an
// allocation stream set, memory comes from the device's stream-ordered pool
// (cudaMallocAsync / cudaFreeAsync), so creating and destroying solvers does not
// synchronise the device under other solvers' work.
struct Workspace {
    char *base = nullptr;
    size_t cap = 0;
    size_t used = 0;
    cudaStream_t stream = nullptr;
    // device word that tensor-core GEMMs run out of this workspace set when one of their
    // bounded waits gives up (null: only the device-wide flag of crt_error_word())
    int *error = nullptr;
    // side stream and events of the look-ahead Cholesky (ml_potrf), created on first use
    // (a factorisation's first run is never inside a stream capture)
    cudaStream_t side = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    Workspace() = default;
    Workspace(const Workspace &) = delete;
    Workspace &operator=(const Workspace &) = delete;
    ~Workspace() {
        release();
        if (side) cudaStreamDestroy(side);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
    void ensure_side() {
        if (side) return;
        SDPG_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
        for (cudaEvent_t &e : ev) SDPG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    void release() {
        if (base) {
            if (stream) cudaFreeAsync(base, stream);
            else cudaFree(base);
        }
        base = nullptr;
        cap = 0;
        used = 0;
    }
    void reserve(size_t bytes) {
        if (bytes <= cap) return;
        if (base) {
            if (!stream) SDPG_CUDA(cudaDeviceSynchronize());
            release();
        }
        if (stream) SDPG_CUDA(cudaMallocAsync((void **)&base, bytes, stream));
        else SDPG_CUDA(cudaMalloc(&base, bytes));
        cap = bytes;
    }
    // carve `bytes` (256-aligned) out of a reservation of `total` made beforehand
    void *carve(size_t bytes) {
        size_t off = (used + 255) & ~(size_t)255;
        if (off + bytes > cap) throw sdpg_error(SDPG_ERR_TOO_LARGE, "workspace exhausted");
        used = off + bytes;
        return base + off;
    }
    void reset() { used = 0; }
};

// Keep memory freed to the device's default pool cached there (instead of returning it
// to the driver at every synchronisation), once per device.
void keep_pool_memory(int device);

// Page-locked host staging buffers of `bytes`, recycled across solvers (allocating
// page-locked memory is slow and serialises); released buffers stay in the pool.
void *pinned_acquire(size_t bytes);
void pinned_release(void *p, size_t bytes);

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }
inline long long round_up(long long a, long long b) { return (a + b - 1) / b * b; }

}  // namespace sdpg
