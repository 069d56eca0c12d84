// Helpers shared by the C-ABI translation units: exception-to-error-code
// guard, limb-count dispatch, RAII device buffers and a per-thread workspace.
#pragma once
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "common.cuh"

namespace sdpg {

void set_last_error(const std::string &m);

template <class F>
int sdpg_guard(F &&f) {
    try {
        return f();
    } catch (const sdpg_error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return SDPG_ERR_ARG;
    } catch (...) {
        set_last_error("unknown failure");
        return SDPG_ERR_ARG;
    }
}

template <class F>
auto dispatch_limbs(int limbs, F &&f) {
    if (limbs == 8) return f(std::integral_constant<int, 8>{});
    if (limbs == 16) return f(std::integral_constant<int, 16>{});
    throw sdpg_error(SDPG_ERR_ARG, "unsupported limb count (use 8 or 16)");
}

struct DeviceBuffer {
    void *p = nullptr;
    size_t bytes = 0;
    explicit DeviceBuffer(size_t b = 0) {
        if (b) {
            SDPG_CUDA(cudaMalloc(&p, b));
            bytes = b;
        }
    }
    ~DeviceBuffer() {
        if (p) cudaFree(p);
    }
    DeviceBuffer(const DeviceBuffer &) = delete;
    DeviceBuffer &operator=(const DeviceBuffer &) = delete;
    DeviceBuffer(DeviceBuffer &&o) noexcept : p(o.p), bytes(o.bytes) {
        o.p = nullptr;
        o.bytes = 0;
    }
};

// Scratch of the standalone entry points: one workspace per (host thread, current
// device, stream).  Calls on one stream are ordered by that stream, so they can reuse
// its workspace; calls on other streams or devices get workspaces of their own, so no
// two calls that may overlap on the GPU share scratch.  Workspaces are plain cudaMalloc
// memory (freed with cudaFree, which waits for the device), and a thread that has used
// more than kMaxWorkspaces (device, stream) pairs releases them all before going on.
inline Workspace &thread_workspace(cudaStream_t stream) {
    constexpr size_t kMaxWorkspaces = 16;
    struct Entry {
        int device;
        cudaStream_t stream;
        std::unique_ptr<Workspace> ws;
    };
    thread_local std::vector<Entry> table;
    int dev = 0;
    SDPG_CUDA(cudaGetDevice(&dev));
    for (auto &e : table)
        if (e.device == dev && e.stream == stream) return *e.ws;
    if (table.size() >= kMaxWorkspaces) {
        for (auto &e : table) {
            SDPG_CUDA(cudaSetDevice(e.device));
            e.ws->release();
        }
        table.clear();
        SDPG_CUDA(cudaSetDevice(dev));
    }
    table.push_back(Entry{dev, stream, std::unique_ptr<Workspace>(new Workspace())});
    return *table.back().ws;
}

}  // namespace sdpg
