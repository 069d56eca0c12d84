// Helpers shared by the C-ABI translation units: exception-to-error-code
// guard, limb-count dispatch, RAII device buffers and a per-thread workspace.
#pragma once
#include <string>
#include <type_traits>

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

inline Workspace &thread_workspace() {
    thread_local Workspace ws;
    return ws;
}

}  // namespace sdpg
