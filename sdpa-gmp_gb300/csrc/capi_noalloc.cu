// An allocation-free variant of the multi-limb GEMM entry point.
//
// sdpg_rgemm_device sizes and allocates its digit-plane scratch on first use (and
// grows it with cudaMalloc when a larger product arrives).  Some callers cannot let a
// library do that: a host program that has already handed all device memory to its
// own pool allocator, or a latency-critical loop in which an allocation (which
// synchronises the device and may fail when memory is tight) is not acceptable.
// sdpg_rgemm_device_noalloc serves them: its scratch is a fixed array in device
// memory that exists from the moment the library's code is loaded onto a GPU, so the
// call itself never allocates.
#include <mutex>

#include "capi_util.cuh"
#include "gemm.cuh"
#include "sdpg.h"

using namespace sdpg;

// Fixed scratch for sdpg_rgemm_device_noalloc: every GPU that loads this library holds
// SDPG_NOALLOC_SCRATCH_BYTES of it until the process exits.  Host code must not use
// the name as an address; it asks the runtime for the device address below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[SDPG_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void *g_scratch[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once per device.
void *scratch_for_current_device() {
    int dev = 0;
    SDPG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw sdpg_error(SDPG_ERR_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch[dev]) {
        void *ptr = nullptr;
        SDPG_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
        g_scratch[dev] = ptr;
    }
    return g_scratch[dev];
}

}  // namespace

extern "C" int sdpg_rgemm_device_noalloc(int limbs, char transa, char transb, int m, int n, int k,
                                         const void *alpha, const void *A, int lda, const void *B, int ldb,
                                         const void *beta, void *C, int ldc, void *stream) {
    return sdpg_guard([&] {
        if (m < 0 || n < 0 || k < 0) throw sdpg_error(SDPG_ERR_ARG, "negative dimension");
        if (!alpha || !beta) throw sdpg_error(SDPG_ERR_ARG, "null alpha or beta");
        const bool ta = (transa == 'T' || transa == 't' || transa == 'C' || transa == 'c');
        const bool tb = (transb == 'T' || transb == 't' || transb == 'C' || transb == 'c');
        if (lda < (ta ? (k > 1 ? k : 1) : (m > 1 ? m : 1)) || ldb < (tb ? (n > 1 ? n : 1) : (k > 1 ? k : 1)) ||
            ldc < (m > 1 ? m : 1))
            throw sdpg_error(SDPG_ERR_ARG, "leading dimension too small");
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            GemmProblem<N> p{};
            p.M = m;
            p.Nn = n;
            p.K = k;
            p.batch = 1;
            p.A = operand_A<N>(ta ? 'T' : 'N', (const mlf<N> *)A, lda, 0);
            p.B = operand_B<N>(tb ? 'T' : 'N', (const mlf<N> *)B, ldb, 0);
            p.C = (mlf<N> *)C;
            p.ldc = ldc;
            p.sc = 0;
            memcpy(&p.alpha, alpha, sizeof(mlf<N>));
            memcpy(&p.beta, beta, sizeof(mlf<N>));
            p.lower_only = 0;
            if (m == 0 || n == 0) return (int)SDPG_OK;
            const size_t need = gemm_bfp_workspace_bytes<N>(p);
            if (need > (size_t)SDPG_NOALLOC_SCRATCH_BYTES)
                throw sdpg_error(SDPG_ERR_TOO_LARGE,
                                 "sdpg_rgemm_device_noalloc: this product needs " + std::to_string(need) +
                                     " bytes of scratch, more than the fixed " +
                                     std::to_string((unsigned long long)SDPG_NOALLOC_SCRATCH_BYTES) +
                                     " bytes; use sdpg_rgemm_device");
            // Every scratch byte the kernels read is written earlier in the same call
            // (digit planes and exponents, padding included), so nothing is cleared.
            ml_gemm_scratch<N>(p, scratch_for_current_device(), (cudaStream_t)stream);
            return (int)SDPG_OK;
        });
    });
}
