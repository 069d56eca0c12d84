// tcgen05 modular GEMM: TMA loads of 128 x 64 fp16 tiles (128-byte swizzle) into a
// three-stage shared-memory ring, one thread issuing tcgen05.mma (M = N = 128,
// K = 16) into fp32 accumulators in tensor memory, and a four-warp epilogue that
// reads the accumulators with tcgen05.ld and reduces them modulo the tile's prime
// (the CRT factor is folded into the reconstruction's table instead).
//
// Every wait on an mbarrier is bounded by a cycle budget; on time-out the kernel
// records an error, lets the copies and products it issued finish (again with a
// bound), frees its tensor memory and returns.
#include <cuda.h>

#include <mutex>

#include "tc_gemm.cuh"
#include "tcgen05.cuh"

namespace sdpg {

namespace {

using namespace tc;

constexpr int kStages = 3;
constexpr int kTileBytes = kTcBM * kTcBK * 2;  // 16 KB, A and B tiles alike (BM == BN)
constexpr int kStageBytes = 2 * kTileBytes;
constexpr int kSmemBytes = kStages * kStageBytes + 1024 + 256;

// a bounded wait gave up: the caller's word and the device-wide flag record it
__device__ __forceinline__ void record_error(const TcModGemm &p, int code) {
    atomicExch(p.error, code);
    if (p.sticky && p.sticky != p.error) atomicExch(p.sticky, code);
}

constexpr uint32_t kIdesc = idesc_f16_f32(kTcBM, kTcBN);

__global__ void __launch_bounds__(128, 1)
    tc_modgemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcModGemm p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + kStages * kStageBytes);
    uint64_t *full = bars;                 // kStages
    uint64_t *empty = bars + kStages;      // kStages
    uint64_t *done = bars + 2 * kStages;   // 1
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * kStages + 1);
    __shared__ int abort_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.x * kTcBN, m0 = blockIdx.y * kTcBM;
    if (p.lower_only && n0 > m0 + kTcBM - 1) return;  // whole tile above the diagonal
    const int z = blockIdx.z;
    const int b = z / p.L, l = z - b * p.L;
    const int arow = ((p.a_batched ? b : 0) * p.L + l) * p.a_rows + m0;
    const int brow = ((p.b_batched ? b : 0) * p.L + l) * p.b_rows + n0;
    const int nk = p.Kpad / kTcBK;
    const int nacc = (p.Kpad + kTcKChunk - 1) / kTcKChunk;
    const uint32_t ncols = nacc <= 1 ? 128u : nacc <= 2 ? 256u : 512u;

    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int s = 0; s < kStages; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        mbar_init(smem_u32(done), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        tmem_alloc(smem_u32(tmem_slot), ncols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // The producer's and the MMA issuer's waits use the primary budget p.wait_cycles;
    // the waits that drain work already issued (products before tensor memory is freed,
    // copies before the CTA exits) always use the full budget.
    int issued = 0;  // TMA stages issued (producer thread)
    if (threadIdx.x == 0) {
        // producer: TMA into the stage ring
        bool ok = true;
        for (int kb = 0; kb < nk; ++kb) {
            const int s = kb % kStages;
            if (kb >= kStages && !mbar_wait(smem_u32(&empty[s]), ((kb / kStages) - 1) & 1, p.wait_cycles)) {
                ok = false;
                break;
            }
            const uint32_t fb = smem_u32(&full[s]);
            mbar_expect_tx(fb, kStageBytes);
            uint8_t *st = smem + s * kStageBytes;
            tma_load_2d(smem_u32(st), &tmA, p.k0 + kb * kTcBK, arow, fb);
            tma_load_2d(smem_u32(st + kTileBytes), &tmB, p.k0 + kb * kTcBK, brow, fb);
            ++issued;
        }
        if (!ok) {
            record_error(p, 1);
            abort_flag = 1;
        }
    } else if (threadIdx.x == 32) {
        // MMA issuer
        bool ok = true;
        for (int kb = 0; kb < nk; ++kb) {
            const int s = kb % kStages;
            if (!mbar_wait(smem_u32(&full[s]), (kb / kStages) & 1, p.wait_cycles)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const int acc = (kb * kTcBK) / kTcKChunk;
            const bool first = (kb * kTcBK) % kTcKChunk == 0;
            const uint32_t dt = tmem + (uint32_t)(acc * kTcBN);
            uint8_t *st = smem + s * kStageBytes;
            const uint64_t ad = sw128_kmajor_desc(smem_u32(st));
            const uint64_t bd = sw128_kmajor_desc(smem_u32(st + kTileBytes));
#pragma unroll
            for (int kk = 0; kk < kTcBK / 16; ++kk)
                tc_mma(dt, ad + (uint64_t)(2 * kk), bd + (uint64_t)(2 * kk), kIdesc, (first && kk == 0) ? 0u : 1u);
            tc_commit(smem_u32(&empty[s]));
        }
        if (!ok) {
            record_error(p, 2);
            abort_flag = 1;
        }
        tc_commit(smem_u32(done));  // arrives once every product issued above has completed
    }
    __syncwarp();
    if (!mbar_wait(smem_u32(done), 0)) {
        record_error(p, 3);
        abort_flag = 1;
    }
    __syncthreads();
    if (abort_flag && threadIdx.x == 0) {
        // let the copies already issued land before the CTA goes away: a stage's last
        // issued copy is among the last kStages (an earlier one was consumed before its
        // stage was refilled)
        for (int kb = (issued > kStages ? issued - kStages : 0); kb < issued; ++kb)
            mbar_wait(smem_u32(&full[kb % kStages]), (kb / kStages) & 1);
    }
    __syncthreads();
    tc_fence_after();

    if (!abort_flag) {
        const int m = p.moduli[l];
        const float inv_m = 1.0f / (float)m;
        const int row = warp * 32 + lane;
        uint16_t *yrow = p.Y + ((size_t)z * p.Mpad + m0 + row) * p.Npad + n0;
#pragma unroll 1
        for (int cb = 0; cb < kTcBN / 32; ++cb) {
            // the accumulators hold exact integers below 2^24: sum them as integers, then
            // reduce once (|x| < 2^26, so the float quotient is off by at most one)
            int r[32];
#pragma unroll
            for (int q = 0; q < 32; ++q) r[q] = 0;
#pragma unroll 1
            for (int a = 0; a < nacc; ++a) {
                uint32_t v[32];
                tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(a * kTcBN + cb * 32), v);
                tmem_ld_wait();
#pragma unroll
                for (int q = 0; q < 32; ++q) r[q] += __float2int_rn(__uint_as_float(v[q]));
            }
            uint4 *dst = reinterpret_cast<uint4 *>(yrow + cb * 32);
            uint32_t prev[16];
            if (p.accumulate) {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const uint4 v = dst[q];
                    prev[4 * q] = v.x;
                    prev[4 * q + 1] = v.y;
                    prev[4 * q + 2] = v.z;
                    prev[4 * q + 3] = v.w;
                }
            }
            uint32_t packed[16];
#pragma unroll
            for (int q = 0; q < 32; q += 2) {
                int y[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int x = r[q + u];
                    int t = x - (int)floorf((float)x * inv_m) * m;
                    t += (t < 0) ? m : 0;
                    t -= (t >= m) ? m : 0;
                    if (p.accumulate) {  // an earlier K chunk of the same product: add mod m
                        t += (int)((prev[q / 2] >> (16 * u)) & 0xFFFFu);
                        t -= (t >= m) ? m : 0;
                    }
                    y[u] = t;
                }
                packed[q / 2] = (uint32_t)y[0] | ((uint32_t)y[1] << 16);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
                dst[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, ncols);
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = [] {
        void *ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        SDPG_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !ptr)
            throw sdpg_error(SDPG_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
        return (EncodeTiledFn)ptr;
    }();
    return fn;
}

// 2D fp16 map over `rows` rows of `cols` elements (rows `pitch` elements apart), box
// 64 x 128, 128-byte swizzle; a box reaching past column `cols` reads zeros there
CUtensorMap make_map(const __half *base, long long rows, int cols, int pitch) {
    CUtensorMap m;
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)pitch * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kTcBK, (cuuint32_t)kTcBM};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, (void *)base, dims, strides, box, estr,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw sdpg_error(SDPG_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return m;
}

}  // namespace

long long g_tc_wait_cycles = 0;

void tc_modgemm(const TcModGemm &p, cudaStream_t s) {
    if (p.Mpad % kTcBM || p.Npad % kTcBN || p.Kpad % kTcBK || p.Kpad <= 0 || p.Kpad > kTcMaxK || p.L <= 0 ||
        p.batch <= 0 || p.k0 % kTcBK || p.k0 < 0 || p.kpitch % kTcBK || p.k0 + p.Kpad > p.kpitch || p.kext < 0 ||
        p.kext > p.kpitch)
        throw sdpg_error(SDPG_ERR_ARG, "tc_modgemm: unsupported shape");
    if (((uintptr_t)p.A | (uintptr_t)p.B | (uintptr_t)p.Y) & 15)
        throw sdpg_error(SDPG_ERR_ARG, "tc_modgemm: operands must be 16-byte aligned");
    static std::once_flag attr_once;
    std::call_once(attr_once, [] {
        SDPG_CUDA(cudaFuncSetAttribute(tc_modgemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    });
    TcModGemm q = p;
    if (q.a_rows <= 0) q.a_rows = p.Mpad;
    if (q.b_rows <= 0) q.b_rows = p.Npad;
    if (q.a_rows < p.Mpad && q.a_batched) throw sdpg_error(SDPG_ERR_ARG, "tc_modgemm: plane stride below the tile extent");
    // the maps cover exactly the planes' rows (a caller whose tiles run past the last
    // plane's end reads the fill value there)
    const long long arows = (long long)(p.a_batched ? p.batch : 1) * p.L * q.a_rows - p.a_skip;
    const long long brows = (long long)(p.b_batched ? p.batch : 1) * p.L * q.b_rows - p.b_skip;
    const int kext = p.kext > 0 ? p.kext : p.kpitch;
    const CUtensorMap ma = make_map(p.A, arows, kext, p.kpitch);
    const CUtensorMap mb = make_map(p.B, brows, kext, p.kpitch);
    dim3 grid(p.Npad / kTcBN, p.Mpad / kTcBM, p.batch * p.L);
    q.wait_cycles = g_tc_wait_cycles > 0 ? g_tc_wait_cycles : kWaitCycles;
    SDPG_KT_BEGIN(s);
    tc_modgemm_kernel<<<grid, 128, kSmemBytes, s>>>(ma, mb, q);
    SDPG_CHECK_LAUNCH_KTW("tc_modgemm_kernel", s, p.alg_flops);
}

}  // namespace sdpg
